// Multi-shift tridiagonal route of the pole solves (sm_103a).
//
// All M/2 poles of a window share its standard-form matrix A = L^-1 H_W L^-T (real
// symmetric): the shifted systems differ only by z_k I.  The route therefore reduces A
// once per Hamiltonian to tridiagonal form T = Q^T A Q (Householder), carries the
// owned-point rows through the same reflectors, Y = F^ Q, and then every pole costs a
// complex-symmetric LDL^T of the tridiagonal z_k I - T (O(n)) and one forward sweep per
// row (O(n)):
//
//     d_k(r) = f^_r (z_k I - A)^-1 f^_r^T = y_r (z_k I - T)^-1 y_r^T = sum_i u_i^2 / D_i,
//     D_0 = z - t_0,   D_i = (z - t_i) - e_{i-1}^2 / D_{i-1},
//     u_0 = y_0,       u_i = y_i + (e_{i-1} / D_{i-1}) u_{i-1}.
//
// For Im z > 0, Im D_i >= Im z > 0, so no pivot vanishes and no pivoting is needed.  This
// is the multi-shift reduction used for transfer functions at many frequencies (A. J.
// Laub, "Efficient multivariable frequency response computations", IEEE Trans. Autom.
// Control 26 (1981) 407-408: one Hessenberg reduction, then each shift in O(n^2); for a
// symmetric matrix the Hessenberg form is tridiagonal and each shift is O(n)).  The
// quantities are the same as those of the LDL^T route (window_ldl.cu): the density, the
// electron count and the band energy of every window at every pole, and the pole sums
// are fused into the pass kernel.
//
// Kernels (R = float for the mixed path, double for the FP64 path):
//   tri_reduce_kernel  one CTA per window (work queue, largest first): blocked Householder
//                      tridiagonalisation of the full symmetric window matrix held in an
//                      L2-resident working copy; the rank-2 updates of each panel of nb
//                      columns are delayed (the panel's v and w vectors in shared memory)
//                      and applied once per panel; three barriers per column (the norm, the
//                      dots and A x taken over the unscaled column in one phase).
//                      Algorithmic work (4/3) n^3 flops.
//   tri_apply_res_kernel  (FP32) one CTA per (window, block of up to 128 rows) with the
//                      rows resident in shared memory through all panels: Y = F^ Q by
//                      panels in compact WY form, Y <- Y - ((Y V) T_p) V^T, 4 x 4 register
//                      tiles.  Algorithmic work 2 m n^2 flops per window.
//   tri_gram_kernel / tri_tfactor_kernel   per (window, panel): V^T V (one CTA), then the
//                      T_p of the compact WY form (one warp), once per Hamiltonian for all
//                      row sets.
//   tri_apply_kernel   one CTA per (window, block of up to 256 rows), one thread per row,
//                      the rows re-read from global memory per panel (FP64 path, and the
//                      configurations without resident rows).
//   tri_pass_kernel    one CTA per (window, batch of rows) from a work queue: thread =
//                      (pole, rows); the pivot recurrence of its pole is shared by its rows,
//                      the row values staged in shared memory by asynchronous copies; the
//                      quadratic forms are reduced over the poles into n(r) and e(r) in
//                      FP64 in a fixed order.  Algorithmic work ~11 real flops per (pole,
//                      row, step) plus the pivot recurrence.
//   tri_sturm_kernel / tri_mineig_kernel   Sturm counts of T - sigma (FP64 arithmetic): the
//                      Sylvester inertia of sigma S_W - H_W, and the smallest eigenvalue of
//                      every window by bisection.
#include "common.cuh"
#include "launch.cuh"
#include "lres_internal.h"

#include <algorithm>
#include <cmath>

namespace lres {
namespace {

template <class R> struct Cplx;
template <> struct Cplx<float> { using T = float2; };
template <> struct Cplx<double> { using T = double2; };

template <class R>
__device__ __forceinline__ R warp_sum(R x) {
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Sum over the CTA; every thread gets the same value, bit for bit (the butterfly gives all
// lanes one result and the warp totals are added in one fixed order).  red: NT/32 slots.
template <int NT, class R>
__device__ __forceinline__ R block_sum(R x, R* red) {
    x = warp_sum(x);
    __syncthreads();                          // red may still be read by a previous call
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    R s = red[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) s += red[w];
    return s;
}

template <class R>
__device__ __forceinline__ void cp_async4(R* dst, const R* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(R) == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int kAppRows = 256;                 // rows of one item of the apply kernel

// ---------------------------------------------------------------------------
// Householder tridiagonalisation
// ---------------------------------------------------------------------------

// Four consecutive rows of a column (16-byte aligned for float, two 16-byte loads for double).
__device__ __forceinline__ void ld4(const float* p, float (&x)[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&x)[4]) {
    const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&x)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&x)[4]) {
    *reinterpret_cast<double2*>(p) = make_double2(x[0], x[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(x[2], x[3]);
}

template <class R>
struct TriReduceParams {
    int nwin;
    const int* order;        // windows, largest first
    int* counter;            // work-queue head (zeroed before launch)
    const int* n_w;
    const long long* offC;   // standard-form blocks (n x n, column-major)
    const long long* offA;   // working blocks (ld x n, ld = n rounded up to 4)
    const long long* offN;   // window vectors (n)
    const R* H;              // standard-form matrices (lower triangle read)
    R* A;                    // working copies; on return the reflectors below the subdiagonal
    R* d;                    // diagonal of T
    R* e;                    // subdiagonal of T (e[i] couples i and i+1)
    R* tau;                  // reflector scalars
    int* status;
    int nb;                  // panel width (<= 32)
    int ldv;                 // length of the shared vectors (multiple of 32, >= every n)
};

// Shared memory of the reduction, in elements of R.
inline size_t reduce_smem_elems(int nb, int ldv, int nt) {
    const size_t big = std::max((size_t)2 * nb * ldv, (size_t)(nt / 32) * 32 * 33);
    return big + 5 * (size_t)ldv + 4 * (size_t)nt + 64 + nt / 32;
}

// CTAs per SM that the FP32 reduction is compiled for (registers: 65536 / (NT * that)).
constexpr int reduce_min_ctas(int nt, int elem) { return elem != 4 ? 1 : 1024 / nt; }

template <class R, int NT>
__global__ void __launch_bounds__(NT, reduce_min_ctas(NT, sizeof(R))) tri_reduce_kernel(TriReduceParams<R> p) {
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ldv = p.ldv, nb = p.nb;
    R* const big = reinterpret_cast<R*>(smem_raw);
    R* const Vs = big;                                   // [nb][ldv]: v_l[i] at Vs[l*ldv + i]
    R* const Ws = big + (size_t)nb * ldv;                // [nb][ldv]
    R* const cv = big + std::max((size_t)2 * nb * ldv, (size_t)NW * 32 * 33);   // [ldv] current column
    R* const pv = cv + ldv;                              // [ldv] p = tau (A v)
    R* const qx = pv + ldv;                              // [ldv] q = A x (unsplit)
    R* const acol = qx + ldv;                            // [2][ldv] panel-start columns j, j+1
    R* const psum = acol + 2 * ldv;                      // [4 NT] split sums of A x
    R* const dots = psum + 4 * NT;                       // [64] W^T x, V^T x, x^T x
    R* const red = dots + 64;                            // [NW]
    __shared__ int item_sh;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (;;) {
        if (tid == 0) item_sh = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= p.nwin) return;
        const int w = p.order[it];
        const int n = p.n_w[w];
        if (n > ldv || n < 1) {
            if (tid == 0) atomicOr(p.status, ST_BAD_SHAPE);
            __syncthreads();
            continue;
        }
        const int ld = (n + 3) & ~3;
        const R* H = p.H + p.offC[w];
        R* A = p.A + p.offA[w];
        R* dw = p.d + p.offN[w];
        R* ew = p.e + p.offN[w];
        R* tw = p.tau + p.offN[w];

        // ---- A = the full symmetric matrix from the lower triangle of H, by 32 x 32 blocks
        //      (each warp owns a padded tile: both the block and its transpose are written
        //      with coalesced stores)
        {
            R* tile = big + (size_t)warp * 32 * 33;
            const int nt = (n + 31) / 32;
            for (int t = warp; t < nt * (nt + 1) / 2; t += NW) {
                int bi = 0, bk = t;                      // t-th block of the lower block triangle
                while (bk > bi) {
                    bk -= bi + 1;
                    ++bi;
                }
                const int i0 = bi * 32, k0 = bk * 32;
                for (int c = 0; c < 32; ++c) {
                    const int i = i0 + lane, k = k0 + c;
                    tile[c * 33 + lane] = (i < n && k < n) ? H[i + (long long)k * n] : R(0);
                }
                __syncwarp();
                for (int c = 0; c < 32; ++c) {
                    const int i = i0 + lane, k = k0 + c;
                    if (i < n && k < n)
                        A[i + (long long)k * ld] = (bi != bk || lane >= c) ? tile[c * 33 + lane] : tile[lane * 33 + c];
                }
                if (bi != bk)
                    for (int c = 0; c < 32; ++c) {
                        const int k = k0 + lane, i = i0 + c;
                        if (i < n && k < n) A[k + (long long)i * ld] = tile[lane * 33 + c];
                    }
                __syncwarp();
            }
        }
        __syncthreads();

        // Each column takes three barriers.  Rows are owned by threads (row i by thread i mod NT)
        // for the column, the reflector and w; the norm, the dots W^T x, V^T x and q = A x are
        // taken over the unscaled column x (rows >= j+2) in one phase, and the reflector's scale
        // is applied afterwards: A v = A e_{j+1} + scal A x, X^T v = X_{j+1} + scal X^T x.  The
        // panel-start column j+1 of the owned rows is fetched by cp.async during column j: it
        // is A e_{j+1} of column j and the start of column j+1.
        R Kprev = R(0);
        for (int j0 = 0; j0 < n - 2; j0 += nb) {
            const int nbp = min(nb, n - 2 - j0);
            for (int jj = 0; jj < nbp; ++jj) {
                const int j = j0 + jj;
                R* const anext = acol + ((j + 1) & 1) * ldv;
                const R* const acur = acol + (j & 1) * ldv;
                for (int i = tid; i < n; i += NT)
                    if (i > j) cp_async4(anext + i, A + i + (long long)(j + 1) * ld);
                cp_commit();
                // (a) column j of the current matrix (panel-start values minus the pending rank-2
                //     updates of this panel) on the owned rows >= j.  w_{jj-1} at row j is
                //     p_j - K (v_{jj-1} is 1 there); every thread forms it from the published p.
                {
                    const R wlast = jj > 0 ? pv[j] - Kprev : R(0);
                    for (int i = tid; i < n; i += NT) {
                        if (i < j) continue;
                        R c = jj > 0 ? acur[i] : A[i + (long long)j * ld];
                        for (int l = 0; l < jj; ++l) {
                            const R wlj = l == jj - 1 ? wlast : Ws[l * ldv + j];
                            c -= Vs[l * ldv + i] * wlj + Ws[l * ldv + i] * Vs[l * ldv + j];
                        }
                        cv[i] = c;
                    }
                }
                __syncthreads();
                // (b) q = A x on rows >= j+1 by quads of rows (16-byte loads) from the aligned row
                //     i0 <= j+1; when the quads are few, the columns are split across thread groups
                //     and the partial sums added in a fixed order.  Sums are blocked: each run of
                //     32 terms from zero.
                const int i0 = (j + 1) & ~3;
                const int nq = (ld - i0) >> 2;
                const int nsplit = nq >= NT ? 1 : NT / nq;
                {
                    const int qstep = nq >= NT ? NT : nq;
                    if (tid < qstep * nsplit) {
                        const int sp = tid / qstep;
                        for (int q = tid % qstep; q < nq; q += qstep) {
                            const R* Aq = A + i0 + 4 * q;
                            R a[4] = {R(0), R(0), R(0), R(0)};
                            for (int kb = j + 2 + sp; kb < n; kb += 32 * nsplit) {
                                const int ke = min(n, kb + 32 * nsplit);
                                R c[4] = {R(0), R(0), R(0), R(0)};
#pragma unroll 8
                                for (int k = kb; k < ke; k += nsplit) {
                                    R x[4];
                                    ld4(Aq + (long long)k * ld, x);
                                    const R xk = cv[k];
#pragma unroll
                                    for (int r = 0; r < 4; ++r) c[r] = fma(x[r], xk, c[r]);
                                }
#pragma unroll
                                for (int r = 0; r < 4; ++r) a[r] += c[r];
                            }
                            if (nsplit > 1) {
                                st4(psum + (sp * nq + q) * 4, a);    // 16-byte stores: no bank conflicts
                            } else {
#pragma unroll
                                for (int r = 0; r < 4; ++r) {
                                    const int i = i0 + 4 * q + r;
                                    if (i > j && i < n) qx[i] = a[r];
                                }
                            }
                        }
                    }
                }
                //     dots[l] = W_l^T x, dots[jj + l] = V_l^T x, dots[2 jj] = x^T x over rows >= j+2,
                //     a warp each (the last warps first: they have the fewest row quads)
                for (int q = NW - 1 - warp; q <= 2 * jj; q += NW) {
                    const R* X = q < jj ? Ws + (size_t)q * ldv : q < 2 * jj ? Vs + (size_t)(q - jj) * ldv : cv;
                    R acc = R(0);
                    for (int i = j + 2 + lane; i < n; i += 32) acc += X[i] * cv[i];
                    acc = warp_sum(acc);
                    if (lane == 0) dots[q] = acc;
                }
                __syncthreads();
                // (c) reflector H_j = I - tau v v^T with v_{j+1} = 1 mapping rows j+1.. of the
                //     column onto beta e_{j+1} (every thread, the same bits); p = tau (A v - V (W^T v)
                //     - W (V^T v)) on the owned rows, partial sums of p^T v
                const R s2 = dots[2 * jj];
                const R alpha = cv[j + 1];
                R beta = alpha, tau = R(0), scal = R(0);
                if (s2 > R(0)) {
                    const R nrm = sqrt(alpha * alpha + s2);
                    beta = alpha >= R(0) ? -nrm : nrm;
                    tau = (beta - alpha) / beta;
                    scal = R(1) / (alpha - beta);
                }
                if (tid == 0) {
                    dw[j] = cv[j];
                    ew[j] = beta;
                    tw[j] = tau;
                    if (!isfinite((double)beta) || !isfinite((double)cv[j])) atomicOr(p.status, ST_ZERO_PIVOT);
                }
                cp_wait<0>();
                R partK = R(0);
                for (int i = tid; i < ldv; i += NT) {
                    R vi = R(0);
                    if (i == j + 1) vi = R(1);
                    else if (i > j + 1 && i < n) vi = cv[i] * scal;
                    Vs[jj * ldv + i] = vi;
                    if (i > j && i < n) {
                        if (i > j + 1) A[i + (long long)j * ld] = vi;      // kept for Y = F^ Q
                        R qi;
                        if (nsplit > 1) {
                            const int q = (i - i0) >> 2, r = (i - i0) & 3;
                            qi = R(0);
                            for (int sp = 0; sp < nsplit; ++sp) qi += psum[(sp * nq + q) * 4 + r];
                        } else {
                            qi = qx[i];
                        }
                        R pi = anext[i] + scal * qi;
                        for (int l = 0; l < jj; ++l) {
                            const R dW = Ws[l * ldv + j + 1] + scal * dots[l];
                            const R dV = Vs[l * ldv + j + 1] + scal * dots[jj + l];
                            pi -= Vs[l * ldv + i] * dW + Ws[l * ldv + i] * dV;
                        }
                        pi *= tau;
                        pv[i] = pi;
                        partK += pi * vi;
                    }
                }
                partK = warp_sum(partK);
                if (lane == 0) red[warp] = partK;
                __syncthreads();
                // (d) K = tau/2 p^T v, w = p - K v on the owned rows
                R sK = red[0];
#pragma unroll
                for (int w2 = 1; w2 < NW; ++w2) sK += red[w2];
                const R K = R(0.5) * tau * sK;
                Kprev = K;
                for (int i = tid; i < ldv; i += NT)
                    Ws[jj * ldv + i] = (i > j && i < n) ? pv[i] - K * Vs[jj * ldv + i] : R(0);
            }
            __syncthreads();
            // ---- trailing update of both triangles: A -= V W^T + W V^T on rows, columns >= t0.
            //      One quad of rows x one aligned quad of columns per thread: the v, w values of
            //      both quads come from shared memory as 16-byte vectors (4 loads per 32 FMAs);
            //      rows and columns below t0 are left unchanged.
            const int t0 = j0 + nbp;
            if (t0 < n) {
                const int q0 = t0 & ~3;
                const int nq = (ld - q0) >> 2;
                const int ncb = (ld - q0) >> 2;
                for (int tile = tid; tile < nq * ncb; tile += NT) {
                    const int q = tile % nq, cb = tile / nq;
                    const int i = q0 + 4 * q, c0 = q0 + 4 * cb;
                    R acc[4][4];
#pragma unroll
                    for (int c = 0; c < 4; ++c)
#pragma unroll
                        for (int r = 0; r < 4; ++r) acc[c][r] = R(0);
                    for (int l = 0; l < nbp; ++l) {
                        R vi[4], wi[4], vk[4], wk[4];
                        ld4(Vs + (size_t)l * ldv + i, vi);
                        ld4(Ws + (size_t)l * ldv + i, wi);
                        ld4(Vs + (size_t)l * ldv + c0, vk);
                        ld4(Ws + (size_t)l * ldv + c0, wk);
#pragma unroll
                        for (int c = 0; c < 4; ++c)
#pragma unroll
                            for (int r = 0; r < 4; ++r) acc[c][r] = fma(vi[r], wk[c], fma(wi[r], vk[c], acc[c][r]));
                    }
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const int col = c0 + c;
                        if (col < t0 || col >= n) continue;
                        R x[4];
                        R* dst = A + i + (long long)col * ld;
                        ld4(dst, x);
#pragma unroll
                        for (int r = 0; r < 4; ++r)
                            if (i + r >= t0) x[r] -= acc[c][r];
                        st4(dst, x);
                    }
                }
            }
            __syncthreads();
        }
        // ---- the last (at most 2 x 2) block, fully updated
        if (tid == 0) {
            if (n >= 2) {
                dw[n - 2] = A[(n - 2) + (long long)(n - 2) * ld];
                ew[n - 2] = A[(n - 1) + (long long)(n - 2) * ld];
                dw[n - 1] = A[(n - 1) + (long long)(n - 1) * ld];
                tw[n - 2] = R(0);
                tw[n - 1] = R(0);
                ew[n - 1] = R(0);
            } else {
                dw[0] = A[0];
                tw[0] = R(0);
                ew[0] = R(0);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Householder tridiagonalisation with the window resident in shared memory (FP32)
// ---------------------------------------------------------------------------
//
// The lower triangle of the window stays in shared memory for the whole reduction, in 4 x 4
// blocks: column c holds rows 4 (c / 4) .. ld-1, i.e. the lower part plus the upper part of
// its diagonal block (kept equal to the lower one), from
//     colstart(c) = c ld - 8 a (a - 1) - 4 a b,   a = c / 4, b = c % 4,
// so that every block's four column segments start on 16-byte boundaries.  p = A v uses
// each stored block twice: for the row quad I, block (I, K) (K <= I) directly and block (K, I)
// (K > I) transposed; a warp takes one row quad at a time, its lanes the column quads K
// (16-byte loads, four per block), and the lanes' partial sums are added by a butterfly in a
// fixed order.  The trailing update touches the stored blocks only (half the FMAs of a full
// update).  One CTA per window (work queue, largest first), windows up to ld <= 320.

constexpr int kResReduceNT = 640;
constexpr int kResReduceMaxN = 320;

__host__ __device__ inline int res_cs(int c, int ld) {
    const int a = c >> 2, b = c & 3;
    return c * ld - 8 * a * (a - 1) - 4 * a * b;
}
// element (r, c) of the stored part (r >= 4 (c / 4))
__host__ __device__ inline int res_at(int r, int c, int ld) { return res_cs(c, ld) + r - 4 * (c >> 2); }

// shared memory without the partial sums of p = A v (nseg x ldv more)
inline size_t res_reduce_smem_elems(int nb, int ldv, int nmax) {
    const int ld = (nmax + 3) & ~3;
    const size_t head = (size_t)res_cs(ld, ld) + 2 * (size_t)nb * ldv + 2 * (size_t)ldv + 64 + kResReduceNT / 32;
    return ((head + 3) & ~(size_t)3) + (size_t)ldv;      // + the column-start table (16-byte aligned)
}

template <int NT>
__global__ void __launch_bounds__(NT, 1) tri_reduce_res_kernel(TriReduceParams<float> p, int nmax, int nseg) {
    constexpr int NW = NT / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ldv = p.ldv, nb = p.nb;
    float* const Vs = reinterpret_cast<float*>(smem_raw);            // [nb][ldv]
    float* const Ws = Vs + (size_t)nb * ldv;                         // [nb][ldv]
    float* const Ls = Ws + (size_t)nb * ldv;                         // blocked lower triangle
    float* const cv = Ls + res_cs((nmax + 3) & ~3, (nmax + 3) & ~3); // [ldv] current column
    float* const pv = cv + ldv;                                      // [ldv] p = tau (A v)
    float* const dots = pv + ldv;                                    // [64]
    float* const red = dots + 64;                                    // [NW]
    const size_t head = (size_t)(red + NW - reinterpret_cast<float*>(smem_raw));
    int* const cst = reinterpret_cast<int*>(smem_raw) + ((head + 3) & ~(size_t)3);   // [ldv] column starts
    float* const psum = reinterpret_cast<float*>(cst + ldv);         // [nseg][ldv] partial A v
    __shared__ int item_sh, nseg_used;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (;;) {
        if (tid == 0) item_sh = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= p.nwin) return;
        const int w = p.order[it];
        const int n = p.n_w[w];
        const int ld = (n + 3) & ~3;
        if (n > ldv || n > nmax || n < 1) {
            if (tid == 0) atomicOr(p.status, ST_BAD_SHAPE);
            __syncthreads();
            continue;
        }
        const int nq = ld >> 2;
        const float* H = p.H + p.offC[w];
        float* A = p.A + p.offA[w];
        float* dw = p.d + p.offN[w];
        float* ew = p.e + p.offN[w];
        float* tw = p.tau + p.offN[w];

        for (int c = tid; c < ld; c += NT) cst[c] = res_cs(c, ld);
        // ---- the stored part of H (lower triangle, mirrored into the diagonal blocks; zero
        //      beyond n), warp per column, rows along the lanes
        for (int c = warp; c < ld; c += NW) {
            const int r0 = 4 * (c >> 2);
            for (int r = r0 + lane; r < ld; r += 32) {
                float x = 0.0f;
                if (r < n && c < n) x = r >= c ? H[r + (long long)c * n] : H[c + (long long)r * n];
                Ls[res_at(r, c, ld)] = x;
            }
        }
        __syncthreads();

        for (int j0 = 0; j0 < n - 2; j0 += nb) {
            const int nbp = min(nb, n - 2 - j0);
            for (int jj = 0; jj < nbp; ++jj) {
                const int j = j0 + jj;
                // (a) column j of the current matrix, rows >= j: panel-start values minus
                //     the pending rank-2 updates; squares of rows >= j+2
                float part = 0.0f;
                {
                    const int i = j + tid;
                    if (i < n) {
                        float c = Ls[res_at(i, j, ld)];
                        for (int l = 0; l < jj; ++l)
                            c -= Vs[l * ldv + i] * Ws[l * ldv + j] + Ws[l * ldv + i] * Vs[l * ldv + j];
                        cv[i] = c;
                        if (i >= j + 2) part = c * c;
                    }
                }
                // (b) reflector H_j = I - tau v v^T, v_{j+1} = 1
                const float s2 = block_sum<NT>(part, red);    // its barriers also publish cv
                const float alpha = cv[j + 1];
                float beta = alpha, tau = 0.0f, scal = 0.0f;
                if (s2 > 0.0f) {
                    const float nrm = sqrtf(alpha * alpha + s2);
                    beta = alpha >= 0.0f ? -nrm : nrm;
                    tau = (beta - alpha) / beta;
                    scal = 1.0f / (alpha - beta);
                }
                if (tid == 0) {
                    dw[j] = cv[j];
                    ew[j] = beta;
                    tw[j] = tau;
                    if (!isfinite(beta) || !isfinite(cv[j])) atomicOr(p.status, ST_ZERO_PIVOT);
                }
                for (int i = tid; i < ldv; i += NT) {
                    float vi = 0.0f;
                    if (i == j + 1) vi = 1.0f;
                    else if (i > j + 1 && i < n) vi = cv[i] * scal;
                    Vs[jj * ldv + i] = vi;
                    if (i > j + 1 && i < n) A[i + (long long)j * ld] = vi;   // kept for Y = F^ Q
                }
                __syncthreads();
                // (c) W^T v, V^T v (warp per product) and A v on the row quads from (j+1)/4,
                //     from the panel-start matrix (v is zero on the rows <= j)
                for (int q = warp; q < 2 * jj; q += NW) {
                    const float* X = q < jj ? Ws + (size_t)q * ldv : Vs + (size_t)(q - jj) * ldv;
                    float acc = 0.0f;
                    for (int i = j + 1 + lane; i < n; i += 32) acc += X[i] * Vs[jj * ldv + i];
                    acc = warp_sum(acc);
                    if (lane == 0) dots[q] = acc;
                }
                {
                    // lanes over 32 row quads I, warps over (row-quad group, segment of the
                    // column quads K); each warp's partial sums go to psum[segment] and are
                    // added in segment order in (d)
                    const float* vv = Vs + (size_t)jj * ldv;
                    const int q0 = (j + 1) >> 2, mq = nq - q0;
                    const int G = (mq + 31) >> 5;
                    const int S = min(NW / G, nseg);
                    const int g = warp / S, s = warp % S;
                    if (g < G) {
                        const int I = q0 + 32 * g + lane;
                        const int k0 = q0 + (int)((long long)mq * s / S), k1 = q0 + (int)((long long)mq * (s + 1) / S);
                        float pr[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                        if (I < nq) {
                            const int4 cI = *reinterpret_cast<const int4*>(cst + 4 * I);
                            const int csI[4] = {cI.x, cI.y, cI.z, cI.w};
                            for (int K = k0; K < k1; ++K) {
                                const float4 vK4 = *reinterpret_cast<const float4*>(vv + 4 * K);
                                const float vk[4] = {vK4.x, vK4.y, vK4.z, vK4.w};
                                if (K > I) {
                                    // block (K, I): column 4I+c, rows 4K..4K+3: p_I[c] += b . v_K
                                    const int base = 4 * K - 4 * I;
#pragma unroll
                                    for (int c = 0; c < 4; ++c) {
                                        const float4 b = *reinterpret_cast<const float4*>(Ls + csI[c] + base);
                                        pr[c] = fmaf(b.x, vk[0], fmaf(b.y, vk[1], fmaf(b.z, vk[2], fmaf(b.w, vk[3], pr[c]))));
                                    }
                                } else {
                                    // block (I, K): column 4K+c, rows 4I..4I+3: p_I[r] += b[r] v_K[c]
                                    const int4 cK = *reinterpret_cast<const int4*>(cst + 4 * K);
                                    const int off = 4 * I - 4 * K;
                                    const int cc[4] = {cK.x, cK.y, cK.z, cK.w};
#pragma unroll
                                    for (int c = 0; c < 4; ++c) {
                                        const float4 b = *reinterpret_cast<const float4*>(Ls + cc[c] + off);
                                        pr[0] = fmaf(b.x, vk[c], pr[0]);
                                        pr[1] = fmaf(b.y, vk[c], pr[1]);
                                        pr[2] = fmaf(b.z, vk[c], pr[2]);
                                        pr[3] = fmaf(b.w, vk[c], pr[3]);
                                    }
                                }
                            }
                            *reinterpret_cast<float4*>(psum + (size_t)s * ldv + 4 * I) = make_float4(pr[0], pr[1], pr[2], pr[3]);
                        }
                    }
                    if (tid == 0) nseg_used = S;
                }
                __syncthreads();
                // (d) p *= tau (with the pending updates), K = tau/2 p.v, w = p - K v
                float partK = 0.0f;
                {
                    const int i = j + 1 + tid;
                    if (i < n) {
                        float pi = psum[i];
                        for (int s2 = 1; s2 < nseg_used; ++s2) pi += psum[(size_t)s2 * ldv + i];
                        for (int l = 0; l < jj; ++l) pi -= Vs[l * ldv + i] * dots[l] + Ws[l * ldv + i] * dots[jj + l];
                        pi *= tau;
                        pv[i] = pi;
                        partK = pi * Vs[jj * ldv + i];
                    }
                }
                const float K = 0.5f * tau * block_sum<NT>(partK, red);
                for (int i = tid; i < ldv; i += NT)
                    Ws[jj * ldv + i] = (i > j && i < n) ? pv[i] - K * Vs[jj * ldv + i] : 0.0f;
                __syncthreads();
            }
            // ---- trailing update of the stored blocks (I >= K >= t0 / 4): B -= V W^T + W V^T;
            //      the blocks in column order from the last column quad, consecutive threads
            //      on consecutive row quads of one column quad, so that the v, w of the rows
            //      and the blocks are contiguous across a warp and those of the columns broadcast
            const int t0 = j0 + nbp;
            if (t0 < n) {
                const int qa = t0 >> 2;
                const int m = nq - qa;
                const int ntile = m * (m + 1) / 2;
                for (int tile = tid; tile < ntile; tile += NT) {
                    int u = (int)((sqrtf(8.0f * tile + 1.0f) - 1.0f) * 0.5f);
                    while ((u + 1) * (u + 2) / 2 <= tile) ++u;
                    while (u * (u + 1) / 2 > tile) --u;
                    const int K = qa + m - 1 - u, I = K + tile - u * (u + 1) / 2;
                    const int i = 4 * I, c0 = 4 * K;
                    float acc[4][4];
#pragma unroll
                    for (int c = 0; c < 4; ++c)
#pragma unroll
                        for (int r = 0; r < 4; ++r) acc[c][r] = 0.0f;
                    for (int l = 0; l < nbp; ++l) {
                        float vi[4], wi[4], vk[4], wk[4];
                        ld4(Vs + (size_t)l * ldv + i, vi);
                        ld4(Ws + (size_t)l * ldv + i, wi);
                        ld4(Vs + (size_t)l * ldv + c0, vk);
                        ld4(Ws + (size_t)l * ldv + c0, wk);
#pragma unroll
                        for (int c = 0; c < 4; ++c)
#pragma unroll
                            for (int r = 0; r < 4; ++r) acc[c][r] = fmaf(vi[r], wk[c], fmaf(wi[r], vk[c], acc[c][r]));
                    }
                    const int4 cK = *reinterpret_cast<const int4*>(cst + c0);
                    const int cc[4] = {cK.x, cK.y, cK.z, cK.w};
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        float* dst = Ls + cc[c] + i - c0;
                        float x[4];
                        ld4(dst, x);
#pragma unroll
                        for (int r = 0; r < 4; ++r) x[r] -= acc[c][r];
                        st4(dst, x);
                    }
                }
            }
            __syncthreads();
        }
        // ---- the last (at most 2 x 2) block, fully updated
        if (tid == 0) {
            if (n >= 2) {
                dw[n - 2] = Ls[res_at(n - 2, n - 2, ld)];
                ew[n - 2] = Ls[res_at(n - 1, n - 2, ld)];
                dw[n - 1] = Ls[res_at(n - 1, n - 1, ld)];
                tw[n - 2] = 0.0f;
                tw[n - 1] = 0.0f;
                ew[n - 1] = 0.0f;
            } else {
                dw[0] = Ls[0];
                tw[0] = 0.0f;
                ew[0] = 0.0f;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Y = F^ Q: the rows through the reflectors, compact WY per panel
// ---------------------------------------------------------------------------

template <class R>
struct TriApplyParams {
    int nitems;
    const int4* items;       // (window, first row, rows <= 256, -)
    const int* n_w;
    const int* m_w;          // rows of each window
    const long long* offA;   // reflectors (working blocks, leading dimension n rounded up to 4)
    const long long* offN;
    const long long* offF;   // row blocks, F[r + a*m]
    const R* A;              // reflectors below the subdiagonal (tri_reduce_kernel)
    const R* tau;
    const R* F;              // standard-form rows
    R* Y;                    // F^ Q, same layout
    int ldv;
};

// Index of v_l[k] in the staged panel: rows of NB values, 16-byte groups of each row permuted
// by XOR with the row index, so that the staging stores (consecutive k, one l) spread over the
// banks while each row is still read as aligned 16-byte vectors.
template <class R, int NB>
__device__ __forceinline__ int panel_index(int k, int l) {
    constexpr int GW = 16 / (int)sizeof(R) < NB ? 16 / (int)sizeof(R) : NB;   // elements per group
    constexpr int NG = NB / GW;                                                 // groups per row
    return k * NB + (((l / GW) ^ (k % NG)) * GW) + (l % GW);
}

// One 16-byte group of a staged row (4 floats or 2 doubles; a narrower panel row whole).
template <class R, int GW>
__device__ __forceinline__ void ld_group(const R* src, R (&x)[GW]) {
    if constexpr (sizeof(R) == 4 && GW == 4) {
        const float4 v = *reinterpret_cast<const float4*>(src);
        x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
    } else if constexpr (sizeof(R) == 8 && GW == 2) {
        const double2 v = *reinterpret_cast<const double2*>(src);
        x[0] = v.x; x[1] = v.y;
    } else {
#pragma unroll
        for (int e = 0; e < GW; ++e) x[e] = src[e];
    }
}

// NT threads handle the item's rows (at most NT * RPT), RPT rows each (rows tid + u NT), so
// that every staged reflector value feeds RPT multiply-adds.
template <class R, int NT, int NB, int RPT>
__global__ void __launch_bounds__(NT, RPT == 1 && NB <= 16 ? 3 : 1) tri_apply_kernel(TriApplyParams<R> p) {
    constexpr int GW = 16 / (int)sizeof(R) < NB ? 16 / (int)sizeof(R) : NB;
    constexpr int NG = NB / GW;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* const Vs = reinterpret_cast<R*>(smem_raw);         // [ldv][NB], panel_index layout
    R* const Tm = Vs + (size_t)p.ldv * NB;                 // [NB][NB] upper triangular factor
    R* const Gm = Tm + NB * NB;                            // [NB][NB] V^T V (above the diagonal)
    const int4 item = p.items[blockIdx.x];
    const int w = item.x, r0 = item.y, nr = item.z;
    const int n = p.n_w[w], m = p.m_w[w];
    if (n > p.ldv) return;                                 // the reduction flagged this window
    const long long ld = (n + 3) & ~3;
    const R* Aw = p.A + p.offA[w];
    const R* tw = p.tau + p.offN[w];
    const R* Fw = p.F + p.offF[w];
    R* Yw = p.Y + p.offF[w];
    const int tid = threadIdx.x;
    bool act[RPT];
    long long rr[RPT];
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
        const int t = tid + u * NT;
        act[u] = t < nr && r0 + t < m;
        rr[u] = act[u] ? r0 + t : 0;
    }
#pragma unroll
    for (int u = 0; u < RPT; ++u)
        if (act[u]) {
#pragma unroll 8
            for (int k = 0; k < n; ++k) Yw[rr[u] + (long long)k * m] = Fw[rr[u] + (long long)k * m];
        }

    for (int j0 = 0; j0 < n - 2; j0 += NB) {
        const int nbp = min(NB, n - 2 - j0);
        const int nk = n - j0 - 1;                         // rows j0+1 .. n-1
        __syncthreads();                                   // the previous panel is consumed
        // v_l (l < nbp) lives on rows j0+l+1 .. n-1 (v_l[j0+l+1] = 1); reads run down the
        // columns of the reflector storage (coalesced)
        for (int idx = tid; idx < nk * NB; idx += NT) {
            const int l = idx / nk, k = j0 + 1 + idx % nk;
            R v = R(0);
            if (l < nbp) {
                const int j = j0 + l;
                if (k == j + 1) v = R(1);
                else if (k > j + 1) v = Aw[k + j * ld];
            }
            Vs[panel_index<R, NB>(k, l)] = v;
        }
        __syncthreads();
        // G = V^T V by 2 x 2 blocks per thread (entries above the diagonal are used)
        for (int q = tid; q < NB * NB / 4; q += NT) {
            const int a0 = 2 * (q / (NB / 2)), b0 = 2 * (q % (NB / 2));
            R g00 = R(0), g01 = R(0), g10 = R(0), g11 = R(0);
            if (b0 + 1 > a0) {
                for (int k = j0 + 1; k < n; ++k) {
                    const R va0 = Vs[panel_index<R, NB>(k, a0)], va1 = Vs[panel_index<R, NB>(k, a0 + 1)];
                    const R vb0 = Vs[panel_index<R, NB>(k, b0)], vb1 = Vs[panel_index<R, NB>(k, b0 + 1)];
                    g00 = fma(va0, vb0, g00);
                    g01 = fma(va0, vb1, g01);
                    g10 = fma(va1, vb0, g10);
                    g11 = fma(va1, vb1, g11);
                }
            }
            Gm[a0 * NB + b0] = g00;
            Gm[a0 * NB + b0 + 1] = g01;
            Gm[(a0 + 1) * NB + b0] = g10;
            Gm[(a0 + 1) * NB + b0 + 1] = g11;
        }
        __syncthreads();
        // T (forward, columnwise): T_ll = tau_l, T[0:l, l] = -tau_l T[0:l, 0:l] (V^T V)[0:l, l]
        if (tid < 32) {
            for (int l = 0; l < NB; ++l) {
                const R tl = l < nbp ? tw[j0 + l] : R(0);
                for (int a = tid; a < NB; a += 32) {
                    R val = R(0);
                    if (a < l) {
                        R sacc = R(0);
                        for (int b = a; b < l; ++b) sacc = fma(Tm[a * NB + b], Gm[b * NB + l], sacc);
                        val = -tl * sacc;
                    } else if (a == l) {
                        val = tl;
                    }
                    Tm[a * NB + l] = val;
                }
                __syncwarp();
            }
        }
        __syncthreads();
        R sv[RPT][NB];
#pragma unroll
        for (int u = 0; u < RPT; ++u)
#pragma unroll
            for (int l = 0; l < NB; ++l) sv[u][l] = R(0);
#pragma unroll 4
        for (int k = j0 + 1; k < n; ++k) {
            R y[RPT];
#pragma unroll
            for (int u = 0; u < RPT; ++u) y[u] = act[u] ? Yw[rr[u] + (long long)k * m] : R(0);
            const R* row = Vs + (size_t)k * NB;
#pragma unroll
            for (int g = 0; g < NG; ++g) {
                R x[GW];
                ld_group<R, GW>(row + ((g ^ (k % NG)) * GW), x);
#pragma unroll
                for (int u = 0; u < RPT; ++u)
#pragma unroll
                    for (int e = 0; e < GW; ++e) sv[u][g * GW + e] = fma(y[u], x[e], sv[u][g * GW + e]);
            }
        }
        // s <- s T in place (T upper triangular: column b needs s_0..s_b, so b descends)
#pragma unroll
        for (int b = NB - 1; b >= 0; --b) {
            R acc[RPT];
#pragma unroll
            for (int u = 0; u < RPT; ++u) acc[u] = R(0);
#pragma unroll
            for (int a = 0; a <= b; ++a) {
                const R t = Tm[a * NB + b];
#pragma unroll
                for (int u = 0; u < RPT; ++u) acc[u] = fma(sv[u][a], t, acc[u]);
            }
#pragma unroll
            for (int u = 0; u < RPT; ++u) sv[u][b] = acc[u];
        }
#pragma unroll 4
        for (int k = j0 + 1; k < n; ++k) {
            const R* row = Vs + (size_t)k * NB;
            R acc[RPT];
#pragma unroll
            for (int u = 0; u < RPT; ++u) acc[u] = R(0);
#pragma unroll
            for (int g = 0; g < NG; ++g) {
                R x[GW];
                ld_group<R, GW>(row + ((g ^ (k % NG)) * GW), x);
#pragma unroll
                for (int u = 0; u < RPT; ++u)
#pragma unroll
                    for (int e = 0; e < GW; ++e) acc[u] = fma(sv[u][g * GW + e], x[e], acc[u]);
            }
#pragma unroll
            for (int u = 0; u < RPT; ++u)
                if (act[u]) Yw[rr[u] + (long long)k * m] -= acc[u];
        }
    }
}

// ---------------------------------------------------------------------------
// Y = F^ Q with the item's rows resident in shared memory (FP32)
// ---------------------------------------------------------------------------
//
// The rows of one item (at most kResRows) stay in shared memory through all panels, so Y
// crosses to global memory once per launch instead of once per panel.  Per panel of NB
// reflectors: S = Y V (a thread = 4 rows x 4 reflectors; a warp = 8 row quads x 4 reflector
// quads, so that every 16-byte shared load serves a broadcast or one conflict-free
// wavefront), S <- S T (same tiles), Y <- Y - S V^T (a thread = 4 rows x 4 columns; a warp =
// 8 row quads x 4 column quads).  The T factor of every (window, panel) is formed once per
// Hamiltonian by tri_gram_kernel and tri_tfactor_kernel.

constexpr int kResRows = 128;                 // rows of an item of the resident application
constexpr int kResNT = 512;

// Staged panel: rows of NB values v_l[k]; the 16-byte groups of row kk permuted by XOR with
// kk / 4, so that rows 4 apart (one per column quad of a warp) hit different banks.
template <int NB>
__device__ __forceinline__ int res_index(int kk, int l) {
    constexpr int NG = NB / 4;
    return kk * NB + ((((l >> 2) ^ (kk >> 2)) & (NG - 1)) << 2) + (l & 3);
}

// v_l (l < nbp) on the panel rows kk = 0..nk-1 (window row j0+1+kk), v_l = 1 on row j0+l+1,
// zero above; reads run down the reflector columns (coalesced).
// The reflector values go by asynchronous copies (all of a thread's copies in flight at
// once), the zeros and ones by plain stores; the caller waits (cp_wait) before the barrier.
template <int NT, int NB>
__device__ __forceinline__ void res_stage(float* Vs, const float* Aw, long long ld, int j0, int nbp, int nk) {
    // warp per reflector column, lanes down its rows (no division by nk)
    const int lane = threadIdx.x & 31;
    for (int l = threadIdx.x >> 5; l < NB; l += NT / 32) {
        const int j = j0 + l;
        const float* src = Aw + (long long)j * ld;
        for (int kk = lane; kk < nk; kk += 32) {
            const int k = j0 + 1 + kk;
            float* dst = Vs + res_index<NB>(kk, l);
            if (l < nbp && k > j + 1) cp_async4(dst, src + k);
            else *dst = (l < nbp && k == j + 1) ? 1.0f : 0.0f;
        }
    }
    cp_commit();
}

constexpr int kTfSplit = 4;                   // row ranges of V^T V in the T-factor kernel

// scratch of the partial blocks of V^T V, in floats (aliases T and what follows it)
__host__ __device__ inline int tf_part_elems(int nb) { return kTfSplit * (nb / 4) * (nb / 4 + 1) / 2 * 16; }

struct TriTParams {
    int nwin;
    int maxp;                // panels per window at most
    const int* n_w;
    const long long* offA;
    const long long* offN;
    const float* A;
    const float* tau;
    float* T;                // [window][panel][NB][NB], upper triangular
    long long tstride;       // per window
    int ldv;
};

// T of the compact WY form of one panel, Q_p = I - V T V^T: T_ll = tau_l,
// T[0:l, l] = -tau_l T[0:l, 0:l] (V^T V)[0:l, l].  One CTA per (window, panel).
template <int NB>
__global__ void __launch_bounds__(128) tri_gram_kernel(TriTParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* const Vs = reinterpret_cast<float*>(smem_raw);      // [ldv][NB]
    float* const Gm = Vs + (size_t)p.ldv * NB;                  // [NB][NB]
    float* const Tm = Gm + NB * NB;                              // [NB][NB]; the partial blocks of G first
    const int w = blockIdx.x / p.maxp, panel = blockIdx.x % p.maxp;
    const int n = p.n_w[w];
    const int j0 = panel * NB;
    if (n > p.ldv || j0 >= n - 2) return;
    const int tid = threadIdx.x;
    const int nbp = min(NB, n - 2 - j0), nk = n - j0 - 1;
    const long long ld = (n + 3) & ~3;
    res_stage<128, NB>(Vs, p.A + p.offA[w], ld, j0, nbp, nk);
    cp_wait<0>();
    __syncthreads();
    // G = V^T V by 4 x 4 blocks on or above the diagonal (16-byte reads of the staged rows),
    // the rows split into kTfSplit ranges whose partial blocks are added in range order
    {
        constexpr int NQ = NB / 4, NTILE = NQ * (NQ + 1) / 2;
        float* const part = Tm;                                  // [kTfSplit][NTILE][16] scratch
        for (int item = tid; item < NTILE * kTfSplit; item += 128) {
            const int tile = item % NTILE, sp = item / NTILE;
            int qa = 0, rem = tile;                              // tile-th (qa <= qb) pair
            while (rem >= NQ - qa) {
                rem -= NQ - qa;
                ++qa;
            }
            const int qb = qa + rem;
            const int k0 = nk * sp / kTfSplit, k1 = nk * (sp + 1) / kTfSplit;
            float g[4][4] = {};
            for (int kk = k0; kk < k1; ++kk) {
                const float4 x = *reinterpret_cast<const float4*>(Vs + kk * NB + (((qa ^ (kk >> 2)) & (NQ - 1)) << 2));
                const float4 y = *reinterpret_cast<const float4*>(Vs + kk * NB + (((qb ^ (kk >> 2)) & (NQ - 1)) << 2));
                const float xa[4] = {x.x, x.y, x.z, x.w}, yb[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) g[r][c] = fmaf(xa[r], yb[c], g[r][c]);
            }
            float* dst = part + ((size_t)sp * NTILE + tile) * 16;
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) dst[r * 4 + c] = g[r][c];
        }
        __syncthreads();
        for (int item = tid; item < NTILE * 16; item += 128) {
            const int tile = item / 16, e = item % 16;
            int qa = 0, rem = tile;
            while (rem >= NQ - qa) {
                rem -= NQ - qa;
                ++qa;
            }
            const int qb = qa + rem;
            float s = 0.0f;
            for (int sp = 0; sp < kTfSplit; ++sp) s += part[((size_t)sp * NTILE + tile) * 16 + e];
            Gm[(4 * qa + e / 4) * NB + 4 * qb + e % 4] = s;
        }
        __syncthreads();
    }
    // G (the blocks on and above the diagonal) into the panel's T slot; tri_tfactor_kernel
    // turns it into T in place
    float* Gw = p.T + (long long)w * p.tstride + (long long)panel * NB * NB;
    for (int i = tid; i < NB * NB; i += 128) Gw[i] = Gm[i];
}

// T of the compact WY form of one panel from its G = V^T V (in the T slot), one warp per
// (window, panel): T_ll = tau_l, T[0:l, l] = -tau_l T[0:l, 0:l] G[0:l, l].  The recurrence is
// sequential in l; a warp per panel keeps many panels in flight on each SM.
template <int NB>
__global__ void __launch_bounds__(32) tri_tfactor_kernel(TriTParams p) {
    static_assert(NB <= 32, "one lane per reflector of the panel");
    __shared__ float Gm[NB * NB], Tm[NB * NB];
    const int w = blockIdx.x / p.maxp, panel = blockIdx.x % p.maxp;
    const int n = p.n_w[w];
    const int j0 = panel * NB;
    if (n > p.ldv || j0 >= n - 2) return;
    const int tid = threadIdx.x;
    const int nbp = min(NB, n - 2 - j0);
    float* Tw = p.T + (long long)w * p.tstride + (long long)panel * NB * NB;
    for (int i = tid; i < NB * NB; i += 32) Gm[i] = Tw[i];
    // the panel's tau, one per lane (NB <= 32), broadcast in the recurrence (no global load on
    // its sequential path)
    const float* tw = p.tau + p.offN[w];
    const float my_tau = tid < nbp ? tw[j0 + tid] : 0.0f;
    __syncwarp();
    for (int l = 0; l < NB; ++l) {
        const float tl = __shfl_sync(0xffffffffu, my_tau, l);
        for (int a = tid; a < NB; a += 32) {
            float val = 0.0f;
            if (a < l) {
                // four independent partial sums (b mod 4), added in a fixed order
                float s[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                int b = a;
                for (; b + 3 < l; b += 4) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) s[u] = fmaf(Tm[a * NB + b + u], Gm[(b + u) * NB + l], s[u]);
                }
                for (; b < l; ++b) s[0] = fmaf(Tm[a * NB + b], Gm[b * NB + l], s[0]);
                val = -tl * ((s[0] + s[1]) + (s[2] + s[3]));
            } else if (a == l) {
                val = tl;
            }
            Tm[a * NB + l] = val;
        }
        __syncwarp();
    }
    for (int i = tid; i < NB * NB; i += 32) Tw[i] = Tm[i];
}

inline size_t res_smem_bytes(int nb, int ldv, int rows) {
    return sizeof(float) * ((size_t)ldv * rows + (size_t)ldv * nb + (size_t)nb * rows + (size_t)nb * nb);
}

template <int NB>
__global__ void __launch_bounds__(kResNT, 1) tri_apply_res_kernel(TriApplyParams<float> p, const float* Tg,
                                                                  long long tstride, int rows) {
    constexpr int NG = NB / 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ldv = p.ldv;
    float* const Ys = reinterpret_cast<float*>(smem_raw);       // [ldv][rows]: Y[r][k] at Ys[k * rows + r]
    float* const Vs = Ys + (size_t)ldv * rows;                   // [ldv][NB], res_index layout
    float* const Ss = Vs + (size_t)ldv * NB;                     // [NB][rows]: S[r][l] at Ss[l * rows + r]
    float* const Tm = Ss + (size_t)NB * rows;                    // [NB][NB]
    const int4 item = p.items[blockIdx.x];
    const int w = item.x, r0 = item.y, nr = item.z;
    const int n = p.n_w[w], m = p.m_w[w];
    if (n > ldv || nr > rows) return;                           // flagged by the reduction / never built
    const long long ld = (n + 3) & ~3;
    const float* Aw = p.A + p.offA[w];
    const float* Fw = p.F + p.offF[w] + r0;
    float* Yw = p.Y + p.offF[w] + r0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rq = (nr + 31) / 32;                               // groups of 8 row quads
    for (int k = warp; k < n; k += kResNT / 32)                  // warp per column, lanes down the rows
        for (int r = lane; r < rq * 32; r += 32) {
            if (r < nr) cp_async4(Ys + (size_t)k * rows + r, Fw + r + (long long)k * m);
            else Ys[(size_t)k * rows + r] = 0.0f;
        }
    cp_commit();
    const int rt_l = lane & 7, ct_l = lane >> 3;                 // lane: row quad, reflector / column quad
    for (int j0 = 0; j0 < n - 2; j0 += NB) {
        const int nbp = min(NB, n - 2 - j0);
        const int nk = n - j0 - 1;
        const float* Tp = Tg + (long long)w * tstride + (long long)(j0 / NB) * NB * NB;
        __syncthreads();                                         // the previous panel is consumed
        res_stage<kResNT, NB>(Vs, Aw, ld, j0, nbp, nk);
        for (int i = tid; i < NB * NB; i += kResNT) cp_async4(Tm + i, Tp + i);
        cp_commit();
        cp_wait<0>();                                            // Y (first panel), V, T
        __syncthreads();
        const int nw1 = rq * (NB / 16);                          // 8 x 4 quad tiles of S (phase 2)
        // S = Y V over the panel rows: a warp = 4 row quads x 4 reflector quads x 2 halves of
        // the panel rows, the halves added by a shuffle
        {
            const int kh = lane >> 4, sub = lane & 15;
            const int rt_h = sub & 3, lt_h = sub >> 2;
            const int nwh = 2 * rq * (NB / 16);                  // warp tiles of S
            const int kmid = (nk + 1) >> 1;
            const int ka = kh ? kmid : 0, kz = kh ? nk : kmid;
            for (int wt = warp; wt < nwh; wt += kResNT / 32) {
                const int rt = (wt % (2 * rq)) * 4 + rt_h, lt = (wt / (2 * rq)) * 4 + lt_h;
                float acc[4][4] = {};
                const float* yp = Ys + (size_t)(j0 + 1) * rows + 4 * rt;
#pragma unroll 4
                for (int kk = ka; kk < kz; ++kk) {
                    const float4 y = *reinterpret_cast<const float4*>(yp + (size_t)kk * rows);
                    const float4 v = *reinterpret_cast<const float4*>(Vs + kk * NB + ((lt ^ (kk >> 2)) & (NG - 1)) * 4);
                    const float yy[4] = {y.x, y.y, y.z, y.w}, vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(yy[i], vv[j], acc[i][j]);
                }
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] += __shfl_xor_sync(0xffffffffu, acc[i][j], 16);
                if (kh == 0) {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        *reinterpret_cast<float4*>(Ss + (size_t)(4 * lt + j) * rows + 4 * rt) =
                            make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
                }
            }
        }
        __syncthreads();
        // S <- S T (T upper triangular)
        float st[4][4] = {};
        int st_rt = -1, st_bt = 0;
        if (warp < nw1) {                                        // nw1 <= 8: one tile per warp
            st_rt = (warp % rq) * 8 + rt_l;
            st_bt = (warp / rq) * 4 + ct_l;
            const int amax = min(NB, 4 * st_bt + 4);
            for (int a = 0; a < amax; ++a) {
                const float4 s = *reinterpret_cast<const float4*>(Ss + (size_t)a * rows + 4 * st_rt);
                const float4 tt = *reinterpret_cast<const float4*>(Tm + a * NB + 4 * st_bt);
                const float ss[4] = {s.x, s.y, s.z, s.w}, t4[4] = {tt.x, tt.y, tt.z, tt.w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) st[i][j] = fmaf(ss[i], t4[j], st[i][j]);
            }
        }
        __syncthreads();
        if (st_rt >= 0) {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                *reinterpret_cast<float4*>(Ss + (size_t)(4 * st_bt + j) * rows + 4 * st_rt) =
                    make_float4(st[0][j], st[1][j], st[2][j], st[3][j]);
        }
        __syncthreads();
        // Y <- Y - S V^T on the panel rows
        const int nw3 = rq * ((nk + 15) / 16);
        for (int wt = warp; wt < nw3; wt += kResNT / 32) {
            const int rt = (wt % rq) * 8 + rt_l, kt = (wt / rq) * 4 + ct_l;
            float acc[4][4] = {};                                // [row][column]
#pragma unroll
            for (int lc = 0; lc < NG; ++lc) {
                float s[4][4], v[4][4];                          // s[l][row], v[column][l]
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) {
                    const float4 x = *reinterpret_cast<const float4*>(Ss + (size_t)(4 * lc + jj) * rows + 4 * rt);
                    s[jj][0] = x.x; s[jj][1] = x.y; s[jj][2] = x.z; s[jj][3] = x.w;
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int kk = 4 * kt + q;
                    const float4 x = *reinterpret_cast<const float4*>(Vs + kk * NB + ((lc ^ kt) & (NG - 1)) * 4);
                    v[q][0] = x.x; v[q][1] = x.y; v[q][2] = x.z; v[q][3] = x.w;
                }
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int jj = 0; jj < 4; ++jj) acc[i][q] = fmaf(s[jj][i], v[q][jj], acc[i][q]);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int kk = 4 * kt + q;
                if (kk < nk) {
                    float4* yp = reinterpret_cast<float4*>(Ys + (size_t)(j0 + 1 + kk) * rows + 4 * rt);
                    float4 y = *yp;
                    y.x -= acc[0][q];
                    y.y -= acc[1][q];
                    y.z -= acc[2][q];
                    y.w -= acc[3][q];
                    *yp = y;
                }
            }
        }
    }
    cp_wait<0>();                                                // (no panel: the rows as loaded)
    __syncthreads();
    for (int k = warp; k < n; k += kResNT / 32)
        for (int r = lane; r < nr; r += 32) Yw[r + (long long)k * m] = Ys[(size_t)k * rows + r];
}

// ---------------------------------------------------------------------------
// shifted tridiagonal solves at all poles, fused with the pole sums
// ---------------------------------------------------------------------------

template <class R>
struct TriPassParams {
    int nitems;
    const int4* items;       // (window, first row, rows <= rows per batch, -)
    int* counter;
    const int* n_w;
    const int* m_w;
    const long long* offN;
    const long long* offF;   // rows Y[r + i*m]
    const long long* offQ;   // first point of each window in Oflat
    const long long* Oflat;  // grid index of every owned point (nullable: no density)
    const R* Y;
    const R* d;
    const R* e;
    int P;                   // poles (upper half plane)
    const typename Cplx<R>::T* shifts;
    const double2* wq;       // w_k
    const double2* wzq;      // w_k z_k
    double* dens;            // nullable
    double* part;            // [2 * nitems]: sum over the item's rows of n(r), e(r)
    int* status;
    int ldv;
};

constexpr int kPassNT = 256;
constexpr int kPassIC = 32;                   // steps per staged chunk
constexpr int kPassMaxRows = 256;             // rows per pass item at most

// Row groups of the pass kernel: thread = (pole, group), each group RR rows.
__host__ __device__ inline int pass_groups(int P, int RR) {
    const int g = kPassNT / P, cap = kPassMaxRows / RR;
    return g < cap ? g : cap;
}

inline size_t pass_smem_bytes(int elem, int P, int RR, int ldv) {
    const int RB = pass_groups(P, RR) * RR;
    return sizeof(double2) * (size_t)RB * P + (size_t)elem * (2 * (size_t)ldv + 2 * (size_t)kPassIC * RB);
}

// Unevaluated pairs of floats (hi + lo): the row sums of the FP32 pass and its pole
// weighting, with the rounding errors kept (Knuth's TwoSum, FMA-exact products), so that no
// FP64 arithmetic runs per item (GB300's FP64 rate is 1/64 of FP32).
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& ph, float& pl) {
    ph = ah * bh;
    pl = fmaf(ah, bh, -ph);
    pl = fmaf(ah, bl, pl);
    pl = fmaf(al, bh, pl);
}
// Re((ar + i ai)(qr + i qi)) as a pair
__device__ __forceinline__ void df_cre(const float4& a, float qrh, float qrl, float qih, float qil, float& h,
                                       float& l) {
    float p1h, p1l, p2h, p2l;
    df_mul(a.x, a.y, qrh, qrl, p1h, p1l);
    df_mul(a.z, a.w, qih, qil, p2h, p2l);
    h = p1h;
    l = p1l;
    df_add(h, l, -p2h);
    l -= p2l;
}
__device__ __forceinline__ float4 df_split(double2 a) {
    const float rh = (float)a.x, ih = (float)a.y;
    return make_float4(rh, (float)(a.x - (double)rh), ih, (float)(a.y - (double)ih));
}

// 1 / x correctly rounded (the value of R(1) / x)
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

template <class R, int NT, int RR>
__global__ void __launch_bounds__(NT) tri_pass_kernel(TriPassParams<R> p) {
    using C = typename Cplx<R>::T;
    constexpr int IC = kPassIC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int P = p.P;
    const int G = pass_groups(P, RR);              // row groups
    const int RB = G * RR;                         // rows per item
    constexpr bool kDF = sizeof(R) == 4;           // FP32 path: float pairs for the sums
    // [RB][P] weighted quadratic forms: (n, e) as double2, or (n_hi, n_lo, e_hi, e_lo)
    double2* const red = reinterpret_cast<double2*>(smem_raw);
    float4* const redf = reinterpret_cast<float4*>(smem_raw);
    R* const ds = reinterpret_cast<R*>(red + (size_t)RB * P);         // [ldv]
    R* const es = ds + p.ldv;                                         // [ldv]
    R* const yb = es + p.ldv;                                         // [2][IC][RB]
    __shared__ double sred[NT / 32];
    __shared__ int item_sh;
    const int tid = threadIdx.x;
    const int k = tid % P, g = tid / P;
    const bool on = g < G;
    float4 wsp = make_float4(0.f, 0.f, 0.f, 0.f), wzsp = wsp;      // w_k, w_k z_k split (FP32 path)
    if (kDF && on) {
        wsp = df_split(p.wq[k]);
        wzsp = df_split(p.wzq[k]);
    }

    for (;;) {
        if (tid == 0) item_sh = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= p.nitems) return;
        const int4 item = p.items[it];
        const int w = item.x, r0 = item.y, nr = item.z;
        const int n = p.n_w[w], m = p.m_w[w];
        if (n > p.ldv || nr > RB) {
            if (tid == 0) atomicOr(p.status, ST_BAD_SHAPE);
            __syncthreads();
            continue;
        }
        const R* Yw = p.Y + p.offF[w] + r0;
        for (int i = tid; i < n; i += NT) {
            ds[i] = p.d[p.offN[w] + i];
            es[i] = i < n - 1 ? p.e[p.offN[w] + i] : R(0);
        }
        // rows [r0, r0 + nr) of the window; steps i staged by chunks of IC
        auto stage = [&](int c, int buf) {
            R* dst = yb + (size_t)buf * IC * RB;
            for (int idx = tid; idx < IC * RB; idx += NT) {
                const int ic = idx / RB, row = idx % RB;
                const int i = c * IC + ic;
                if (row < nr && i < n) cp_async4(dst + idx, Yw + row + (long long)i * m);
                else dst[idx] = R(0);
            }
            cp_commit();
        };
        const int nch = (n + IC - 1) / IC;
        stage(0, 0);

        const C z = p.shifts[k < P ? k : 0];
        C gp = C{R(0), R(0)};                       // 1 / D_{i-1}
        C uc[RR], pr[RR];
        double2 acc[RR];                            // FP64 path: row sums
        float4 accf[RR];                            // FP32 path: (re_hi, re_lo, im_hi, im_lo)
#pragma unroll
        for (int u = 0; u < RR; ++u) {
            uc[u] = C{R(0), R(0)};
            pr[u] = C{R(0), R(0)};
            acc[u] = make_double2(0.0, 0.0);
            accf[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int c = 0; c < nch; ++c) {
            if (c + 1 < nch) {
                stage(c + 1, (c + 1) & 1);
                cp_wait<1>();
            } else {
                cp_wait<0>();
            }
            __syncthreads();                          // chunk c (and d, e) visible
            const R* yc = yb + (size_t)(c & 1) * IC * RB + g * RR;
            const int i0 = c * IC, i1 = min(n, i0 + IC);
            if (on) {
                for (int i = i0; i < i1; ++i) {
                    const R di = ds[i];
                    C t, D;
                    if (i == 0) {
                        t = C{R(0), R(0)};
                        D = C{z.x - di, z.y};
                    } else {
                        const R ei = es[i - 1];
                        t = C{ei * gp.x, ei * gp.y};
                        D = C{z.x - di - ei * t.x, z.y - ei * t.y};
                    }
                    const R inv = rcp_rn(D.x * D.x + D.y * D.y);
                    gp = C{D.x * inv, -D.y * inv};
                    // u^2 / D = (ur^2 - ui^2 + 2i ur ui) gp: the factor 2 (exact in binary) is
                    // carried by the pole's g2 = 2 gp, so each row takes one product ur ui
                    const C g2 = C{R(2) * gp.x, R(2) * gp.y};
                    const R* yi = yc + (size_t)(i - i0) * RB;
                    // the group's RR staged values of step i as 16-byte vectors (the chunk, the
                    // group offset g RR and the step stride RB are multiples of 16 bytes)
                    R yv[RR];
                    if constexpr (sizeof(R) == 4 && RR % 4 == 0) {
#pragma unroll
                        for (int q4 = 0; q4 < RR / 4; ++q4) {
                            const float4 v = reinterpret_cast<const float4*>(yi)[q4];
                            yv[4 * q4] = v.x;
                            yv[4 * q4 + 1] = v.y;
                            yv[4 * q4 + 2] = v.z;
                            yv[4 * q4 + 3] = v.w;
                        }
                    } else if constexpr (sizeof(R) == 8 && RR % 2 == 0) {
#pragma unroll
                        for (int q2 = 0; q2 < RR / 2; ++q2) {
                            const double2 v = reinterpret_cast<const double2*>(yi)[q2];
                            yv[2 * q2] = v.x;
                            yv[2 * q2 + 1] = v.y;
                        }
                    } else {
#pragma unroll
                        for (int u = 0; u < RR; ++u) yv[u] = yi[u];
                    }
#pragma unroll
                    for (int u = 0; u < RR; ++u) {
                        const R y = yv[u];
                        const R ur = fma(t.x, uc[u].x, fma(-t.y, uc[u].y, y));
                        const R ui = fma(t.x, uc[u].y, t.y * uc[u].x);
                        uc[u] = C{ur, ui};
                        const R sr = fma(ur, ur, -ui * ui);
                        const R q = ur * ui;
                        pr[u].x = fma(sr, gp.x, fma(-q, g2.y, pr[u].x));
                        pr[u].y = fma(sr, gp.y, fma(q, g2.x, pr[u].y));
                    }
                }
                // each chunk's sum is formed from zero and added to the row sums
#pragma unroll
                for (int u = 0; u < RR; ++u) {
                    if constexpr (kDF) {
                        df_add(accf[u].x, accf[u].y, (float)pr[u].x);
                        df_add(accf[u].z, accf[u].w, (float)pr[u].y);
                    } else {
                        acc[u].x += (double)pr[u].x;
                        acc[u].y += (double)pr[u].y;
                    }
                    pr[u] = C{R(0), R(0)};
                }
            }
            __syncthreads();                          // buffer c & 1 is free for chunk c + 2
        }
        // pole sums: n(r) = 4 Re sum_k w_k d_k(r), e(r) = 4 Re sum_k w_k z_k d_k(r)
        if (on) {
            if constexpr (kDF) {
#pragma unroll
                for (int u = 0; u < RR; ++u) {
                    float nh, nl, eh, el;
                    df_cre(wsp, accf[u].x, accf[u].y, accf[u].z, accf[u].w, nh, nl);
                    df_cre(wzsp, accf[u].x, accf[u].y, accf[u].z, accf[u].w, eh, el);
                    redf[(size_t)(g * RR + u) * P + k] = make_float4(nh, nl, eh, el);
                }
            } else {
                const double2 a = p.wq[k], b = p.wzq[k];
#pragma unroll
                for (int u = 0; u < RR; ++u) {
                    const double qx = acc[u].x, qy = acc[u].y;
                    red[(size_t)(g * RR + u) * P + k] = make_double2(a.x * qx - a.y * qy, b.x * qx - b.y * qy);
                }
            }
        }
        __syncthreads();
        double tn = 0.0, te = 0.0;
        for (int row = tid; row < nr; row += NT) {
            double sn = 0.0, se = 0.0;
            if constexpr (kDF) {
                float nh = 0.f, nl = 0.f, eh = 0.f, el = 0.f;
                for (int kk = 0; kk < P; ++kk) {
                    const float4 v = redf[(size_t)row * P + kk];
                    df_add(nh, nl, v.x);
                    nl += v.y;
                    df_add(eh, el, v.z);
                    el += v.w;
                }
                sn = (double)nh + (double)nl;
                se = (double)eh + (double)el;
            } else {
                for (int kk = 0; kk < P; ++kk) {
                    const double2 v = red[(size_t)row * P + kk];
                    sn += v.x;
                    se += v.y;
                }
            }
            const double nrow = 4.0 * sn, erow = 4.0 * se;
            if (!isfinite(nrow) || !isfinite(erow)) atomicOr(p.status, ST_ZERO_PIVOT);
            if (p.dens) p.dens[p.Oflat[p.offQ[w] + r0 + row]] = nrow;
            tn += nrow;
            te += erow;
        }
        tn = block_sum<NT>(tn, sred);
        te = block_sum<NT>(te, sred);
        if (tid == 0) {
            p.part[2 * (size_t)it] = tn;
            p.part[2 * (size_t)it + 1] = te;
        }
        __syncthreads();
    }
}

// per-window totals from the items of each window (contiguous, fixed order)
__global__ void tri_window_sums_kernel(int nwin, const int* first, const int* count, const double* part, double dV,
                                       double* nw, double* ew) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwin) return;
    double sn = 0.0, se = 0.0;
    for (int i = first[w]; i < first[w] + count[w]; ++i) {
        sn += part[2 * (size_t)i];
        se += part[2 * (size_t)i + 1];
    }
    nw[w] = sn * dV;
    ew[w] = se * dV;
}

// ---------------------------------------------------------------------------
// Sturm counts on T (FP64 arithmetic)
// ---------------------------------------------------------------------------

// Eigenvalues of the tridiagonal (d, e) below sigma = negative pivots of T - sigma I.
template <class R>
__device__ int sturm_count(int n, const R* d, const R* e, double sigma) {
    constexpr double pivmin = 1e-290;
    int cnt = 0;
    double q = (double)d[0] - sigma;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) ++cnt;
    for (int i = 1; i < n; ++i) {
        const double ee = (double)e[i - 1];
        q = ((double)d[i] - sigma) - ee * ee / q;
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0.0) ++cnt;
    }
    return cnt;
}

template <class R>
__global__ void tri_sturm_kernel(int nwin, const int* n_w, const long long* offN, const R* d, const R* e,
                                 double sigma, int* below) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwin) return;
    below[w] = sturm_count(n_w[w], d + offN[w], e + offN[w], sigma);
}

// Smallest eigenvalue of every window: bisection on the Sturm count from the Gershgorin
// interval down to width tol; lam[w] = midpoint of the last bracket.
template <class R>
__global__ void tri_mineig_kernel(int nwin, const int* n_w, const long long* offN, const R* d, const R* e,
                                  double tol, double* lam) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwin) return;
    const int n = n_w[w];
    const R* dw = d + offN[w];
    const R* ew = e + offN[w];
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < n; ++i) {
        const double r = (i > 0 ? fabs((double)ew[i - 1]) : 0.0) + (i < n - 1 ? fabs((double)ew[i]) : 0.0);
        lo = fmin(lo, (double)dw[i] - r);
        hi = fmax(hi, (double)dw[i] + r);
    }
    const double pad = 1e-12 * fmax(1.0, fmax(fabs(lo), fabs(hi)));
    double a = lo - pad, b = hi + pad;
    for (int iter = 0; iter < 200 && b - a > tol; ++iter) {
        const double mid = 0.5 * (a + b);
        if (sturm_count(n, dw, ew, mid) >= 1) b = mid;
        else a = mid;
    }
    lam[w] = 0.5 * (a + b);
}

}  // namespace

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

// Tile configurations of the tridiagonal route: reduction panel width and threads, row
// application panel width, rows per thread of the row-per-thread application and whether
// the rows stay resident in shared memory (res; FP32 only).  Panel widths are capped by
// what fits the shared memory at windows of nmax.
struct TriCfg {
    int nb, nt, nba, rpt, res, rres;     // rres: the reduction with the window in shared memory
    int rows;                            // resident application: rows per item at most
};
// Measured at 1024 electrons (mixed): reduction 6.7 ms with the L2-resident working copy
// (nb 16, 512 threads, two CTAs per SM; nb 8 6.75 ms, nb 32 7.35 ms; 256 threads at four CTAs
// per SM and 384 at three 7.8 ms), 8.1 ms with the window in shared memory (nb 8); row
// application 2.0 ms with resident rows (NB 32), 6.3 ms one row per thread.
static const TriCfg kTriCfg[6] = {{16, 512, 32, 1, 1, 0, 128}, {16, 512, 32, 1, 1, 1, 128},
                                  {16, 512, 32, 1, 0, 0, 0},    {16, 512, 16, 1, 1, 0, 64},
                                  {16, 512, 32, 1, 1, 0, 32},   {8, 512, 32, 1, 1, 1, 128}};

int tri_pick(bool fp32, int nmax, size_t smem_budget, int cfg, TriPick* out) {
    const int el = fp32 ? 4 : 8;
    TriPick r;
    r.ldv = (std::max(nmax, 1) + 31) / 32 * 32;
    if (cfg < 0 || cfg >= 6) cfg = 0;
    const TriCfg& t = kTriCfg[cfg];
    r.nt = t.nt;
    if (t.rres && fp32 && nmax <= kResReduceMaxN)
        for (int b : {16, 8, 4})
            if (b <= t.nb && !r.nb && (res_reduce_smem_elems(b, r.ldv, nmax) + r.ldv) * el <= smem_budget) {
                r.nb = b;
                r.nt = kResReduceNT;
                r.rres = 1;
            }
    for (int b : {32, 16, 8, 4})
        if (b <= t.nb && !r.nb && reduce_smem_elems(b, r.ldv, t.nt) * el <= smem_budget) r.nb = b;
    if (t.res && fp32)
        for (int b : {32, 16})
            for (int rows = std::min(kResRows, t.rows); rows >= 32 && !r.nb_apply; rows -= 32)
                if (b <= t.nba && res_smem_bytes(b, r.ldv, rows) <= smem_budget) {
                    r.nb_apply = b;
                    r.arows = rows;
                    r.rpt = 0;
                }
    if (!r.nb_apply) {
        for (int b : {32, 16, 8, 4})
            if (b <= t.nba && !r.nb_apply && (size_t)el * ((size_t)r.ldv * b + 2 * b * b) <= smem_budget) r.nb_apply = b;
        r.rpt = r.nb_apply >= 16 ? t.rpt : 1;
        r.arows = kAppRows;
    }
    if (!r.nb || !r.nb_apply) {
        lres_set_error("windows of %d functions exceed the shared memory of the tridiagonal reduction", nmax);
        return LRES_EINVAL;
    }
    // T factors of the resident application: panels of nb_apply, per window
    r.tstride = r.rpt == 0 ? (long long)(r.ldv / r.nb_apply + 1) * r.nb_apply * r.nb_apply : 0;
    *out = r;
    return LRES_OK;
}

template <class R, int NT>
static int launch_reduce(const TriReduceParams<R>& p, size_t smem_budget, cudaStream_t s) {
    const size_t smem = reduce_smem_elems(p.nb, p.ldv, NT) * sizeof(R);
    if (smem > smem_budget) {
        lres_set_error("tridiagonal reduction needs %zu B of shared memory", smem);
        return LRES_EINVAL;
    }
    int per_sm = 0;
    if (int rc = prepare_kernel<tri_reduce_kernel<R, NT>>(NT, smem, &per_sm)) return rc;
    const int grid = std::min(p.nwin, std::max(1, per_sm) * device_sms());
    tri_reduce_kernel<R, NT><<<grid, NT, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int tri_reduce(bool fp32, int nwin, const int* order, int* counter, const int* n_w, const long long* offC,
               const long long* offA, const long long* offN, const void* H, void* A, void* d, void* e, void* tau,
               int* status, const TriPick& pk, int nmax, size_t smem_budget, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    const int nb = pk.nb, nt = pk.nt, ldv = pk.ldv;
    LRES_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), s));
    if (fp32) {
        TriReduceParams<float> p{nwin, order, counter, n_w, offC, offA, offN, (const float*)H, (float*)A,
                                 (float*)d, (float*)e, (float*)tau, status, nb, ldv};
        if (pk.rres) {
            // as many partial-sum rows of p = A v (one per column segment) as fit, at most a warp each
            const size_t fixed = res_reduce_smem_elems(nb, ldv, nmax) * sizeof(float);
            const int nseg = fixed + sizeof(float) * ldv > smem_budget
                                 ? 0
                                 : (int)std::min<size_t>(kResReduceNT / 32, (smem_budget - fixed) / (sizeof(float) * ldv));
            if (nseg < 1 || nmax > kResReduceMaxN) {
                lres_set_error("resident tridiagonal reduction needs %zu B of shared memory", fixed + sizeof(float) * ldv);
                return LRES_EINVAL;
            }
            const size_t smem = fixed + sizeof(float) * (size_t)nseg * ldv;
            int per_sm = 0;
            if (int rc = prepare_kernel<tri_reduce_res_kernel<kResReduceNT>>(kResReduceNT, smem, &per_sm)) return rc;
            const int grid = std::min(nwin, std::max(1, per_sm) * device_sms());
            tri_reduce_res_kernel<kResReduceNT><<<grid, kResReduceNT, smem, s>>>(p, nmax, nseg);
            LRES_CUDA_TRY(cudaGetLastError());
            return LRES_OK;
        }
        return nt == 512 ? launch_reduce<float, 512>(p, smem_budget, s) : launch_reduce<float, 256>(p, smem_budget, s);
    }
    TriReduceParams<double> p{nwin, order, counter, n_w, offC, offA, offN, (const double*)H, (double*)A,
                              (double*)d, (double*)e, (double*)tau, status, nb, ldv};
    return nt == 512 ? launch_reduce<double, 512>(p, smem_budget, s) : launch_reduce<double, 256>(p, smem_budget, s);
}

template <class R, int NB, int RPT>
static int launch_apply(const TriApplyParams<R>& p, cudaStream_t s) {
    constexpr int NT = kAppRows / RPT;
    const size_t smem = sizeof(R) * ((size_t)p.ldv * NB + 2 * NB * NB);
    int per_sm = 0;
    if (int rc = prepare_kernel<tri_apply_kernel<R, NT, NB, RPT>>(NT, smem, &per_sm)) return rc;
    tri_apply_kernel<R, NT, NB, RPT><<<p.nitems, NT, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

template <class R>
static int dispatch_apply(const TriApplyParams<R>& p, int nb, int rpt, cudaStream_t s) {
    if (nb == 32 && rpt == 2) return launch_apply<R, 32, 2>(p, s);
    if (nb == 16 && rpt == 4) return launch_apply<R, 16, 4>(p, s);
    if (nb == 16 && rpt == 2) return launch_apply<R, 16, 2>(p, s);
    switch (nb) {
        case 32: return launch_apply<R, 32, 1>(p, s);
        case 16: return launch_apply<R, 16, 1>(p, s);
        case 8: return launch_apply<R, 8, 1>(p, s);
        case 4: return launch_apply<R, 4, 1>(p, s);
        default:
            lres_set_error("tridiagonal panel width %d not compiled", nb);
            return LRES_EINVAL;
    }
}

template <int NB>
static int launch_apply_res(const TriApplyParams<float>& p, const TriTParams& tp, int rows, size_t smem_budget,
                            cudaStream_t s) {
    const size_t smem_t = sizeof(float) * ((size_t)p.ldv * NB + NB * NB + std::max(NB * NB, tf_part_elems(NB)));
    const size_t smem = res_smem_bytes(NB, p.ldv, rows);
    if (smem > smem_budget || rows > kResRows || rows % 32) {
        lres_set_error("resident row application needs %zu B of shared memory", smem);
        return LRES_EINVAL;
    }
    int per_sm = 0;
    if (tp.maxp > 0 && tp.nwin > 0) {
        if (int rc = prepare_kernel<tri_gram_kernel<NB>>(128, smem_t, &per_sm)) return rc;
        tri_gram_kernel<NB><<<(unsigned)tp.nwin * tp.maxp, 128, smem_t, s>>>(tp);
        LRES_CUDA_TRY(cudaGetLastError());
        tri_tfactor_kernel<NB><<<(unsigned)tp.nwin * tp.maxp, 32, 0, s>>>(tp);
        LRES_CUDA_TRY(cudaGetLastError());
    }
    if (int rc = prepare_kernel<tri_apply_res_kernel<NB>>(kResNT, smem, &per_sm)) return rc;
    tri_apply_res_kernel<NB><<<p.nitems, kResNT, smem, s>>>(p, tp.T, tp.tstride, rows);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int tri_apply(bool fp32, int nitems, const int4* items, const int* n_w, const int* m_w, const long long* offA,
              const long long* offN, const long long* offF, const void* A, const void* tau, const void* F, void* Y,
              const TriPick& pk, int nwin, bool tfactors, void* T, size_t smem_budget, cudaStream_t s) {
    if (!nitems) return LRES_OK;
    if (fp32) {
        TriApplyParams<float> p{nitems, items, n_w, m_w, offA, offN, offF, (const float*)A, (const float*)tau,
                                (const float*)F, (float*)Y, pk.ldv};
        if (pk.rpt == 0) {
            if (!T) {
                lres_set_error("resident row application without a T-factor buffer");
                return LRES_ESTATE;
            }
            const int maxp = tfactors ? (pk.ldv + pk.nb_apply - 1) / pk.nb_apply : 0;
            TriTParams tp{nwin, maxp, n_w, offA, offN, (const float*)A, (const float*)tau, (float*)T, pk.tstride,
                          pk.ldv};
            if (pk.nb_apply == 32) return launch_apply_res<32>(p, tp, pk.arows, smem_budget, s);
            if (pk.nb_apply == 16) return launch_apply_res<16>(p, tp, pk.arows, smem_budget, s);
            lres_set_error("resident row application: panel width %d not compiled", pk.nb_apply);
            return LRES_EINVAL;
        }
        return dispatch_apply(p, pk.nb_apply, pk.rpt, s);
    }
    TriApplyParams<double> p{nitems, items, n_w, m_w, offA, offN, offF, (const double*)A, (const double*)tau,
                             (const double*)F, (double*)Y, pk.ldv};
    return dispatch_apply(p, pk.nb_apply, pk.rpt, s);
}

int tri_rows_per_item(bool fp32, int P) {
    const int RR = fp32 ? 8 : 4;
    return pass_groups(std::max(P, 1), RR) * RR;
}

template <class R, int RR>
static int launch_pass(const TriPassParams<R>& p, size_t smem_budget, cudaStream_t s) {
    const size_t smem = pass_smem_bytes(sizeof(R), p.P, RR, p.ldv);
    if (smem > smem_budget) {
        lres_set_error("pole pass needs %zu B of shared memory (P = %d, windows up to %d)", smem, p.P, p.ldv);
        return LRES_EINVAL;
    }
    int per_sm = 0;
    if (int rc = prepare_kernel<tri_pass_kernel<R, kPassNT, RR>>(kPassNT, smem, &per_sm)) return rc;
    const int grid = std::min(p.nitems, std::max(1, per_sm) * device_sms());
    tri_pass_kernel<R, kPassNT, RR><<<grid, kPassNT, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int tri_pass(bool fp32, int nitems, const int4* items, int* counter, const int* n_w, const int* m_w,
             const long long* offN, const long long* offF, const long long* offQ, const long long* Oflat,
             const void* Y, const void* d, const void* e, int P, const void* shifts, const double2* wq,
             const double2* wzq, double* dens, double* part, int* status, int ldv, size_t smem_budget,
             cudaStream_t s) {
    if (!nitems) return LRES_OK;
    if (P < 1 || P > kPassNT) {
        lres_set_error("pole pass supports 1..%d poles per half plane (got %d)", kPassNT, P);
        return LRES_EINVAL;
    }
    LRES_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), s));
    if (fp32) {
        TriPassParams<float> p{nitems, items, counter, n_w, m_w, offN, offF, offQ, Oflat, (const float*)Y,
                               (const float*)d, (const float*)e, P, (const float2*)shifts, wq, wzq, dens, part,
                               status, ldv};
        return launch_pass<float, 8>(p, smem_budget, s);
    }
    TriPassParams<double> p{nitems, items, counter, n_w, m_w, offN, offF, offQ, Oflat, (const double*)Y,
                            (const double*)d, (const double*)e, P, (const double2*)shifts, wq, wzq, dens, part,
                            status, ldv};
    return launch_pass<double, 4>(p, smem_budget, s);
}

int tri_window_sums(int nwin, const int* first, const int* count, const double* part, double dV, double* nw,
                    double* ew, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    tri_window_sums_kernel<<<(nwin + 127) / 128, 128, 0, s>>>(nwin, first, count, part, dV, nw, ew);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int tri_sturm(bool fp32, int nwin, const int* n_w, const long long* offN, const void* d, const void* e,
              double sigma, int* below, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    const int grid = (nwin + 63) / 64;
    if (fp32) tri_sturm_kernel<float><<<grid, 64, 0, s>>>(nwin, n_w, offN, (const float*)d, (const float*)e, sigma, below);
    else tri_sturm_kernel<double><<<grid, 64, 0, s>>>(nwin, n_w, offN, (const double*)d, (const double*)e, sigma, below);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int tri_min_eig(bool fp32, int nwin, const int* n_w, const long long* offN, const void* d, const void* e,
                double tol, double* lam, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    const int grid = (nwin + 31) / 32;
    if (fp32) tri_mineig_kernel<float><<<grid, 32, 0, s>>>(nwin, n_w, offN, (const float*)d, (const float*)e, tol, lam);
    else tri_mineig_kernel<double><<<grid, 32, 0, s>>>(nwin, n_w, offN, (const double*)d, (const double*)e, tol, lam);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

}  // namespace lres

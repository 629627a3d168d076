// Batched, fused window factor/solve for the LRes-DFT pole route (sm_103a).
//
// One CTA owns one work item (window w, shift k) at a time, pulled from a device
// work queue ordered largest window first.  For A = z_k B_w - C_w (complex
// symmetric for complex z; B = S_w or the identity, C = H_w or the standard-form
// H^_w) it runs a right-looking, pivot-free LDL^T factorisation of the
// AUGMENTED matrix
//
//        [ A     F ]        F = X[own(w), W]^T  (n x m basis values on owned points)
//        [ F^T   0 ]
//
// eliminating only the first n pivots.  The multipliers of the F^T rows are
// D^-1 L^-1 x_r, so the Schur-complement diagonal gives the quadratic forms
//
//        d_k(r) = x_r^T A^-1 x_r = sum_j l_rj^2 D_j         (no back substitution)
//
// which are all the pole route needs (density, electron count and band energy
// of window w follow by a weighted sum over poles).  For Im z > 0, Im A = Im(z) S
// is positive definite, so every leading block is nonsingular and no pivoting is
// required.  The same template runs in real double precision for
// Sylvester-inertia counts of (sigma S - H) and for the scaled multipliers that
// give L_c^-1 (Cholesky inverse) and L_c^-1 F when B = S and C = 0.
//
// Per panel of NB columns: (1) one warp factors the NB x NB diagonal block in
// shared memory, (2) every thread forward-solves its own rows of the panel
// against it in registers (no block-wide syncs), (3) the whole CTA applies the
// rank-NB update to the trailing lower trapezoid held in an L2-resident global
// workspace, with TR x TC register tiles.
//
// Work per item (the algorithmic unit used for roofline figures is the fixed
// (32/3) n^3 real flops of a complex LU + full inverse): about
// (2/3) n^3 + 2 n^2 m real FMAs (complex case: 4 real FMAs per complex MAC).
#include "common.cuh"
#include "launch.cuh"
#include "lres_internal.h"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace lres {

__device__ __forceinline__ double shfl(double x, int src) { return __shfl_sync(0xffffffffu, x, src); }
__device__ __forceinline__ double2 shfl(double2 x, int src) {
    return make_double2(__shfl_sync(0xffffffffu, x.x, src), __shfl_sync(0xffffffffu, x.y, src));
}
__device__ __forceinline__ float2 shfl(float2 x, int src) {
    return make_float2(__shfl_sync(0xffffffffu, x.x, src), __shfl_sync(0xffffffffu, x.y, src));
}

template <class T>
struct LdlParams {
    int nitems;
    const int2* items;          // (window, shift index)
    int* counter;               // work-queue head (zeroed before launch)
    const int* n_w;             // window dimension
    const int* m_w;             // right-hand-side rows (owned points)
    const long long* offC;      // window offset into C/B (n*n, column-major)
    const long long* offF;      // window offset into F (m*n, F[r + a*m])
    const long long* offQ;      // window offset into the point index space
    const typename El<T>::R* C; // nullable -> 0
    const typename El<T>::R* B; // nullable -> identity
    const typename El<T>::R* F; // nullable -> no right-hand sides
    const T* shifts;
    T* q;                       // q[k*qstride + offQ[w] + r]; nullable
    long long qstride;
    double* mult;               // real case: sqrt(D_j) l_rj at mult[offF[w] + r + j*m]; nullable
    int* npos;                  // per item: pivots with positive real part; nullable
    int* status;
    T* ws;                      // per-CTA workspace, ws_stride elements each
    long long ws_stride;
    int ldp;                    // shared panel leading dimension (>= max n + m)
    int nmax, mmax;
    int keep;                   // left-looking kernel: one workspace slot per item, the complete
                                // factor G (diagonal blocks and last panel included) is kept
    const int* c0;              // per window (nullable): F is zero in the columns before c0[w], so
                                // its rows of G are zero there too and are not computed
};

template <class T, int NB, int TR, int TC, int NT>
__global__ void __launch_bounds__(NT) ldl_aug_kernel(LdlParams<T> p) {
    using E = El<T>;
    using R = typename E::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* P = reinterpret_cast<T*>(smem_raw);          // NB x ldp panel, column kk at P + kk*ldp
    T* WL = P + (size_t)NB * p.ldp;                  // WL[kk*NB + kk2] = D_kk L_kk2,kk
    T* Dsh = WL + NB * NB;
    T* Dinv = Dsh + NB;
    T* Dsq = Dinv + NB;                              // sqrt(D) (complex case)
    T* qsh = Dsq + NB;                               // mmax
    __shared__ int item_sh;
    __shared__ int npos_sh;
    const int tid = threadIdx.x;
    const int ldp = p.ldp;
    T* ws = p.ws + (size_t)blockIdx.x * p.ws_stride;

    for (;;) {
        if (tid == 0) item_sh = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= p.nitems) return;
        const int w = p.items[it].x, k = p.items[it].y;
        const int n = p.n_w[w];
        const int m = p.F ? p.m_w[w] : 0;
        const int rows = n + m;
        const long long ld = rows;
        if (n > p.nmax || m > p.mmax) {
            if (tid == 0) atomicOr(p.status, ST_BAD_SHAPE);
            __syncthreads();
            continue;
        }
        const T z = p.shifts[k];
        const R* C = p.C ? p.C + p.offC[w] : nullptr;
        const R* B = p.B ? p.B + p.offC[w] : nullptr;
        const R* F = p.F ? p.F + p.offF[w] : nullptr;

        // ---- build the augmented lower trapezoid (one warp per column, lanes down the rows)
        {
            const int warp = tid >> 5, lane = tid & 31;
            for (int j = warp; j < n; j += NT / 32) {
                T* wcol = ws + (long long)j * ld;
                const R* Ccol = C ? C + (long long)j * n : nullptr;
                const R* Bcol = B ? B + (long long)j * n : nullptr;
                for (int i = j + lane; i < n; i += 32) {
                    const R b = Bcol ? Bcol[i] : (i == j ? R(1) : R(0));
                    const R c = Ccol ? Ccol[i] : R(0);
                    wcol[i] = E::shift_minus(z, b, c);
                }
                const R* Fcol = F ? F + (long long)j * m : nullptr;
                for (int r = lane; r < m; r += 32) wcol[n + r] = E::from(Fcol[r]);
            }
        }
        for (int r = tid; r < m; r += blockDim.x) qsh[r] = E::zero();
        if (tid == 0) npos_sh = 0;
        __syncthreads();

        for (int j0 = 0; j0 < n; j0 += NB) {
            const int nbj = min(NB, n - j0);
            const int prow = rows - j0;
            // ---- load panel columns [j0, j0+nbj), rows [j0, rows)
            for (int kk = tid >> 5; kk < nbj; kk += NT / 32) {
                const T* src = ws + j0 + (long long)(j0 + kk) * ld;
                for (int i = kk + (tid & 31); i < prow; i += 32) P[kk * ldp + i] = src[i];
            }
            __syncthreads();

            // ---- (1) diagonal block, one warp: lane = row, the row held in registers,
            //      multipliers exchanged by warp shuffles
            if (tid < 32) {
                const int lane = tid;
                T row[NB];
#pragma unroll
                for (int c = 0; c < NB; ++c)
                    row[c] = (c < nbj && lane < nbj && c <= lane) ? P[c * ldp + lane] : E::zero();
#pragma unroll
                for (int kk = 0; kk < NB; ++kk) {
                    if (kk < nbj) {
                        const T d = shfl(row[kk], kk);
                        const T dinv = E::inv(d);
                        const bool mine = lane > kk && lane < nbj;
                        const T l = mine ? E::mul(row[kk], dinv) : E::zero();
                        if (mine) row[kk] = l;
                        if (lane == kk) {
                            Dsh[kk] = d;
                            Dinv[kk] = dinv;
                            if constexpr (E::complex) Dsq[kk] = E::csqrt(d);
                            const double m2 = (double)E::mag2(d);
                            if (!(m2 > 0.0) || !isfinite(m2)) atomicOr(p.status, ST_ZERO_PIVOT);
                            if (E::re(d) > R(0)) ++npos_sh;
                        }
                        const T ldv = E::mul(l, d);
#pragma unroll
                        for (int c = kk + 1; c < NB; ++c) {
                            const T lc = shfl(l, c);
                            if (mine && c <= lane) row[c] = E::fms(ldv, lc, row[c]);
                        }
                    }
                }
                __syncwarp();
                // L below the diagonal back to shared memory; WL[kk*NB + lane] = D_kk L_lane,kk
#pragma unroll
                for (int kk = 0; kk < NB; ++kk) {
                    if (kk < nbj && lane > kk && lane < nbj) {
                        P[kk * ldp + lane] = row[kk];
                        WL[kk * NB + lane] = E::mul(Dsh[kk], row[kk]);
                    }
                }
            }
            __syncthreads();

            // ---- (2) panel rows below the diagonal block: per-row forward solve
            for (int i = nbj + tid; i < prow; i += blockDim.x) {
                T a[NB];
#pragma unroll
                for (int kk = 0; kk < NB; ++kk) a[kk] = (kk < nbj) ? P[kk * ldp + i] : E::zero();
#pragma unroll
                for (int kk = 0; kk < NB; ++kk) {
                    if (kk < nbj) {
                        const T l = E::mul(a[kk], Dinv[kk]);
#pragma unroll
                        for (int kk2 = kk + 1; kk2 < NB; ++kk2)
                            if (kk2 < nbj) a[kk2] = E::fms(l, WL[kk * NB + kk2], a[kk2]);
                        a[kk] = l;
                    }
                }
                // complex case: store l sqrt(D), so that the trailing update is a plain product
                // (L D L^T = (L sqrt D)(L sqrt D)^T for complex-symmetric A); real case: l
#pragma unroll
                for (int kk = 0; kk < NB; ++kk)
                    if (kk < nbj) P[kk * ldp + i] = E::complex ? E::mul(a[kk], Dsq[kk]) : a[kk];
                const int gi = j0 + i;
                if (gi >= n) {
                    const int r = gi - n;
                    if (p.q) {
                        T qv = qsh[r];
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk)
                            if (kk < nbj) qv = E::fma(E::mul(a[kk], a[kk]), Dsh[kk], qv);
                        qsh[r] = qv;
                    }
                    if constexpr (!E::complex) {
                        if (p.mult) {
                            double* mo = p.mult + p.offF[w];
#pragma unroll
                            for (int kk = 0; kk < NB; ++kk)
                                if (kk < nbj) mo[r + (long long)(j0 + kk) * m] = a[kk] * sqrt(Dsh[kk]);
                        }
                    }
                }
            }
            __syncthreads();

            // ---- (3) trailing update of rows [r0, rows) x cols [r0, n), lower part.
            //      Warp tile = (32*TR rows) x TC columns; lane l owns rows base + l + 32u, so
            //      shared loads are consecutive across the warp and column operands broadcast.
            const int r0 = j0 + nbj;
            if (r0 < n) {
                const int warp = tid >> 5, lane = tid & 31;
                const int nr = rows - r0, nc = n - r0;
                const int nrb = (nr + 32 * TR - 1) / (32 * TR), ncb = (nc + TC - 1) / TC;
                for (int wt = warp; wt < nrb * ncb; wt += NT / 32) {
                    const int rb = wt % nrb, cb = wt / nrb;
                    const int ib = r0 + rb * 32 * TR, c0 = r0 + cb * TC;
                    if (ib + 32 * TR - 1 < c0) continue;     // warp tile strictly above the diagonal
                    T cur[TR][TC];
                    bool ok[TR][TC];
#pragma unroll
                    for (int u = 0; u < TR; ++u) {
                        const int i = ib + lane + 32 * u;
#pragma unroll
                        for (int v = 0; v < TC; ++v) {
                            const int c = c0 + v;
                            ok[u][v] = i < rows && c < n && (i >= n || i >= c);
                            cur[u][v] = ok[u][v] ? ws[i + (long long)c * ld] : E::zero();
                        }
                    }
                    T acc[TR][TC];
#pragma unroll
                    for (int u = 0; u < TR; ++u)
#pragma unroll
                        for (int v = 0; v < TC; ++v) acc[u][v] = E::zero();
                    const T* Pr = P - j0 + ib + lane;
                    const T* Pc = P - j0 + c0;
                    for (int kk = 0; kk < nbj; ++kk) {
                        T wr[TR], lc[TC];
                        if constexpr (E::complex) {
#pragma unroll
                            for (int u = 0; u < TR; ++u)
                                wr[u] = (ib + lane + 32 * u < rows) ? Pr[kk * ldp + 32 * u] : E::zero();
                        } else {
                            const T dk = Dsh[kk];
#pragma unroll
                            for (int u = 0; u < TR; ++u)
                                wr[u] = (ib + lane + 32 * u < rows) ? E::mul(Pr[kk * ldp + 32 * u], dk) : E::zero();
                        }
#pragma unroll
                        for (int v = 0; v < TC; ++v) lc[v] = (c0 + v < n) ? Pc[kk * ldp + v] : E::zero();
#pragma unroll
                        for (int u = 0; u < TR; ++u)
#pragma unroll
                            for (int v = 0; v < TC; ++v) acc[u][v] = E::fma(wr[u], lc[v], acc[u][v]);
                    }
#pragma unroll
                    for (int u = 0; u < TR; ++u) {
                        const int i = ib + lane + 32 * u;
#pragma unroll
                        for (int v = 0; v < TC; ++v)
                            if (ok[u][v]) ws[i + (long long)(c0 + v) * ld] = E::sub(cur[u][v], acc[u][v]);
                    }
                }
            }
            __syncthreads();
        }

        // ---- outputs
        if (p.q) {
            T* qo = p.q + (long long)k * p.qstride + p.offQ[w];
            for (int r = tid; r < m; r += blockDim.x) qo[r] = qsh[r];
        }
        if (p.npos && tid == 0) p.npos[it] = npos_sh;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Left-looking variant for the complex pole solves (the production path).
//
// Panel j (columns [j0, j0+NB)) is accumulated in registers, one augmented row per
// thread, as  A[i, panel] - sum_{k < j0} G[i, k] G[panel, k]^T  with G = L sqrt(D)
// (complex symmetric: L D L^T = G G^T); the G rows of the panel columns are staged in
// shared memory in chunks of KC and broadcast, the row's own G[i, k] streams from the
// L2-resident workspace with coalesced loads.  The panel is then factored in place: the
// NB x NB diagonal block by one warp (registers and shuffles), every other row by a
// forward solve in its own registers, and only the finished G columns are written back.
// Compared with the right-looking form the trailing matrix is never read-modified-written:
// global traffic per item drops from ~rows*n*n/NB to ~rows*n*n/(2 NB) reads plus one write
// of G, and all loads are independent of the FMAs they feed.
// ---------------------------------------------------------------------------
// asynchronous global -> shared copies (cp.async, one element per instruction)
template <class T>
__device__ __forceinline__ void cp_async_el(T* dst, const T* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 16)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Copies rows [j0, j0+NB) x columns [k0, k0+kc) of G into buf[kk*NB + c].
template <class T, int NB, int NT, int KC>
__device__ __forceinline__ void stage_chunk(T* buf, const T* G, long long ld, int j0, int k0, int kc) {
    for (int idx = threadIdx.x; idx < kc * NB; idx += NT) {
        const int kk = idx / NB, c = idx % NB;
        cp_async_el(buf + idx, G + (j0 + c) + (long long)(k0 + kk) * ld);
    }
    cp_async_commit();
}

// SKIP: owned-point rows start at each window's first owned-point panel (compiled separately,
// so that contexts where no window can skip a panel run the plain batch loop).
template <class T, int NB, int NT, int KC, bool SKIP>
__global__ void __launch_bounds__(NT, 512 / NT) ldl_left_kernel(LdlParams<T> p) {
    using E = El<T>;
    using R = typename E::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* Bs = reinterpret_cast<T*>(smem_raw);          // [2][KC][NB]: Bs[kk*NB + c] = G[j0 + c, k0 + kk], double-buffered
    T* Dg = Bs + 2 * KC * NB;                        // [32][NB+1]: warp 0's rows (the diagonal block first)
    T* WL = Dg + 32 * (NB + 1);                      // [NB][NB]: WL[kk*NB + kk2] = D_kk L_kk2,kk
    T* Dsh = WL + NB * NB;
    T* Dinv = Dsh + NB;
    T* Dsq = Dinv + NB;
    T* accS = Dsq + NB;                              // [NB][NT]: the row's running panel values
    __shared__ int item_sh;
    const int tid = threadIdx.x;
    T* const Gcta = p.ws + (size_t)blockIdx.x * p.ws_stride;

    for (;;) {
        if (tid == 0) item_sh = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= p.nitems) return;
        T* const G = p.keep ? p.ws + (size_t)it * p.ws_stride : Gcta;
        const int w = p.items[it].x, k = p.items[it].y;
        const int n = p.n_w[w];
        const int m = p.F ? p.m_w[w] : 0;
        // The window is padded to np = a multiple of NB with identity rows/columns
        // (pivot 1, no coupling): every panel is full and the quadratic forms are unchanged.
        const int np = (n + NB - 1) / NB * NB;
        const int rows = np + m;
        const long long ld = rows;
        if (n > p.nmax || m > p.mmax) {
            if (tid == 0) atomicOr(p.status, ST_BAD_SHAPE);
            __syncthreads();
            continue;
        }
        const T z = p.shifts[k];
        const R* C = p.C ? p.C + p.offC[w] : nullptr;
        const R* B = p.B ? p.B + p.offC[w] : nullptr;
        const R* F = p.F ? p.F + p.offF[w] : nullptr;
        // quadratic forms accumulate in place in the output (any number of owned rows)
        T* const qg = p.q ? p.q + (long long)k * p.qstride + p.offQ[w] : nullptr;
        if (qg)
            for (int r = tid; r < m; r += NT) qg[r] = E::zero();
        __syncthreads();

        if constexpr (SKIP) {
        // Owned-point rows are zero before the window's first owned-point column c0 (the
        // solver orders the atoms that touch no owned point first), so their rows of G are
        // zero there too: they are processed from the panel holding c0 on, in row batches of
        // their own whose k sums start at that panel.
        // When no panel can be skipped (p0 == 0) the rows keep one common batch sequence.
        const int p0 = (p.c0 && m > 0) ? min(p.c0[w] / NB * NB, np) : 0;
        const bool split = p0 > 0;
        for (int j0 = 0; j0 < np; j0 += NB) {
            // one batch of NT rows starting b0 rows below the panel's first row; rows at
            // rend and beyond are inactive; the k sums start at kstart
            auto batch = [&](const int b0, const int rend, const int kstart) {
                const int ir = b0 + tid;              // row within the panel
                const int i = j0 + ir;
                const bool active = ir < rend;
                T acc[NB];
                if (active && i < n) {
                    const R* cp = C ? C + i + (long long)j0 * n : nullptr;
                    const R* bp = B ? B + i + (long long)j0 * n : nullptr;
#pragma unroll
                    for (int c = 0; c < NB; ++c) {
                        const int col = j0 + c;
                        T a = E::zero();
                        if (col <= i) {                // lower triangle (col < n follows)
                            const R bb = bp ? bp[(long long)c * n] : (i == col ? R(1) : R(0));
                            const R cc = cp ? cp[(long long)c * n] : R(0);
                            a = E::shift_minus(z, bb, cc);
                        }
                        acc[c] = a;
                    }
                } else if (active && i < np) {        // padding row: identity
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c == i) ? E::from(R(1)) : E::zero();
                } else if (active) {                  // right-hand-side row r = i - np
                    const R* fp = F + (i - np) + (long long)j0 * m;
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c < n) ? E::from(fp[(long long)c * m]) : E::zero();
                } else {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = E::zero();
                }
                // Blocked accumulation: each KC-chunk of the k sum is formed from zero in
                // registers and subtracted from the row's running value, kept in shared memory
                // (the same rounding pattern as a right-looking update by KC-wide panels).
                // chunks of the panel's G rows are copied asynchronously into a double buffer:
                // chunk ci+1 is in flight while chunk ci is used; one barrier per chunk
                const int nch = (j0 - kstart + KC - 1) / KC;
                if (nch > 0) {
#pragma unroll
                    for (int c = 0; c < NB; ++c) accS[c * NT + tid] = acc[c];
                    __syncthreads();                  // the previous loop's last buffer is free
                    stage_chunk<T, NB, NT, KC>(Bs, G, ld, j0, kstart, min(KC, j0 - kstart));
                }
                for (int ci = 0; ci < nch; ++ci) {
                    const int k0 = kstart + ci * KC;
                    const int kc = min(KC, j0 - k0);   // a multiple of 8
                    cp_async_wait_all();
                    __syncthreads();                  // chunk ci visible; chunk ci-1 consumed
                    if (ci + 1 < nch)
                        stage_chunk<T, NB, NT, KC>(Bs + ((ci + 1) & 1) * KC * NB, G, ld, j0, k0 + KC,
                                                   min(KC, j0 - k0 - KC));
                    if (active) {
                        const T* gi = G + i + (long long)k0 * ld;
                        const T* bbuf = Bs + (ci & 1) * KC * NB;
                        T tmp[NB];
#pragma unroll
                        for (int c = 0; c < NB; ++c) tmp[c] = E::zero();
                        T g0 = gi[0], g1 = gi[ld];
                        for (int kk = 0; kk < kc; kk += 2) {
                            T n0 = g0, n1 = g1;
                            if (kk + 2 < kc) {        // prefetch the next pair of the row's G values
                                n0 = gi[(long long)(kk + 2) * ld];
                                n1 = gi[(long long)(kk + 3) * ld];
                            }
                            const T* b = bbuf + kk * NB;
#pragma unroll
                            for (int c = 0; c < NB; ++c) {
                                T a = tmp[c];
                                a = E::fma(g0, b[c], a);
                                a = E::fma(g1, b[NB + c], a);
                                tmp[c] = a;
                            }
                            g0 = n0;
                            g1 = n1;
                        }
#pragma unroll
                        for (int c = 0; c < NB; ++c) accS[c * NT + tid] = E::sub(accS[c * NT + tid], tmp[c]);
                    }
                }
                if (nch > 0) {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = accS[c * NT + tid];
                }
                if (b0 == 0) {
                    // warp 0 parks its accumulated rows (the diagonal block is rows 0..NB-1)
                    // in shared memory while it factors the block, then reloads them
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) Dg[tid * (NB + 1) + c] = acc[c];
                    }
                    __syncthreads();
                    if (tid < 32) {
                        // LDL^T of the NB x NB diagonal block in shared memory: lane = row;
                        // the column operand L_c,kk is a broadcast read of row c
                        const int lane = tid;
                        T* myrow = Dg + lane * (NB + 1);
                        for (int kk = 0; kk < NB; ++kk) {
                            __syncwarp();
                            const T d = Dg[kk * (NB + 1) + kk];
                            const T dinv = E::inv(d);
                            const bool mine = lane > kk && lane < NB;
                            T l = E::zero();
                            if (mine) {
                                l = E::mul(myrow[kk], dinv);
                                myrow[kk] = l;
                            }
                            if (lane == kk) {
                                Dsh[kk] = d;
                                Dinv[kk] = dinv;
                                Dsq[kk] = E::csqrt(d);
                                const double m2 = (double)E::mag2(d);
                                if (!(m2 > 0.0) || !isfinite(m2)) atomicOr(p.status, ST_ZERO_PIVOT);
                            }
                            __syncwarp();
                            if (mine) {
                                const T ldv = E::mul(l, d);
                                for (int c = kk + 1; c <= lane; ++c)
                                    myrow[c] = E::fms(ldv, Dg[c * (NB + 1) + kk], myrow[c]);
                            }
                        }
                        __syncwarp();
                        for (int kk = 0; kk < NB; ++kk)
                            if (lane > kk && lane < NB) WL[kk * NB + lane] = E::mul(Dsh[kk], myrow[kk]);
                        if (p.keep && lane < NB) {     // the block's G = L sqrt(D), lower part
                            T* gd = G + (j0 + lane) + (long long)j0 * ld;
                            for (int c = 0; c <= lane; ++c)
                                gd[(long long)c * ld] = c == lane ? Dsq[c] : E::mul(myrow[c], Dsq[c]);
                        }
                    }
                    __syncthreads();
                    // warp 0 reloads its parked rows (rows below the block still need the solve)
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) acc[c] = Dg[tid * (NB + 1) + c];
                    }
                    __syncthreads();
                }
                if (active && ir >= NB) {
#pragma unroll
                    for (int kk = 0; kk < NB; ++kk) {
                        const T l = E::mul(acc[kk], Dinv[kk]);
#pragma unroll
                        for (int kk2 = kk + 1; kk2 < NB; ++kk2) acc[kk2] = E::fms(l, WL[kk * NB + kk2], acc[kk2]);
                        acc[kk] = l;
                    }
                    if (i >= np && qg) {
                        // the panel's NB terms of the quadratic form summed from zero, then added
                        // (blocked summation: one FP32 chain over all n terms loses ~10x accuracy)
                        T part = E::zero();
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) part = E::fma(E::mul(acc[kk], acc[kk]), Dsh[kk], part);
                        qg[i - np] = E::add(qg[i - np], part);
                    }
                    if (j0 + NB < np || p.keep) {
                        T* gout = G + i + (long long)j0 * ld;
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) gout[(long long)kk * ld] = E::mul(acc[kk], Dsq[kk]);
                    }
                }
            };
            if (!split) {
                const int na = rows - j0;
                for (int b0 = 0; b0 < na; b0 += NT) batch(b0, na, 0);
            } else {
                const int nA = np - j0;               // window rows, then (from panel p0 on) owned rows
                for (int b0 = 0; b0 < nA; b0 += NT) batch(b0, nA, 0);
                if (j0 >= p0)
                    for (int b0 = nA; b0 < rows - j0; b0 += NT) batch(b0, rows - j0, p0);
            }
            __syncthreads();                          // finished G columns visible to the next panel
        }
        } else {
        for (int j0 = 0; j0 < np; j0 += NB) {
            const int na = rows - j0;
            for (int b0 = 0; b0 < na; b0 += NT) {
                const int ir = b0 + tid;              // row within the panel
                const int i = j0 + ir;
                const bool active = ir < na;
                T acc[NB];
                if (active && i < n) {
                    const R* cp = C ? C + i + (long long)j0 * n : nullptr;
                    const R* bp = B ? B + i + (long long)j0 * n : nullptr;
#pragma unroll
                    for (int c = 0; c < NB; ++c) {
                        const int col = j0 + c;
                        T a = E::zero();
                        if (col <= i) {                // lower triangle (col < n follows)
                            const R bb = bp ? bp[(long long)c * n] : (i == col ? R(1) : R(0));
                            const R cc = cp ? cp[(long long)c * n] : R(0);
                            a = E::shift_minus(z, bb, cc);
                        }
                        acc[c] = a;
                    }
                } else if (active && i < np) {        // padding row: identity
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c == i) ? E::from(R(1)) : E::zero();
                } else if (active) {                  // right-hand-side row r = i - np
                    const R* fp = F + (i - np) + (long long)j0 * m;
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c < n) ? E::from(fp[(long long)c * m]) : E::zero();
                } else {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = E::zero();
                }
                // Blocked accumulation: each KC-chunk of the k sum is formed from zero in
                // registers and subtracted from the row's running value, kept in shared memory
                // (the same rounding pattern as a right-looking update by KC-wide panels).
                if (j0 > 0) {
#pragma unroll
                    for (int c = 0; c < NB; ++c) accS[c * NT + tid] = acc[c];
                }
                // chunks of the panel's G rows are copied asynchronously into a double buffer:
                // chunk ci+1 is in flight while chunk ci is used; one barrier per chunk
                const int nch = (j0 + KC - 1) / KC;
                if (nch > 0) {
                    __syncthreads();                  // the previous loop's last buffer is free
                    stage_chunk<T, NB, NT, KC>(Bs, G, ld, j0, 0, min(KC, j0));
                }
                for (int ci = 0; ci < nch; ++ci) {
                    const int k0 = ci * KC;
                    const int kc = min(KC, j0 - k0);   // a multiple of 8
                    cp_async_wait_all();
                    __syncthreads();                  // chunk ci visible; chunk ci-1 consumed
                    if (ci + 1 < nch)
                        stage_chunk<T, NB, NT, KC>(Bs + ((ci + 1) & 1) * KC * NB, G, ld, j0, k0 + KC,
                                                   min(KC, j0 - k0 - KC));
                    if (active) {
                        const T* gi = G + i + (long long)k0 * ld;
                        const T* bbuf = Bs + (ci & 1) * KC * NB;
                        T tmp[NB];
#pragma unroll
                        for (int c = 0; c < NB; ++c) tmp[c] = E::zero();
                        T g0 = gi[0], g1 = gi[ld];
                        for (int kk = 0; kk < kc; kk += 2) {
                            T n0 = g0, n1 = g1;
                            if (kk + 2 < kc) {        // prefetch the next pair of the row's G values
                                n0 = gi[(long long)(kk + 2) * ld];
                                n1 = gi[(long long)(kk + 3) * ld];
                            }
                            const T* b = bbuf + kk * NB;
#pragma unroll
                            for (int c = 0; c < NB; ++c) {
                                T a = tmp[c];
                                a = E::fma(g0, b[c], a);
                                a = E::fma(g1, b[NB + c], a);
                                tmp[c] = a;
                            }
                            g0 = n0;
                            g1 = n1;
                        }
#pragma unroll
                        for (int c = 0; c < NB; ++c) accS[c * NT + tid] = E::sub(accS[c * NT + tid], tmp[c]);
                    }
                }
                if (j0 > 0) {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = accS[c * NT + tid];
                }
                if (b0 == 0) {
                    // warp 0 parks its accumulated rows (the diagonal block is rows 0..NB-1)
                    // in shared memory while it factors the block, then reloads them
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) Dg[tid * (NB + 1) + c] = acc[c];
                    }
                    __syncthreads();
                    if (tid < 32) {
                        // LDL^T of the NB x NB diagonal block in shared memory: lane = row;
                        // the column operand L_c,kk is a broadcast read of row c
                        const int lane = tid;
                        T* myrow = Dg + lane * (NB + 1);
                        for (int kk = 0; kk < NB; ++kk) {
                            __syncwarp();
                            const T d = Dg[kk * (NB + 1) + kk];
                            const T dinv = E::inv(d);
                            const bool mine = lane > kk && lane < NB;
                            T l = E::zero();
                            if (mine) {
                                l = E::mul(myrow[kk], dinv);
                                myrow[kk] = l;
                            }
                            if (lane == kk) {
                                Dsh[kk] = d;
                                Dinv[kk] = dinv;
                                Dsq[kk] = E::csqrt(d);
                                const double m2 = (double)E::mag2(d);
                                if (!(m2 > 0.0) || !isfinite(m2)) atomicOr(p.status, ST_ZERO_PIVOT);
                            }
                            __syncwarp();
                            if (mine) {
                                const T ldv = E::mul(l, d);
                                for (int c = kk + 1; c <= lane; ++c)
                                    myrow[c] = E::fms(ldv, Dg[c * (NB + 1) + kk], myrow[c]);
                            }
                        }
                        __syncwarp();
                        for (int kk = 0; kk < NB; ++kk)
                            if (lane > kk && lane < NB) WL[kk * NB + lane] = E::mul(Dsh[kk], myrow[kk]);
                        if (p.keep && lane < NB) {     // the block's G = L sqrt(D), lower part
                            T* gd = G + (j0 + lane) + (long long)j0 * ld;
                            for (int c = 0; c <= lane; ++c)
                                gd[(long long)c * ld] = c == lane ? Dsq[c] : E::mul(myrow[c], Dsq[c]);
                        }
                    }
                    __syncthreads();
                    // warp 0 reloads its parked rows (rows below the block still need the solve)
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) acc[c] = Dg[tid * (NB + 1) + c];
                    }
                    __syncthreads();
                }
                if (active && ir >= NB) {
#pragma unroll
                    for (int kk = 0; kk < NB; ++kk) {
                        const T l = E::mul(acc[kk], Dinv[kk]);
#pragma unroll
                        for (int kk2 = kk + 1; kk2 < NB; ++kk2) acc[kk2] = E::fms(l, WL[kk * NB + kk2], acc[kk2]);
                        acc[kk] = l;
                    }
                    if (i >= np && qg) {
                        // the panel's NB terms of the quadratic form summed from zero, then added
                        // (blocked summation: one FP32 chain over all n terms loses ~10x accuracy)
                        T part = E::zero();
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) part = E::fma(E::mul(acc[kk], acc[kk]), Dsh[kk], part);
                        qg[i - np] = E::add(qg[i - np], part);
                    }
                    if (j0 + NB < np || p.keep) {
                        T* gout = G + i + (long long)j0 * ld;
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) gout[(long long)kk * ld] = E::mul(acc[kk], Dsq[kk]);
                    }
                }
            }
            __syncthreads();                          // finished G columns visible to the next panel
        }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Tensor-core variant of the left-looking kernel (complex FP32 path, tile configuration 4).
//
// The panel update of a 16-column chunk, tmp[r, c] = sum_k g[r, k] b[c, k] (complex), is a
// real GEMM  [Re g | Im g] (128 x 32) . B' (64 x 32)^T  with B' built from the panel's G rows
// ([b_re, -b_im ; b_im, b_re] per complex entry), run on the 5th-generation tensor cores:
// operands in shared memory (K-major, no swizzle, 8 x 16-byte core matrices), accumulator in
// tensor memory, tcgen05.mma issued by one thread, completion through an mbarrier.  FP32
// accuracy from TF32 operands by the 3xTF32 split x = hi + lo: hi.hi + hi.lo + lo.hi, each
// chunk accumulated from zero in FP32 and subtracted from the row's running value in
// registers (blocked summation, as the SIMT kernel).
//
// Pipeline: two shared-memory stages and two TMEM accumulators.  While the tensor core runs
// the MMAs of chunk c+1, the threads read back chunk c and split/stage chunk c+2, whose
// operands were loaded into registers two chunks earlier.  128 threads = 128 rows = 128 TMEM
// lanes; two CTAs per SM, so that one CTA's panel factorisation overlaps the other's MMAs.
// Every wait on an mbarrier is bounded: on a timeout the kernel sets ST_TIMEOUT, waits
// (bounded) for the MMAs it has in flight, frees its tensor memory and returns.
// ---------------------------------------------------------------------------
namespace tc {
constexpr int M = 128, N = 64, KR = 32, KCC = 16;   // real GEMM per chunk; complex columns per chunk
constexpr int LBO = 128;                             // bytes between core matrices along K
constexpr int SBO = (KR / 4) * 128;                  // bytes between 8-row groups
constexpr int A_BYTES = M * KR * 4, B_BYTES = N * KR * 4;
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;   // Ahi, Alo, Bhi, Blo
constexpr int TMEM_COLS = 128;                       // two 64-column accumulators
__device__ __forceinline__ int off(int row, int k) { return (row >> 3) * SBO + (k >> 2) * LBO + (row & 7) * 16 + (k & 3) * 4; }
__device__ __forceinline__ uint64_t desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((LBO >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((SBO >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
__device__ __forceinline__ float tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
__device__ __forceinline__ void split(float x, float& hi, float& lo) {
    hi = tf32(x);
    lo = tf32(x - hi);
}
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t accumulate) {
    asm volatile("{ .reg .pred p; setp.ne.u32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }"
                 ::"r"(tmem), "l"(ad), "l"(bd), "r"(IDESC), "r"(accumulate));
}
__device__ __forceinline__ void ld64(uint32_t taddr, float* v) {
    uint32_t r[64];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
                 "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
                 "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                   "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                   "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
                   "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
                   "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
                   "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
                   "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 64; ++j) v[j] = __uint_as_float(r[j]);
}
// bounded wait on an mbarrier phase; true when it completed
__device__ __forceinline__ bool wait_phase(uint32_t mbar, uint32_t phase) {
    uint32_t done = 0;
    for (int spin = 0; spin < (1 << 24) && !done; ++spin)
        asm volatile("{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n"
                     "selp.u32 %0, 1, 0, q; }" : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
    return done != 0;
}
}  // namespace tc

__global__ void __launch_bounds__(128, 2) ldl_left_tc_kernel(LdlParams<float2> p) {
    using T = float2;
    using E = El<T>;
    constexpr int NB = 32, NT = 128, KCC = tc::KCC;
    extern __shared__ __align__(128) unsigned char smem_tc[];
    // stage s: Ahi, Alo (128 x 32 real), Bhi, Blo (64 x 32 real), K-major core matrices
    unsigned char* stage0 = smem_tc;
    T* WL = reinterpret_cast<T*>(smem_tc + 2 * tc::STAGE_BYTES);    // [NB][NB]
    T* Dsh = WL + NB * NB;
    T* Dinv = Dsh + NB;
    T* Dsq = Dinv + NB;
    T* Dg = reinterpret_cast<T*>(smem_tc + tc::STAGE_BYTES);        // [32][NB+1], aliases stage 1 (free then)
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int item_sh, bail_sh;
    const int tid = threadIdx.x, warp = tid >> 5;
    T* G = p.ws + (size_t)blockIdx.x * p.ws_stride;
    const uint32_t mb0 = (uint32_t)__cvta_generic_to_shared(&mbar[0]);
    const uint32_t mb1 = (uint32_t)__cvta_generic_to_shared(&mbar[1]);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(stage0);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb0));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb1));
        bail_sh = 0;
    }
    if (warp == 0) {
        const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "n"(tc::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    const uint32_t my_lane = (uint32_t)(warp * 32) << 16;
    uint32_t ph0 = 0u, ph1 = 0u;                        // mbarrier phases
    int pend0 = 0, pend1 = 0;                           // MMAs committed and not yet waited for

    for (;;) {
        if (tid == 0) item_sh = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= p.nitems || bail_sh) break;
        const int w = p.items[it].x, k = p.items[it].y;
        const int n = p.n_w[w];
        const int m = p.F ? p.m_w[w] : 0;
        const int np = (n + NB - 1) / NB * NB;
        const int rows = np + m;
        const long long ld = rows;
        if (n > p.nmax || m > p.mmax) {
            if (tid == 0) atomicOr(p.status, ST_BAD_SHAPE);
            __syncthreads();
            continue;
        }
        const T z = p.shifts[k];
        const float* C = p.C ? p.C + p.offC[w] : nullptr;
        const float* F = p.F ? p.F + p.offF[w] : nullptr;
        T* const qg = p.q ? p.q + (long long)k * p.qstride + p.offQ[w] : nullptr;
        if (qg)
            for (int r = tid; r < m; r += NT) qg[r] = E::zero();
        __syncthreads();

        for (int j0 = 0; j0 < np && !bail_sh; j0 += NB) {
            const int na = rows - j0;
            for (int b0 = 0; b0 < na; b0 += NT) {
                const int ir = b0 + tid;
                const int i = j0 + ir;
                const bool active = ir < na;
                T acc[NB];
                if (active && i < n) {
                    const float* cp = C + i + (long long)j0 * n;
#pragma unroll
                    for (int c = 0; c < NB; ++c) {
                        const int col = j0 + c;
                        acc[c] = (col <= i) ? E::shift_minus(z, (i == col ? 1.f : 0.f), cp[(long long)c * n]) : E::zero();
                    }
                } else if (active && i < np) {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c == i) ? E::from(1.f) : E::zero();
                } else if (active) {
                    const float* fp = F + (i - np) + (long long)j0 * m;
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c < n) ? E::from(fp[(long long)c * m]) : E::zero();
                } else {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = E::zero();
                }
                const int nch = j0 / KCC;                 // j0 is a multiple of 32: nch even
                if (nch > 0) {
                    // operands of two chunks in registers (slot a0/b0r: even chunks, a1/b1r: odd)
                    T a0[KCC], a1[KCC], b0r[4], b1r[4];
                    const T* grow = G + i;
                    auto load = [&](int c, T (&ar)[KCC], T (&br)[4]) {
                        const int k0 = c * KCC;
#pragma unroll
                        for (int kk = 0; kk < KCC; ++kk) ar[kk] = active ? grow[(long long)(k0 + kk) * ld] : E::zero();
                        // panel values: thread = (row cc = tid % 32, k pairs 2p, 2p+1 and 2p+8, 2p+9)
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int cc = tid & 31, kk = 2 * (tid >> 5) + (q & 1) + 8 * (q >> 1);
                            br[q] = G[(j0 + cc) + (long long)(k0 + kk) * ld];
                        }
                    };
                    auto stage = [&](const T (&ar)[KCC], const T (&br)[4], int st) {
                        unsigned char* Ahi = stage0 + st * tc::STAGE_BYTES;
                        unsigned char* Alo = Ahi + tc::A_BYTES;
                        unsigned char* Bhi = Ahi + 2 * tc::A_BYTES;
                        unsigned char* Blo = Bhi + tc::B_BYTES;
                        // 16-byte stores: two complex k values = the 4 real K of one core-matrix row
#pragma unroll
                        for (int kk = 0; kk < KCC; kk += 2) {
                            float rh0, rl0, ih0, il0, rh1, rl1, ih1, il1;
                            tc::split(ar[kk].x, rh0, rl0);
                            tc::split(ar[kk].y, ih0, il0);
                            tc::split(ar[kk + 1].x, rh1, rl1);
                            tc::split(ar[kk + 1].y, ih1, il1);
                            *reinterpret_cast<float4*>(Ahi + tc::off(tid, 2 * kk)) = make_float4(rh0, ih0, rh1, ih1);
                            *reinterpret_cast<float4*>(Alo + tc::off(tid, 2 * kk)) = make_float4(rl0, il0, rl1, il1);
                        }
#pragma unroll
                        for (int q = 0; q < 4; q += 2) {
                            const int cc = tid & 31, kk = 2 * (tid >> 5) + 8 * (q >> 1);
                            float rh0, rl0, ih0, il0, rh1, rl1, ih1, il1;
                            tc::split(br[q].x, rh0, rl0);
                            tc::split(br[q].y, ih0, il0);
                            tc::split(br[q + 1].x, rh1, rl1);
                            tc::split(br[q + 1].y, ih1, il1);
                            // rows 2cc (real part of the output) and 2cc+1 (imaginary), K columns 2kk..2kk+3
                            *reinterpret_cast<float4*>(Bhi + tc::off(2 * cc, 2 * kk)) = make_float4(rh0, -ih0, rh1, -ih1);
                            *reinterpret_cast<float4*>(Blo + tc::off(2 * cc, 2 * kk)) = make_float4(rl0, -il0, rl1, -il1);
                            *reinterpret_cast<float4*>(Bhi + tc::off(2 * cc + 1, 2 * kk)) = make_float4(ih0, rh0, ih1, rh1);
                            *reinterpret_cast<float4*>(Blo + tc::off(2 * cc + 1, 2 * kk)) = make_float4(il0, rl0, il1, rl1);
                        }
                    };
                    // stage st staged by every thread; one thread issues its 12 MMAs into
                    // accumulator st and commits them to mbarrier st
                    auto issue = [&](int st) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        __syncthreads();
                        asm volatile("tcgen05.fence::after_thread_sync;");
                        if (tid == 0) {
                            const uint32_t aH = sbase + st * tc::STAGE_BYTES, aL = aH + tc::A_BYTES;
                            const uint32_t bH = aH + 2 * tc::A_BYTES, bL = bH + tc::B_BYTES;
                            const uint32_t acc_t = tmem + (uint32_t)(st * 64);
#pragma unroll
                            for (int kb = 0; kb < tc::KR / 8; ++kb)
                                tc::mma(acc_t, tc::desc(aH + kb * 2 * tc::LBO), tc::desc(bH + kb * 2 * tc::LBO), kb > 0);
#pragma unroll
                            for (int kb = 0; kb < tc::KR / 8; ++kb)
                                tc::mma(acc_t, tc::desc(aH + kb * 2 * tc::LBO), tc::desc(bL + kb * 2 * tc::LBO), 1);
#pragma unroll
                            for (int kb = 0; kb < tc::KR / 8; ++kb)
                                tc::mma(acc_t, tc::desc(aL + kb * 2 * tc::LBO), tc::desc(bH + kb * 2 * tc::LBO), 1);
                            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                                         ::"r"(st ? mb1 : mb0));
                        }
                    };
                    // wait for accumulator st, subtract it from the row's running values, release it
                    auto finish = [&](int st, uint32_t& ph, int& pend) {
                        const bool ok = tc::wait_phase(st ? mb1 : mb0, ph);
                        if (ok) {
                            ph ^= 1u;
                            pend = 0;
                        } else {
                            atomicOr(p.status, ST_TIMEOUT);
                            atomicOr(&bail_sh, 1);
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;");
                        if (ok) {
                            float v[64];
                            tc::ld64(tmem + my_lane + (uint32_t)(st * 64), v);
#pragma unroll
                            for (int cc = 0; cc < NB; ++cc)
                                acc[cc] = E::sub(acc[cc], make_float2(v[2 * cc], v[2 * cc + 1]));
                        }
                        // no barrier here: the next issue()'s barrier orders this read-back before
                        // the MMA that reuses accumulator st, and this thread has itself waited
                        // for the MMAs that read the stage it restages next
                    };
                    load(0, a0, b0r);
                    load(1, a1, b1r);                     // nch is even (>= 2)
                    stage(a0, b0r, 0);
                    issue(0);
                    pend0 = 1;
                    if (nch > 2) load(2, a0, b0r);
                    for (int c = 0; c < nch; c += 2) {
                        // chunk c+1 into stage 1 while the MMAs of chunk c run (stage 1 and its
                        // accumulator were released by finish(1) of the previous pair); the bail
                        // flag is read only right after a barrier, so every thread decides alike
                        stage(a1, b1r, 1);
                        issue(1);
                        pend1 = 1;
                        if (bail_sh) break;
                        if (c + 3 < nch) load(c + 3, a1, b1r);
                        finish(0, ph0, pend0);
                        if (c + 2 < nch) {
                            stage(a0, b0r, 0);
                            issue(0);
                            pend0 = 1;
                            if (bail_sh) break;
                            if (c + 4 < nch) load(c + 4, a0, b0r);
                        }
                        finish(1, ph1, pend1);
                    }
                    __syncthreads();                      // every read-back done; bail flag visible
                }
                if (bail_sh) break;
                if (b0 == 0) {
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) Dg[tid * (NB + 1) + c] = acc[c];
                    }
                    __syncthreads();
                    if (tid < 32) {
                        const int lane = tid;
                        T* myrow = Dg + lane * (NB + 1);
                        for (int kk = 0; kk < NB; ++kk) {
                            __syncwarp();
                            const T d = Dg[kk * (NB + 1) + kk];
                            const T dinv = E::inv(d);
                            const bool mine = lane > kk;
                            T l = E::zero();
                            if (mine) {
                                l = E::mul(myrow[kk], dinv);
                                myrow[kk] = l;
                            }
                            if (lane == kk) {
                                Dsh[kk] = d;
                                Dinv[kk] = dinv;
                                Dsq[kk] = E::csqrt(d);
                                const double m2 = (double)E::mag2(d);
                                if (!(m2 > 0.0) || !isfinite(m2)) atomicOr(p.status, ST_ZERO_PIVOT);
                            }
                            __syncwarp();
                            if (mine) {
                                const T ldv = E::mul(l, d);
                                for (int c = kk + 1; c <= lane; ++c)
                                    myrow[c] = E::fms(ldv, Dg[c * (NB + 1) + kk], myrow[c]);
                            }
                        }
                        __syncwarp();
                        for (int kk = 0; kk < NB; ++kk)
                            if (lane > kk) WL[kk * NB + lane] = E::mul(Dsh[kk], myrow[kk]);
                    }
                    __syncthreads();
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) acc[c] = Dg[tid * (NB + 1) + c];
                    }
                    __syncthreads();                      // Dg (stage 1) free for the next batch
                }
                if (active && ir >= NB) {
#pragma unroll
                    for (int kk = 0; kk < NB; ++kk) {
                        const T l = E::mul(acc[kk], Dinv[kk]);
#pragma unroll
                        for (int kk2 = kk + 1; kk2 < NB; ++kk2) acc[kk2] = E::fms(l, WL[kk * NB + kk2], acc[kk2]);
                        acc[kk] = l;
                    }
                    if (i >= np && qg) {
                        // the panel's NB terms of the quadratic form summed from zero, then added
                        T part = E::zero();
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) part = E::fma(E::mul(acc[kk], acc[kk]), Dsh[kk], part);
                        qg[i - np] = E::add(qg[i - np], part);
                    }
                    if (j0 + NB < np) {
                        T* gout = G + i + (long long)j0 * ld;
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) gout[(long long)kk * ld] = E::mul(acc[kk], Dsq[kk]);
                    }
                }
            }
            __syncthreads();
        }
        __syncthreads();
    }
    // MMAs still in flight after a timeout: bounded wait before the tensor memory is released
    if (pend0) (void)tc::wait_phase(mb0, ph0);
    if (pend1) (void)tc::wait_phase(mb1, ph1);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(tc::TMEM_COLS));
}

// ---------------------------------------------------------------------------
// Bulk-copy variant of the left-looking kernel (tile configuration 5).  The row operand
// (128 rows x KC columns of G) and the panel operand (NB rows x KC columns) of every chunk
// are brought into shared memory by the bulk-copy engine (cp.async.bulk, one contiguous
// copy per column, completion counted in bytes on an mbarrier), double-buffered, so that
// many kilobytes are in flight per CTA instead of two loads per thread.  The accumulators
// stay in registers (blocked: each chunk is summed from zero and subtracted).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint32_t a, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count));
}
__device__ __forceinline__ void mbar_expect(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}
// bounded wait; returns false if the phase did not complete
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t phase) {
    uint32_t done = 0;
    for (int spin = 0; spin < (1 << 24) && !done; ++spin)
        asm volatile("{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n"
                     "selp.u32 %0, 1, 0, q; }" : "=r"(done) : "r"(a), "r"(phase) : "memory");
    return done != 0;
}

template <class T, int NB, int KC>
__global__ void __launch_bounds__(128, 2) ldl_left_bulk_kernel(LdlParams<T> p) {
    using E = El<T>;
    using R = typename E::R;
    constexpr int NT = 128;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* As = reinterpret_cast<T*>(smem_raw);          // [2][KC][NT]: As[kk*NT + r] = G[i0 + r, k0 + kk]
    T* Bs = As + 2 * KC * NT;                        // [2][KC][NB]: Bs[kk*NB + c] = G[j0 + c, k0 + kk]
    T* Dg = Bs + 2 * KC * NB;                        // [32][NB+1]
    T* WL = Dg + 32 * (NB + 1);
    T* Dsh = WL + NB * NB;
    T* Dinv = Dsh + NB;
    T* Dsq = Dinv + NB;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int item_sh, bail_sh;
    const int tid = threadIdx.x;
    T* G = p.ws + (size_t)blockIdx.x * p.ws_stride;
    const uint32_t mb0 = (uint32_t)__cvta_generic_to_shared(&mbar[0]);
    const uint32_t mb1 = (uint32_t)__cvta_generic_to_shared(&mbar[1]);
    if (tid == 0) {
        mbar_init(mb0, 1);
        mbar_init(mb1, 1);
        bail_sh = 0;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    uint32_t ph0 = 0, ph1 = 0;

    for (;;) {
        if (tid == 0) item_sh = atomicAdd(p.counter, 1);
        __syncthreads();
        const int it = item_sh;
        if (it >= p.nitems || bail_sh) break;
        const int w = p.items[it].x, k = p.items[it].y;
        const int n = p.n_w[w];
        const int m = p.F ? p.m_w[w] : 0;
        const int np = (n + NB - 1) / NB * NB;
        const int rows = np + m;
        const long long ld = rows + (rows & 1);          // even: 16-byte aligned columns
        if (n > p.nmax || m > p.mmax) {
            if (tid == 0) atomicOr(p.status, ST_BAD_SHAPE);
            __syncthreads();
            continue;
        }
        const T z = p.shifts[k];
        const R* C = p.C ? p.C + p.offC[w] : nullptr;
        const R* B = p.B ? p.B + p.offC[w] : nullptr;
        const R* F = p.F ? p.F + p.offF[w] : nullptr;
        // quadratic forms accumulate in place in the output (any number of owned rows)
        T* const qg = p.q ? p.q + (long long)k * p.qstride + p.offQ[w] : nullptr;
        if (qg)
            for (int r = tid; r < m; r += NT) qg[r] = E::zero();
        __syncthreads();

        for (int j0 = 0; j0 < np && !bail_sh; j0 += NB) {
            const int na = rows - j0;
            for (int b0 = 0; b0 < na; b0 += NT) {
                const int ir = b0 + tid;
                const int i = j0 + ir;
                const int i0 = j0 + b0;                   // first row of the batch (even)
                const bool active = ir < na;
                const int nrow = min(NT, na - b0);
                const uint32_t abytes = (uint32_t)(((nrow + 1) & ~1) * sizeof(T));
                T acc[NB];
                if (active && i < n) {
                    const R* cp = C ? C + i + (long long)j0 * n : nullptr;
                    const R* bp = B ? B + i + (long long)j0 * n : nullptr;
#pragma unroll
                    for (int c = 0; c < NB; ++c) {
                        const int col = j0 + c;
                        T a = E::zero();
                        if (col <= i) {
                            const R bb = bp ? bp[(long long)c * n] : (i == col ? R(1) : R(0));
                            const R cc = cp ? cp[(long long)c * n] : R(0);
                            a = E::shift_minus(z, bb, cc);
                        }
                        acc[c] = a;
                    }
                } else if (active && i < np) {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c == i) ? E::from(R(1)) : E::zero();
                } else if (active) {
                    const R* fp = F + (i - np) + (long long)j0 * m;
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = (j0 + c < n) ? E::from(fp[(long long)c * m]) : E::zero();
                } else {
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = E::zero();
                }
                const int nch = (j0 + KC - 1) / KC;
                // issue chunk ci into buffer ci & 1 (one thread; one copy per column)
                auto issue = [&](int ci) {
                    const int k0 = ci * KC, kc = min(KC, j0 - k0);
                    const int buf = ci & 1;
                    const uint32_t mb = buf ? mb1 : mb0;
                    T* a_dst = As + buf * KC * NT;
                    T* b_dst = Bs + buf * KC * NB;
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_expect(mb, (uint32_t)kc * (abytes + NB * sizeof(T)));
                    for (int kk = 0; kk < kc; ++kk) {
                        const T* col = G + (long long)(k0 + kk) * ld;
                        bulk_g2s((uint32_t)__cvta_generic_to_shared(a_dst + kk * NT), col + i0, abytes, mb);
                        bulk_g2s((uint32_t)__cvta_generic_to_shared(b_dst + kk * NB), col + j0,
                                 NB * (uint32_t)sizeof(T), mb);
                    }
                };
                if (nch > 0) {
                    __syncthreads();                      // buffers free (previous users done)
                    if (tid == 0) issue(0);
                }
                for (int ci = 0; ci < nch; ++ci) {
                    const int k0 = ci * KC, kc = min(KC, j0 - k0);
                    if (tid == 0 && ci + 1 < nch) issue(ci + 1);
                    const int buf = ci & 1;
                    const bool ok = mbar_wait(buf ? mb1 : mb0, buf ? ph1 : ph0);
                    if (buf) ph1 ^= 1u; else ph0 ^= 1u;
                    if (!ok) {
                        atomicOr(p.status, ST_TIMEOUT);
                        atomicOr(&bail_sh, 1);
                    }
                    if (active && ok) {
                        const T* a = As + buf * KC * NT + tid;
                        const T* bb = Bs + buf * KC * NB;
                        T tmp[NB];
#pragma unroll
                        for (int c = 0; c < NB; ++c) tmp[c] = E::zero();
                        for (int kk = 0; kk < kc; kk += 2) {
                            const T g0 = a[kk * NT], g1 = a[(kk + 1) * NT];
                            const T* b = bb + kk * NB;
#pragma unroll
                            for (int c = 0; c < NB; ++c) {
                                T t = tmp[c];
                                t = E::fma(g0, b[c], t);
                                t = E::fma(g1, b[NB + c], t);
                                tmp[c] = t;
                            }
                        }
#pragma unroll
                        for (int c = 0; c < NB; ++c) acc[c] = E::sub(acc[c], tmp[c]);
                    }
                    __syncthreads();                      // buffer ci & 1 consumed by everyone
                    if (bail_sh) break;
                }
                if (bail_sh) break;
                if (b0 == 0) {
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) Dg[tid * (NB + 1) + c] = acc[c];
                    }
                    __syncthreads();
                    if (tid < 32) {
                        const int lane = tid;
                        T* myrow = Dg + lane * (NB + 1);
                        for (int kk = 0; kk < NB; ++kk) {
                            __syncwarp();
                            const T d = Dg[kk * (NB + 1) + kk];
                            const T dinv = E::inv(d);
                            const bool mine = lane > kk && lane < NB;
                            T l = E::zero();
                            if (mine) {
                                l = E::mul(myrow[kk], dinv);
                                myrow[kk] = l;
                            }
                            if (lane == kk) {
                                Dsh[kk] = d;
                                Dinv[kk] = dinv;
                                Dsq[kk] = E::csqrt(d);
                                const double m2 = (double)E::mag2(d);
                                if (!(m2 > 0.0) || !isfinite(m2)) atomicOr(p.status, ST_ZERO_PIVOT);
                            }
                            __syncwarp();
                            if (mine) {
                                const T ldv = E::mul(l, d);
                                for (int c = kk + 1; c <= lane; ++c)
                                    myrow[c] = E::fms(ldv, Dg[c * (NB + 1) + kk], myrow[c]);
                            }
                        }
                        __syncwarp();
                        for (int kk = 0; kk < NB; ++kk)
                            if (lane > kk && lane < NB) WL[kk * NB + lane] = E::mul(Dsh[kk], myrow[kk]);
                    }
                    __syncthreads();
                    if (tid < 32) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) acc[c] = Dg[tid * (NB + 1) + c];
                    }
                }
                if (active && ir >= NB) {
#pragma unroll
                    for (int kk = 0; kk < NB; ++kk) {
                        const T l = E::mul(acc[kk], Dinv[kk]);
#pragma unroll
                        for (int kk2 = kk + 1; kk2 < NB; ++kk2) acc[kk2] = E::fms(l, WL[kk * NB + kk2], acc[kk2]);
                        acc[kk] = l;
                    }
                    if (i >= np && qg) {
                        // the panel's NB terms of the quadratic form summed from zero, then added
                        // (blocked summation: one FP32 chain over all n terms loses ~10x accuracy)
                        T part = E::zero();
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) part = E::fma(E::mul(acc[kk], acc[kk]), Dsh[kk], part);
                        qg[i - np] = E::add(qg[i - np], part);
                    }
                    if (j0 + NB < np) {
                        T* gout = G + i + (long long)j0 * ld;
#pragma unroll
                        for (int kk = 0; kk < NB; ++kk) gout[(long long)kk * ld] = E::mul(acc[kk], Dsq[kk]);
                    }
                }
            }
            __syncthreads();                              // G columns of this panel complete
        }
        __syncthreads();
    }
}

template <class T, int NB, int KC>
static int launch_left_bulk(const LdlParams<T>& p, int grid, cudaStream_t s) {
    const size_t smem = sizeof(T) * ((size_t)2 * KC * 128 + 2 * KC * NB + 32 * (NB + 1) + NB * NB + 3 * NB);
    auto kern = ldl_left_bulk_kernel<T, NB, KC>;
    int per_sm = 0;
    if (int rc = prepare_kernel<ldl_left_bulk_kernel<T, NB, KC>>(128, smem, &per_sm)) return rc;
    grid = std::min(grid, std::max(1, per_sm) * device_sms());
    kern<<<grid, 128, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

static int launch_left_tc(const LdlParams<float2>& p, int grid, cudaStream_t s) {
    // two stages, then WL and the pivots (the diagonal block aliases stage 1)
    const size_t smem = 2 * (size_t)tc::STAGE_BYTES + sizeof(float2) * ((size_t)32 * 32 + 3 * 32);
    int per_sm = 0;
    if (int rc = prepare_kernel<ldl_left_tc_kernel>(128, smem, &per_sm)) return rc;
    // two CTAs per SM (2 x 105 KB shared memory, 2 x 30 K registers, 2 x 128 of the 512 TMEM
    // columns); the occupancy query reports one, but two run co-resident (measured: 185 -> 129 ms
    // per pass at 1024 electrons).  CTAs never wait on one another, so a CTA that finds no room
    // simply starts later and finds the queue empty.
    (void)per_sm;
    grid = std::min(grid, 2 * device_sms());
    ldl_left_tc_kernel<<<grid, 128, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

template <class T, int NB, int NT, int KC, bool SKIP = false>
static int launch_left_v(const LdlParams<T>& p, int grid, cudaStream_t s) {
    const size_t smem = sizeof(T) * ((size_t)2 * KC * NB + 32 * (NB + 1) + NB * NB + 3 * NB + (size_t)NB * NT);
    auto kern = ldl_left_kernel<T, NB, NT, KC, SKIP>;
    // persistent grid: as many CTAs as fit on the device, at most one workspace slot each
    int per_sm = 0;
    if (int rc = prepare_kernel<ldl_left_kernel<T, NB, NT, KC, SKIP>>(NT, smem, &per_sm)) return rc;
    grid = std::min(grid, std::max(1, per_sm) * device_sms());
    kern<<<grid, NT, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

template <class T, int NB, int NT, int KC>
static int launch_left(const LdlParams<T>& p, int grid, cudaStream_t s) {
    return p.c0 ? launch_left_v<T, NB, NT, KC, true>(p, grid, s) : launch_left_v<T, NB, NT, KC, false>(p, grid, s);
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

template <class T, int NB, int TR, int TC, int NT>
static int launch_ldl(const LdlParams<T>& p, int grid, cudaStream_t s) {
    const size_t smem = sizeof(T) * ((size_t)NB * p.ldp + NB * NB + 3 * NB + p.mmax);
    int per_sm = 0;
    if (int rc = prepare_kernel<ldl_aug_kernel<T, NB, TR, TC, NT>>(NT, smem, &per_sm)) return rc;
    ldl_aug_kernel<T, NB, TR, TC, NT><<<grid, NT, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

size_t ldl_smem_bytes(int elem_bytes, int nb, int ldp, int mmax) {
    return (size_t)elem_bytes * ((size_t)nb * ldp + nb * nb + 3 * nb + mmax);
}

// Chooses the widest panel that fits the shared-memory budget.
template <class T>
static int pick_nb(int ldp, int mmax, size_t budget) {
    for (int nb : {32, 16, 8})
        if (ldl_smem_bytes(sizeof(T), nb, ldp, mmax) <= budget) return nb;
    return 0;
}

template <class T>
static int dispatch(const LdlParams<T>& p, int grid, size_t budget, cudaStream_t s) {
    int nb = pick_nb<T>(p.ldp, p.mmax, budget);
    if constexpr (sizeof(T) == 16) nb = nb > 16 ? 16 : nb;     // complex double: register budget
    constexpr int NT = sizeof(T) == 8 && El<T>::complex ? 512 : 256;   // complex float: 16 warps
    constexpr int TC = 4;
    switch (nb) {
        case 32: return launch_ldl<T, 32, 4, TC, NT>(p, grid, s);
        case 16: return launch_ldl<T, 16, 4, TC, NT>(p, grid, s);
        case 8: return launch_ldl<T, 8, 4, TC, NT>(p, grid, s);
        default:
            lres_set_error("window too large for the shared-memory panel (ldp=%d, mmax=%d)", p.ldp, p.mmax);
            return LRES_EINVAL;
    }
}

int run_ldl(const LdlJob& j, cudaStream_t s) {
    const size_t budget = j.smem_budget;
    if (j.kind == LdlJob::C128) {
        LdlParams<double2> p{};
        p.nitems = j.nitems; p.items = j.items; p.counter = j.counter;
        p.n_w = j.n_w; p.m_w = j.m_w; p.offC = j.offC; p.offF = j.offF; p.offQ = j.offQ;
        p.C = (const double*)j.C; p.B = (const double*)j.B; p.F = (const double*)j.F;
        p.shifts = (const double2*)j.shifts; p.q = (double2*)j.q; p.qstride = j.qstride;
        p.mult = nullptr; p.npos = j.npos; p.status = j.status;
        p.ws = (double2*)j.ws; p.ws_stride = j.ws_stride; p.ldp = j.ldp; p.nmax = j.nmax; p.mmax = j.mmax;
        p.keep = j.keep;
        p.c0 = j.keep ? nullptr : j.c0;
        if (j.keep) return launch_left_v<double2, kKeepNB128, 256, 32, false>(p, j.grid, s);
        switch (j.config) {
            case 1: return launch_left<double2, 16, 128, 32>(p, j.grid, s);
            case 2: return launch_left<double2, 16, 256, 16>(p, j.grid, s);
            case 3: return launch_left<double2, 8, 256, 32>(p, j.grid, s);
            case 4: return launch_left<double2, 8, 128, 32>(p, j.grid, s);
            case 5: return launch_left_bulk<double2, 16, 16>(p, j.grid, s);
            default: return launch_left<double2, 16, 256, 32>(p, j.grid, s);
        }
    } else if (j.kind == LdlJob::C64) {
        LdlParams<float2> p{};
        p.nitems = j.nitems; p.items = j.items; p.counter = j.counter;
        p.n_w = j.n_w; p.m_w = j.m_w; p.offC = j.offC; p.offF = j.offF; p.offQ = j.offQ;
        p.C = (const float*)j.C; p.B = (const float*)j.B; p.F = (const float*)j.F;
        p.shifts = (const float2*)j.shifts; p.q = (float2*)j.q; p.qstride = j.qstride;
        p.mult = nullptr; p.npos = j.npos; p.status = j.status;
        p.ws = (float2*)j.ws; p.ws_stride = j.ws_stride; p.ldp = j.ldp; p.nmax = j.nmax; p.mmax = j.mmax;
        p.keep = j.keep;
        p.c0 = j.keep ? nullptr : j.c0;
        if (j.keep) return launch_left_v<float2, kKeepNB64, 256, 32, false>(p, j.grid, s);
        switch (j.config) {
            case 1: return launch_left<float2, 32, 128, 32>(p, j.grid, s);
            case 2: return launch_left<float2, 32, 256, 16>(p, j.grid, s);
            case 3: return launch_left<float2, 16, 256, 32>(p, j.grid, s);
            case 4: return launch_left_tc(p, j.grid, s);
            case 5: return launch_left_bulk<float2, 32, 32>(p, j.grid, s);
            default: return launch_left<float2, 32, 256, 32>(p, j.grid, s);
        }
    } else {
        LdlParams<double> p{};
        p.nitems = j.nitems; p.items = j.items; p.counter = j.counter;
        p.n_w = j.n_w; p.m_w = j.m_w; p.offC = j.offC; p.offF = j.offF; p.offQ = j.offQ;
        p.C = (const double*)j.C; p.B = (const double*)j.B; p.F = (const double*)j.F;
        p.shifts = (const double*)j.shifts; p.q = nullptr; p.qstride = 0;
        p.mult = j.mult; p.npos = j.npos; p.status = j.status;
        p.ws = (double*)j.ws; p.ws_stride = j.ws_stride; p.ldp = j.ldp; p.nmax = j.nmax; p.mmax = j.mmax;
        return dispatch(p, j.grid, budget, s);
    }
}

}  // namespace lres

// ---------------------------------------------------------------------------
// Window inertia counts with no device allocation.
//
// Some callers cannot allocate GPU memory on their own: hosts that hand out all device
// memory from their own arena or caching allocator and forbid foreign cudaMalloc, and
// latency-critical loops where the device-wide synchronisation of cudaMalloc/cudaFree
// is not acceptable.  lres_inertia_noalloc serves them: the caller passes device
// arrays for inputs and outputs, and the kernel's scratch (work queue, status word,
// shift, work items, per-CTA factorisation workspaces) lives in the file-scope array
// below, which every GPU that loads this library holds until the process exits.
// ---------------------------------------------------------------------------

namespace lres {
namespace {

constexpr int NOALLOC_MAX_N = 512;            // largest window dimension
constexpr int NOALLOC_MAX_WIN = 65536;        // most windows per call
constexpr int NOALLOC_SLOTS = 8;              // CTAs (one factorisation workspace each)
constexpr size_t NA_HDR = 256;                // counter, status, shift
constexpr size_t NA_ITEMS = sizeof(int2) * NOALLOC_MAX_WIN;
constexpr size_t NA_WS = sizeof(double) * (size_t)NOALLOC_MAX_N * NOALLOC_MAX_N * NOALLOC_SLOTS;
constexpr size_t NA_BYTES = NA_HDR + NA_ITEMS + NA_WS;   // 16.5 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

struct NoallocDevice {
    bool ready = false;
    unsigned char* base = nullptr;   // device address of g_noalloc_scratch on this device
    int smem_budget = 0;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[kMaxDevices];

__global__ void noalloc_init_kernel(unsigned char* base, int nwin, double sigma) {
    int* counter = reinterpret_cast<int*>(base);
    int* status = counter + 1;
    double* shift = reinterpret_cast<double*>(base + 8);
    int2* items = reinterpret_cast<int2*>(base + NA_HDR);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        *counter = 0;
        *status = 0;
        *shift = sigma;
    }
    for (int w = t; w < nwin; w += gridDim.x * blockDim.x) items[w] = make_int2(w, 0);
}

// Device address of the scratch array on the current device (set up on first use).
int noalloc_device(NoallocDevice** out) {
    int dev = 0;
    LRES_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        lres_set_error("device index %d outside the supported range 0..%d", dev, kMaxDevices - 1);
        return LRES_EINVAL;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) {
            lres_set_error("cudaGetSymbolAddress of the scratch array failed: %s", cudaGetErrorString(e));
            return LRES_ECUDA;
        }
        int optin = 0;
        LRES_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        d.base = static_cast<unsigned char*>(ptr);
        d.smem_budget = optin - 1024;
        d.ready = true;
    }
    *out = &d;
    return LRES_OK;
}

}  // namespace

}  // namespace lres

extern "C" int lres_inertia_noalloc(int32_t nwin, const int32_t* n_w, const int64_t* offC, const double* H,
                                    const double* S, double sigma, int32_t* below, int32_t nmax, void* stream) {
    using namespace lres;
    if (nwin <= 0 || !n_w || !offC || !H || !S || !below) {
        lres_set_error("lres_inertia_noalloc: null or empty argument");
        return LRES_EINVAL;
    }
    if (nwin > NOALLOC_MAX_WIN || nmax <= 0 || nmax > NOALLOC_MAX_N) {
        lres_set_error("lres_inertia_noalloc: %d windows of dimension up to %d exceed the limits "
                       "(%d windows, dimension %d)", nwin, nmax, NOALLOC_MAX_WIN, NOALLOC_MAX_N);
        return LRES_EINVAL;
    }
    if (!std::isfinite(sigma)) {
        lres_set_error("lres_inertia_noalloc: sigma must be finite");
        return LRES_EINVAL;
    }
    NoallocDevice* dv = nullptr;
    int rc = noalloc_device(&dv);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* base = dv->base;
    // counter, status, shift and the work items must start fresh on every call
    noalloc_init_kernel<<<(nwin + 255) / 256, 256, 0, s>>>(base, nwin, sigma);
    LRES_CUDA_TRY(cudaGetLastError());
    LdlParams<double> p{};
    p.nitems = nwin;
    p.items = reinterpret_cast<const int2*>(base + NA_HDR);
    p.counter = reinterpret_cast<int*>(base);
    p.status = reinterpret_cast<int*>(base) + 1;
    p.n_w = n_w;
    p.m_w = n_w;
    p.offC = reinterpret_cast<const long long*>(offC);
    p.offF = reinterpret_cast<const long long*>(offC);
    p.offQ = reinterpret_cast<const long long*>(offC);
    p.C = H;
    p.B = S;
    p.F = nullptr;
    p.shifts = reinterpret_cast<const double*>(base + 8);
    p.q = nullptr;
    p.mult = nullptr;
    p.npos = below;        // work item w is window w: positive pivots of (sigma S - H) = eigenvalues below sigma
    p.ws = reinterpret_cast<double*>(base + NA_HDR + NA_ITEMS);
    p.ws_stride = (long long)NOALLOC_MAX_N * NOALLOC_MAX_N;
    p.ldp = nmax;
    p.nmax = nmax;
    p.mmax = 0;
    rc = dispatch(p, NOALLOC_SLOTS, (size_t)dv->smem_budget, s);
    if (rc) return rc;
    int st = 0;
    LRES_CUDA_TRY(cudaMemcpyAsync(&st, p.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & ST_BAD_SHAPE) {
        lres_set_error("lres_inertia_noalloc: a window is larger than nmax = %d", nmax);
        return LRES_EINVAL;
    }
    if (st & ST_ZERO_PIVOT) {
        // a zero or non-finite pivot (NaN/Inf in H or S, or sigma on an eigenvalue): the
        // counts of that window are meaningless
        lres_set_error("lres_inertia_noalloc: zero or non-finite pivot in a window factorisation");
        return LRES_ENUMERIC;
    }
    return LRES_OK;
}

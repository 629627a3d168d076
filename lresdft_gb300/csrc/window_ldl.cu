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
#include "lres_internal.h"

namespace lres {

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
};

template <class T, int NB, int TR, int TC>
__global__ void __launch_bounds__(256) ldl_aug_kernel(LdlParams<T> p) {
    using E = El<T>;
    using R = typename E::R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* P = reinterpret_cast<T*>(smem_raw);          // NB x ldp panel, column kk at P + kk*ldp
    T* WL = P + (size_t)NB * p.ldp;                  // WL[kk*NB + kk2] = D_kk L_kk2,kk
    T* Dsh = WL + NB * NB;
    T* Dinv = Dsh + NB;
    T* qsh = Dinv + NB;                              // mmax
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

        // ---- build the augmented lower trapezoid
        const long long tot = (long long)rows * n;
        for (long long idx = tid; idx < tot; idx += blockDim.x) {
            const int i = (int)(idx % rows), j = (int)(idx / rows);
            T val;
            if (i < n) {
                if (i < j) continue;
                const R b = B ? B[i + (long long)j * n] : (i == j ? R(1) : R(0));
                const R c = C ? C[i + (long long)j * n] : R(0);
                val = E::shift_minus(z, b, c);
            } else {
                val = E::from(F[(i - n) + (long long)j * m]);
            }
            ws[i + (long long)j * ld] = val;
        }
        for (int r = tid; r < m; r += blockDim.x) qsh[r] = E::zero();
        if (tid == 0) npos_sh = 0;
        __syncthreads();

        for (int j0 = 0; j0 < n; j0 += NB) {
            const int nbj = min(NB, n - j0);
            const int prow = rows - j0;
            // ---- load panel columns [j0, j0+nbj), rows [j0, rows)
            for (int idx = tid; idx < nbj * prow; idx += blockDim.x) {
                const int i = idx % prow, kk = idx / prow;
                if (i >= kk) P[kk * ldp + i] = ws[(j0 + i) + (long long)(j0 + kk) * ld];
            }
            __syncthreads();

            // ---- (1) diagonal block, one warp, lane = row
            if (tid < 32) {
                const int lane = tid;
                for (int kk = 0; kk < nbj; ++kk) {
                    __syncwarp();
                    const T d = P[kk * ldp + kk];
                    const T dinv = E::inv(d);
                    T l = E::zero();
                    const bool mine = lane > kk && lane < nbj;
                    if (mine) l = E::mul(P[kk * ldp + lane], dinv);
                    __syncwarp();
                    if (mine) P[kk * ldp + lane] = l;
                    if (lane == kk) {
                        Dsh[kk] = d;
                        Dinv[kk] = dinv;
                        const double m2 = (double)E::mag2(d);
                        if (!(m2 > 0.0) || !isfinite(m2)) atomicOr(p.status, ST_ZERO_PIVOT);
                        if (E::re(d) > R(0)) ++npos_sh;
                    }
                    __syncwarp();
                    if (mine) {
                        const T ldv = E::mul(l, d);
                        for (int c = kk + 1; c <= lane; ++c)
                            P[c * ldp + lane] = E::fms(ldv, P[kk * ldp + c], P[c * ldp + lane]);
                    }
                }
                __syncwarp();
                for (int idx = lane; idx < nbj * nbj; idx += 32) {
                    const int kk = idx / nbj, kk2 = idx % nbj;
                    if (kk2 > kk) WL[kk * NB + kk2] = E::mul(Dsh[kk], P[kk * ldp + kk2]);
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
#pragma unroll
                for (int kk = 0; kk < NB; ++kk)
                    if (kk < nbj) P[kk * ldp + i] = a[kk];
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

            // ---- (3) trailing update of rows [r0, rows) x cols [r0, n), lower part
            const int r0 = j0 + nbj;
            if (r0 < n) {
                const int nr = rows - r0, nc = n - r0;
                const int nrt = (nr + TR - 1) / TR, nct = (nc + TC - 1) / TC;
                for (int t = tid; t < nrt * nct; t += blockDim.x) {
                    const int ti = t % nrt, tc = t / nrt;
                    const int i0 = r0 + ti * TR, c0 = r0 + tc * TC;
                    if (i0 + TR - 1 < c0) continue;          // tile strictly above the diagonal
                    T acc[TR][TC];
#pragma unroll
                    for (int u = 0; u < TR; ++u)
#pragma unroll
                        for (int v = 0; v < TC; ++v) acc[u][v] = E::zero();
                    for (int kk = 0; kk < nbj; ++kk) {
                        const T dk = Dsh[kk];
                        const T* Pk = P + kk * ldp - j0;
                        T wr[TR], lc[TC];
#pragma unroll
                        for (int u = 0; u < TR; ++u) wr[u] = (i0 + u < rows) ? Pk[i0 + u] : E::zero();
#pragma unroll
                        for (int v = 0; v < TC; ++v) lc[v] = (c0 + v < n) ? E::mul(Pk[c0 + v], dk) : E::zero();
#pragma unroll
                        for (int u = 0; u < TR; ++u)
#pragma unroll
                            for (int v = 0; v < TC; ++v) acc[u][v] = E::fma(wr[u], lc[v], acc[u][v]);
                    }
#pragma unroll
                    for (int v = 0; v < TC; ++v) {
                        const int c = c0 + v;
                        if (c >= n) continue;
#pragma unroll
                        for (int u = 0; u < TR; ++u) {
                            const int i = i0 + u;
                            if (i < rows && (i >= n || i >= c)) {
                                T* x = ws + i + (long long)c * ld;
                                *x = E::sub(*x, acc[u][v]);
                            }
                        }
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
// host launchers
// ---------------------------------------------------------------------------

template <class T, int NB, int TR, int TC>
static int launch_ldl(const LdlParams<T>& p, int grid, cudaStream_t s) {
    const size_t smem = sizeof(T) * ((size_t)NB * p.ldp + NB * NB + 2 * NB + p.mmax);
    auto kern = ldl_aug_kernel<T, NB, TR, TC>;
    LRES_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, 256, smem, s>>>(p);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

size_t ldl_smem_bytes(int elem_bytes, int nb, int ldp, int mmax) {
    return (size_t)elem_bytes * ((size_t)nb * ldp + nb * nb + 2 * nb + mmax);
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
    switch (nb) {
        case 32: return launch_ldl<T, 32, 4, 4>(p, grid, s);
        case 16: return launch_ldl<T, 16, 4, 4>(p, grid, s);
        case 8: return launch_ldl<T, 8, 4, 4>(p, grid, s);
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
        return dispatch(p, j.grid, budget, s);
    } else if (j.kind == LdlJob::C64) {
        LdlParams<float2> p{};
        p.nitems = j.nitems; p.items = j.items; p.counter = j.counter;
        p.n_w = j.n_w; p.m_w = j.m_w; p.offC = j.offC; p.offF = j.offF; p.offQ = j.offQ;
        p.C = (const float*)j.C; p.B = (const float*)j.B; p.F = (const float*)j.F;
        p.shifts = (const float2*)j.shifts; p.q = (float2*)j.q; p.qstride = j.qstride;
        p.mult = nullptr; p.npos = j.npos; p.status = j.status;
        p.ws = (float2*)j.ws; p.ws_stride = j.ws_stride; p.ldp = j.ldp; p.nmax = j.nmax; p.mmax = j.mmax;
        return dispatch(p, j.grid, budget, s);
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

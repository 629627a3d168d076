// Adjoint of the window solve: gradient of the band energy at fixed electron number with
// respect to the window matrices H_W, S_W and the grid potential v.
//
// For window B and upper-half-plane pole z_k the forward kernel (keep mode) leaves the
// complete factor of the augmented matrix [[A, F^T], [F, 0]], A = z_k S_W - H_W (or
// z_k I - H^_W in the standard form of the mixed path), A = G G^T, in one workspace slot:
// rows [0, np) hold G, rows [np, np + m) hold G21 = F G^-T.  Then
//
//   Z_k = A^-1 F^T = G^-T G21^T                       (adj_backsolve_kernel, in place)
//   A_c = Re sum_k c_k Z_k Z_k^T,  c in {w, w z, w z^2} (adj_accum_kernel)
//
// and with U_c = 4 dV <S_W, A_c> summed over windows (identity S in the standard form),
// N and E_band from the same pass, the fixed-N derivatives are
//
//   dN/dmu = N/(2R) - U_{w z'},  dE/dmu = E/R + N/2 - c N/(2R) - U_{w z z'},
//   z' = (1 + zeta)/2 written as real combinations of 1 and z,  kappa = dE/dmu / dN/dmu,
//   dE/dH_W = 4 dV (A_wz - kappa A_w),  dE/dS_W = -4 dV (A_wz2 - kappa A_wz).
//
// The mixed path maps these back with L^-T ( . ) L^-1.  dE/dv(r) = dV x_r^T (sum_B dE/dH_W) x_r
// over the atom pairs that share the point r (the adjoint of the H(v) assembly).
#include "common.cuh"
#include "lres_internal.h"

namespace lres {

// ---------------------------------------------------------------------------
// back-substitution  y G = g21  for every owned-point row (thread = row), blocks of NB
// columns from the last: the row's finished y entries stream from the slot, the G rows
// of the finished entries are staged in shared memory in chunks of KC, and every chunk's
// sum is formed from zero before it is subtracted (the forward kernel's rounding pattern).
// ---------------------------------------------------------------------------
template <class T, int NB, int NT, int KC>
__global__ void __launch_bounds__(NT) adj_backsolve_kernel(const int2* items, int nitems, const int* n_w,
                                                            const int* m_w, T* ws, long long ws_stride,
                                                            int* status) {
    using E = El<T>;
    __shared__ T Bs[KC * NB];               // Bs[kk*NB + c] = G[i0 + kk, j0 + c]
    __shared__ T Dblk[NB * (NB + 1)];       // Dblk[c*(NB+1) + c2] = G[j0 + c, j0 + c2], c2 <= c
    __shared__ T Dinv[NB];
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const int w = items[it].x;
    const int n = n_w[w], m = m_w[w];
    const int np = (n + NB - 1) / NB * NB;
    const long long ld = np + m;
    T* G = ws + (size_t)it * ws_stride;
    const int tid = threadIdx.x;
    for (int b0 = 0; b0 < m; b0 += NT) {
        const int r = b0 + tid;
        const bool active = r < m;
        T* yrow = G + np + r;                // y_i of this row at yrow[i*ld] (in place of g21)
        for (int j0 = np - NB; j0 >= 0; j0 -= NB) {
            T acc[NB];
#pragma unroll
            for (int c = 0; c < NB; ++c) acc[c] = active ? yrow[(long long)(j0 + c) * ld] : E::zero();
            for (int i0 = j0 + NB; i0 < np; i0 += KC) {
                const int kc = min(KC, np - i0);
                __syncthreads();
                for (int idx = tid; idx < kc * NB; idx += NT) {
                    const int c = idx / kc, kk = idx % kc;   // column segments are contiguous
                    Bs[kk * NB + c] = G[(i0 + kk) + (long long)(j0 + c) * ld];
                }
                __syncthreads();
                if (active) {
                    T tmp[NB];
#pragma unroll
                    for (int c = 0; c < NB; ++c) tmp[c] = E::zero();
                    for (int kk = 0; kk < kc; ++kk) {
                        const T y = yrow[(long long)(i0 + kk) * ld];
#pragma unroll
                        for (int c = 0; c < NB; ++c) tmp[c] = E::fma(y, Bs[kk * NB + c], tmp[c]);
                    }
#pragma unroll
                    for (int c = 0; c < NB; ++c) acc[c] = E::sub(acc[c], tmp[c]);
                }
            }
            __syncthreads();
            for (int idx = tid; idx < NB * NB; idx += NT) {
                const int c2 = idx / NB, c = idx % NB;       // column c2, row c
                if (c2 <= c) Dblk[c * (NB + 1) + c2] = G[(j0 + c) + (long long)(j0 + c2) * ld];
            }
            __syncthreads();
            if (tid < NB) {
                const T d = Dblk[tid * (NB + 1) + tid];
                const double m2 = (double)E::mag2(d);
                if (!(m2 > 0.0) || !isfinite(m2)) atomicOr(status, ST_ZERO_PIVOT);
                Dinv[tid] = E::inv(d);
            }
            __syncthreads();
            if (active) {
#pragma unroll
                for (int c = NB - 1; c >= 0; --c) {
                    const T y = E::mul(acc[c], Dinv[c]);
                    acc[c] = y;
#pragma unroll
                    for (int c2 = 0; c2 < c; ++c2) acc[c2] = E::fms(y, Dblk[c * (NB + 1) + c2], acc[c2]);
                }
#pragma unroll
                for (int c = 0; c < NB; ++c) yrow[(long long)(j0 + c) * ld] = acc[c];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// A_c[a, b] = Re sum_k c_k sum_r Z_k[a, r] Z_k[b, r]  for one 32 x 32 tile (a-block I >=
// b-block J) of one window; 16 x 16 threads with 2 x 2 outputs each.  Per pole the r sum is
// taken in chunks of 32 in the working precision, each chunk added in FP64.
// ---------------------------------------------------------------------------
template <class T, int NBF>
__global__ void __launch_bounds__(256) adj_accum_kernel(const int* wins, int P, const int* n_w, const int* m_w,
                                                         const long long* offC, const T* ws, long long ws_stride,
                                                         const double2* cw, double* A0, double* A1, double* A2) {
    using E = El<T>;
    __shared__ T Ya[32][33];
    __shared__ T Yb[32][33];
    const int bw = blockIdx.y;
    const int w = wins[bw];
    const int n = n_w[w], m = m_w[w];
    const int t = blockIdx.x;
    int I = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((I + 1) * (I + 2) / 2 <= t) ++I;
    while (I * (I + 1) / 2 > t) --I;
    const int J = t - I * (I + 1) / 2;
    if (I * 32 >= n) return;
    const int np = (n + NBF - 1) / NBF * NBF;
    const long long ld = np + m;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    double acc[3][2][2] = {};
    for (int k = 0; k < P; ++k) {
        const T* Y = ws + (size_t)(bw * P + k) * ws_stride + np;    // Z_k[a, r] at Y[r + a*ld]
        double ud[2][2][2] = {};
        for (int r0 = 0; r0 < m; r0 += 32) {
            const int rc = min(32, m - r0);
            __syncthreads();
            for (int idx = tid; idx < 32 * 32; idx += 256) {
                const int ii = idx / 32, rr = idx % 32;
                const int a = I * 32 + ii, b = J * 32 + ii;
                Ya[rr][ii] = (rr < rc && a < n) ? Y[(r0 + rr) + (long long)a * ld] : E::zero();
                Yb[rr][ii] = (rr < rc && b < n) ? Y[(r0 + rr) + (long long)b * ld] : E::zero();
            }
            __syncthreads();
            T tmp[2][2];
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int v = 0; v < 2; ++v) tmp[u][v] = E::zero();
            for (int rr = 0; rr < rc; ++rr) {
                const T a0 = Ya[rr][tx], a1 = Ya[rr][tx + 16];
                const T b0 = Yb[rr][ty], b1 = Yb[rr][ty + 16];
                tmp[0][0] = E::fma(a0, b0, tmp[0][0]);
                tmp[0][1] = E::fma(a0, b1, tmp[0][1]);
                tmp[1][0] = E::fma(a1, b0, tmp[1][0]);
                tmp[1][1] = E::fma(a1, b1, tmp[1][1]);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int v = 0; v < 2; ++v) {
                    ud[u][v][0] += (double)tmp[u][v].x;
                    ud[u][v][1] += (double)tmp[u][v].y;
                }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double2 cc = cw[c * P + k];
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int v = 0; v < 2; ++v) acc[c][u][v] += cc.x * ud[u][v][0] - cc.y * ud[u][v][1];
        }
    }
    double* outs[3] = {A0, A1, A2};
    const long long o = offC[w];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            const int a = I * 32 + tx + 16 * u, b = J * 32 + ty + 16 * v;
            if (a >= n || b >= n) continue;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                outs[c][o + a + (long long)b * n] = acc[c][u][v];
                if (I != J) outs[c][o + b + (long long)a * n] = acc[c][u][v];
            }
        }
}

// Pole weights of the three accumulations: c_0 = w_k, c_1 = w_k z_k, c_2 = w_k z_k^2,
// nodes as the forward pass computes them (lrft/core.py:130-139).
__global__ void adj_weights_kernel(int P, int M, double mu, double e_lo, double2* cw) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    const double cc = 0.5 * (mu + e_lo), R = 0.5 * (mu - e_lo);
    double sn, cs;
    sincospi((double)(2 * k + 1) / (double)M, &sn, &cs);
    const double zr = cc + R * cs, zi = R * sn;
    const double wr = R * cs / M, wi = R * sn / M;
    const double w1r = wr * zr - wi * zi, w1i = wr * zi + wi * zr;
    cw[k] = make_double2(wr, wi);
    cw[P + k] = make_double2(w1r, w1i);
    cw[2 * P + k] = make_double2(w1r * zr - w1i * zi, w1r * zi + w1i * zr);
}

// u[c*nwin + w] = <S_W, A_c> (S given) or tr(A_c) (S null), fixed-order reduction.
__global__ void __launch_bounds__(256) adj_inner_kernel(int nwin, const int* n_w, const long long* offC,
                                                         const double* S, const double* A0, const double* A1,
                                                         const double* A2, double* u) {
    const int w = blockIdx.x;
    if (w >= nwin) return;
    const int n = n_w[w];
    const long long o = offC[w];
    const long long cnt = S ? (long long)n * n : n;
    double s[3] = {0.0, 0.0, 0.0};
    for (long long i = threadIdx.x; i < cnt; i += 256) {
        const long long e = S ? o + i : o + i + i * n;
        const double f = S ? S[e] : 1.0;
        s[0] = fma(f, A0[e], s[0]);
        s[1] = fma(f, A1[e], s[1]);
        s[2] = fma(f, A2[e], s[2]);
    }
    __shared__ double red[3][256];
    for (int c = 0; c < 3; ++c) red[c][threadIdx.x] = s[c];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int c = 0; c < 3; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 3) u[threadIdx.x * nwin + w] = red[threadIdx.x][0];
}

// X = a (A1 - kappa A0), Y = b (A2 - kappa A1), elementwise.
__global__ void adj_combine_kernel(long long nval, const double* A0, const double* A1, const double* A2,
                                   double kappa, double a, double b, double* X, double* Y) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nval) return;
    const double x = a * (A1[i] - kappa * A0[i]);
    const double y = b * (A2[i] - kappa * A1[i]);
    X[i] = x;
    Y[i] = y;
}

// Global gradient blocks: gH[block (g,h)] = sum over the windows holding g and h of their
// dE/dH_W block, windows in ascending order (one warp per block).
__global__ void __launch_bounds__(256) adj_block_gather_kernel(int nblk, const int* brow, const int* bcol,
                                                                const int* gptr, const long long* boff,
                                                                const long long* eoff, const int4* ent,
                                                                const int* n_w, const long long* offC,
                                                                const double* dHW, double* gH) {
    const int b = blockIdx.x * 8 + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (b >= nblk) return;
    const int g = brow[b], h = bcol[b];
    const int nfg = gptr[g + 1] - gptr[g], nfh = gptr[h + 1] - gptr[h];
    const int nv = nfg * nfh;
    for (int vi = lane; vi < nv; vi += 32) {
        const int a = vi / nfh, c = vi % nfh;
        double s = 0.0;
        for (long long e = eoff[b]; e < eoff[b + 1]; ++e) {
            const int4 t = ent[e];             // (window, local offset of g, local offset of h)
            s += dHW[offC[t.x] + (t.y + a) + (long long)(t.z + c) * n_w[t.x]];
        }
        gH[boff[b] + vi] = s;
    }
}

// dE/dv(r) = dV sum_{g,h covering r} x_g(r)^T gH_gh x_h(r) (thread = grid point).
__global__ void __launch_bounds__(256) adj_point_kernel(long long ng, const long long* poff, const int2* pent,
                                                         const double* sval, const int* gptr, const int* bptr,
                                                         const int* bcol, const long long* boff,
                                                         const double* gH, double dV, double* dv) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= ng) return;
    const long long e0 = poff[r], e1 = poff[r + 1];
    double s = 0.0;
    for (long long e = e0; e < e1; ++e) {
        const int2 gs = pent[e];
        const int g = gs.x;
        const int nfg = gptr[g + 1] - gptr[g];
        const double* xg = sval + (size_t)gs.y * 8;
        const int b0 = bptr[g], b1 = bptr[g + 1];
        for (long long f = e0; f < e1; ++f) {
            const int2 hs = pent[f];
            const int h = hs.x;
            int lo = b0, hi = b1;              // block (g, h) in the sorted block row g
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (bcol[mid] < h) lo = mid + 1;
                else hi = mid;
            }
            if (lo >= b1 || bcol[lo] != h) continue;
            const int nfh = gptr[h + 1] - gptr[h];
            const double* xh = sval + (size_t)hs.y * 8;
            const double* blk = gH + boff[lo];
            for (int a = 0; a < nfg; ++a) {
                double t = 0.0;
                for (int c = 0; c < nfh; ++c) t = fma(blk[a * nfh + c], xh[c], t);
                s = fma(xg[a], t, s);
            }
        }
    }
    dv[r] = dV * s;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int adj_backsolve(bool fp32, const int2* items, int nitems, const int* n_w, const int* m_w, void* ws,
                  long long ws_stride, int* status, cudaStream_t s) {
    if (!nitems) return LRES_OK;
    if (fp32)
        adj_backsolve_kernel<float2, kKeepNB64, 128, 32><<<nitems, 128, 0, s>>>(items, nitems, n_w, m_w,
                                                                                (float2*)ws, ws_stride, status);
    else
        adj_backsolve_kernel<double2, kKeepNB128, 128, 32><<<nitems, 128, 0, s>>>(items, nitems, n_w, m_w,
                                                                                  (double2*)ws, ws_stride, status);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int adj_accumulate(bool fp32, const int* wins, int nwin_batch, int P, int nmax, const int* n_w, const int* m_w,
                   const long long* offC, const void* ws, long long ws_stride, const double2* cw, double* A0,
                   double* A1, double* A2, cudaStream_t s) {
    if (!nwin_batch) return LRES_OK;
    const int T = (nmax + 31) / 32;
    dim3 grid(T * (T + 1) / 2, nwin_batch);
    if (fp32)
        adj_accum_kernel<float2, kKeepNB64><<<grid, 256, 0, s>>>(wins, P, n_w, m_w, offC, (const float2*)ws,
                                                                 ws_stride, cw, A0, A1, A2);
    else
        adj_accum_kernel<double2, kKeepNB128><<<grid, 256, 0, s>>>(wins, P, n_w, m_w, offC, (const double2*)ws,
                                                                   ws_stride, cw, A0, A1, A2);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int adj_weights(int P, int M, double mu, double e_lo, double2* cw, cudaStream_t s) {
    adj_weights_kernel<<<(P + 63) / 64, 64, 0, s>>>(P, M, mu, e_lo, cw);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int adj_inner(int nwin, const int* n_w, const long long* offC, const double* S, const double* A0, const double* A1,
              const double* A2, double* u, cudaStream_t s) {
    adj_inner_kernel<<<nwin, 256, 0, s>>>(nwin, n_w, offC, S, A0, A1, A2, u);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int adj_combine(long long nval, const double* A0, const double* A1, const double* A2, double kappa, double a,
                double b, double* X, double* Y, cudaStream_t s) {
    adj_combine_kernel<<<(unsigned)((nval + 255) / 256), 256, 0, s>>>(nval, A0, A1, A2, kappa, a, b, X, Y);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int adj_block_gather(const BlockPattern& bp, const long long* eoff, const int4* ent, const int* n_w,
                     const long long* offC, const double* dHW, double* gH, cudaStream_t s) {
    adj_block_gather_kernel<<<(bp.nblk + 7) / 8, 256, 0, s>>>(bp.nblk, bp.brow, bp.bcol, bp.gptr, bp.boff, eoff,
                                                              ent, n_w, offC, dHW, gH);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int adj_point(long long ng, const long long* poff, const int2* pent, const Supports& sp, const BlockPattern& bp,
              const double* gH, double dV, double* dv, cudaStream_t s) {
    adj_point_kernel<<<(unsigned)((ng + 255) / 256), 256, 0, s>>>(ng, poff, pent, sp.sval, bp.gptr, bp.bptr,
                                                                   bp.bcol, bp.boff, gH, dV, dv);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

}  // namespace lres

// Atom-pair assembly of H(v) = T + X^T diag(v) X dV, gathers of the dense window
// blocks, the owned-point basis blocks F_W, a batched FP64 GEMM for the standard-form
// transform, and the pole-weighted reductions to density / electron count / band
// energy.  All bandwidth-bound except the GEMM.
//
// H(v) (lrft/lcao3d.py:98-100): functions of one atom share one support, so
// H_gh = T_gh + dV sum_{r in supp g and supp h} v_r x_g(r) x_h(r)^T over the common
// grid points of each overlapping atom pair, listed once per geometry.  Algorithmic
// bytes per assembly: per common point 8 B slot pair + 8 B v + 2 x 8 x 8 B basis
// values, plus the T and H blocks (8 B per stored value, read + write).
#include "common.cuh"
#include "lres_internal.h"

#include <algorithm>
#include <numeric>
#include <type_traits>

namespace lres {

// ---------------------------------------------------------------------------
// common points of overlapping atom pairs
// ---------------------------------------------------------------------------

__device__ __forceinline__ long long lower_bound_int(const int* a, long long lo, long long hi, int key) {
    while (lo < hi) {
        long long mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void pair_count_kernel(int npair, const int* pg, const int* ph, const long long* soff, const int* sgrid,
                                  long long* counts) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= npair) return;
    const int g = pg[warp], h = ph[warp];
    const long long g0 = soff[g], g1 = soff[g + 1], h0 = soff[h], h1 = soff[h + 1];
    long long c = 0;
    for (long long s = g0 + lane; s < g1; s += 32) {
        const int key = sgrid[s];
        const long long pos = lower_bound_int(sgrid, h0, h1, key);
        c += (pos < h1 && sgrid[pos] == key);
    }
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) counts[warp] = c;
}

__global__ void pair_fill_kernel(int npair, const int* pg, const int* ph, const long long* soff, const int* sgrid,
                                 const long long* coff, int2* cslot) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= npair) return;
    const int g = pg[warp], h = ph[warp];
    const long long g0 = soff[g], g1 = soff[g + 1], h0 = soff[h], h1 = soff[h + 1];
    long long out = coff[warp];
    for (long long base = g0; base < g1; base += 32) {
        const long long s = base + lane;
        bool hit = false;
        long long pos = 0;
        if (s < g1) {
            const int key = sgrid[s];
            pos = lower_bound_int(sgrid, h0, h1, key);
            hit = pos < h1 && sgrid[pos] == key;
        }
        const unsigned mask = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int before = __popc(mask & ((1u << lane) - 1u));
            cslot[out + before] = make_int2((int)(s - g0), (int)(pos - h0));
        }
        out += __popc(mask);
    }
}

int pair_common_points(const BlockPattern& bp, Supports& sp, int ngroups, const std::vector<int>& pair_g,
                       const std::vector<int>& pair_h, cudaStream_t s) {
    const int npair = (int)pair_g.size();
    int *dg = nullptr, *dh = nullptr;
    long long* dcount = nullptr;
    LRES_CUDA_TRY(cudaMalloc(&dg, sizeof(int) * std::max(npair, 1)));
    LRES_CUDA_TRY(cudaMalloc(&dh, sizeof(int) * std::max(npair, 1)));
    LRES_CUDA_TRY(cudaMalloc(&dcount, sizeof(long long) * std::max(npair, 1)));
    LRES_CUDA_TRY(cudaMemcpyAsync(dg, pair_g.data(), sizeof(int) * npair, cudaMemcpyHostToDevice, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(dh, pair_h.data(), sizeof(int) * npair, cudaMemcpyHostToDevice, s));
    const int threads = 256, blocks = (int)(((long long)npair * 32 + threads - 1) / threads);
    if (npair) pair_count_kernel<<<blocks, threads, 0, s>>>(npair, dg, dh, sp.soff, sp.sgrid, dcount);
    LRES_CUDA_TRY(cudaGetLastError());
    std::vector<long long> counts(npair), off(npair + 1, 0);
    LRES_CUDA_TRY(cudaMemcpyAsync(counts.data(), dcount, sizeof(long long) * npair, cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    for (int p = 0; p < npair; ++p) off[p + 1] = off[p] + counts[p];
    sp.ncommon = off[npair];
    LRES_CUDA_TRY(cudaMalloc(&sp.coff, sizeof(long long) * (npair + 1)));
    LRES_CUDA_TRY(cudaMalloc(&sp.cslot, sizeof(int2) * std::max<long long>(sp.ncommon, 1)));
    LRES_CUDA_TRY(cudaMemcpyAsync(sp.coff, off.data(), sizeof(long long) * (npair + 1), cudaMemcpyHostToDevice, s));
    if (npair) pair_fill_kernel<<<blocks, threads, 0, s>>>(npair, dg, dh, sp.soff, sp.sgrid, sp.coff, sp.cslot);
    LRES_CUDA_TRY(cudaGetLastError());
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(dg);
    cudaFree(dh);
    cudaFree(dcount);
    (void)bp;
    (void)ngroups;
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// H(v) assembly: one warp per overlapping pair (g <= h)
// ---------------------------------------------------------------------------

template <int NF>
__global__ void __launch_bounds__(256) assemble_h_kernel(int npair, const int* pair_blk, const int* brow,
                                                         const int* bcol, const long long* boff, const int* btrans,
                                                         const int* gptr, const long long* soff, const int* sgrid,
                                                         const double* sval, const long long* coff,
                                                         const int2* cslot, const double* Tblk, const double* v,
                                                         double dV, double* Hblk) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= npair) return;
    const int b = pair_blk[warp];
    const int g = brow[b], h = bcol[b];
    const int nfg = gptr[g + 1] - gptr[g], nfh = gptr[h + 1] - gptr[h];
    const long long sg0 = soff[g], sh0 = soff[h];
    double acc[NF][NF];
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int e = 0; e < NF; ++e) acc[f][e] = 0.0;
    const long long c1 = coff[warp + 1];
    for (long long c = coff[warp] + lane; c < c1; c += 32) {
        const int2 ss = cslot[c];
        const long long a = sg0 + ss.x, bb = sh0 + ss.y;
        const double vv = v[sgrid[a]];
        double xg[NF], xh[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            xg[f] = sval[a * 8 + f];
            xh[f] = sval[bb * 8 + f] * vv;
        }
#pragma unroll
        for (int f = 0; f < NF; ++f)
#pragma unroll
            for (int e = 0; e < NF; ++e) acc[f][e] = fma(xg[f], xh[e], acc[f][e]);
    }
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int e = 0; e < NF; ++e) {
            double x = acc[f][e];
            for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            acc[f][e] = x;
        }
    const long long o = boff[b];
    const long long ot = boff[btrans[b]];
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int e = 0; e < NF; ++e) {
            if ((f * NF + e) % 32 != lane || f >= nfg || e >= nfh) continue;
            const double val = Tblk[o + f * nfh + e] + acc[f][e] * dV;
            Hblk[o + f * nfh + e] = val;
            if (h != g) Hblk[ot + e * nfg + f] = Tblk[ot + e * nfg + f] + acc[f][e] * dV;
        }
}

int assemble_h(const BlockPattern& bp, const Supports& sp, const double* Tblk, const double* v, double dV,
               double* Hblk, cudaStream_t s) {
    const int threads = 256;
    const int blocks = (int)(((long long)bp.npair * 32 + threads - 1) / threads);
    if (!bp.npair) return LRES_OK;
    if (bp.nfmax <= 6)
        assemble_h_kernel<6><<<blocks, threads, 0, s>>>(bp.npair, bp.pair_blk, bp.brow, bp.bcol, bp.boff, bp.btrans,
                                                        bp.gptr, sp.soff, sp.sgrid, sp.sval, sp.coff, sp.cslot, Tblk,
                                                        v, dV, Hblk);
    else
        assemble_h_kernel<8><<<blocks, threads, 0, s>>>(bp.npair, bp.pair_blk, bp.brow, bp.bcol, bp.boff, bp.btrans,
                                                        bp.gptr, sp.soff, sp.sgrid, sp.sval, sp.coff, sp.cslot, Tblk,
                                                        v, dV, Hblk);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// H(v) assembly for the mixed precision: FP32 products summed in FP32 over blocks of 32
// common points per lane, the block sums accumulated as unevaluated FP32 pairs (hi + lo,
// Knuth's TwoSum), the lanes' pairs reduced the same way and converted to FP64 once per
// element.  The unblocked FP32 sum drifts (~1e-6 Ha per window in the band energy, one
// sign); the blocked one is as accurate as the FP64 assembly ahead of the FP32 window
// reduction.  No FP64 arithmetic per point (GB300's FP64 rate is 1/64 of FP32).
// ---------------------------------------------------------------------------

// v at every support slot, FP32 (the FP32 kernel reads it next to the basis values)
__global__ void slot_potential_kernel(long long nslot, const int* sgrid, const double* v, float* vslot) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a < nslot) vslot[a] = (float)v[sgrid[a]];
}

template <int NF>
__device__ __forceinline__ void load_slot(const float* p, float (&x)[NF]) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
    if constexpr (NF > 4) {
        const float4 b = *reinterpret_cast<const float4*>(p + 4);
        const float t[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int f = 4; f < NF; ++f) x[f] = t[f - 4];
    }
}

constexpr int kAsmBlock = 32;                   // common points per lane and FP32 block

constexpr int kAsmThreads = 128;

// (hi, lo) <- (hi, lo) + x with the rounding error of hi + x kept in lo (Knuth's TwoSum).
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += err;
}

// One warp per pair; the pair sums of each lane live in shared memory ([element][thread],
// conflict-free), which keeps the kernel below 100 registers.
template <int NF>
__global__ void __launch_bounds__(kAsmThreads, 5) assemble_h32_kernel(int npair, const int* pair_blk, const int* brow,
                                                                      const int* bcol, const long long* boff,
                                                                      const int* btrans, const int* gptr,
                                                                      const long long* soff, const float* sval32,
                                                                      const float* vslot, const long long* coff,
                                                                      const int2* cslot, const double* Tblk,
                                                                      double dV, double* Hblk) {
    __shared__ float2 acc_s[NF * NF][kAsmThreads];
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, t = threadIdx.x;
    if (warp >= npair) return;
    const int b = pair_blk[warp];
    const int g = brow[b], h = bcol[b];
    const int nfg = gptr[g + 1] - gptr[g], nfh = gptr[h + 1] - gptr[h];
    const long long sg0 = soff[g], sh0 = soff[h];
#pragma unroll
    for (int k = 0; k < NF * NF; ++k) acc_s[k][t] = make_float2(0.0f, 0.0f);
    const long long c0 = coff[warp], c1 = coff[warp + 1];
    for (long long base = c0; base < c1; base += 32 * kAsmBlock) {
        const long long cend = min(c1, base + 32 * kAsmBlock);
        float blk[NF][NF];
#pragma unroll
        for (int f = 0; f < NF; ++f)
#pragma unroll
            for (int e = 0; e < NF; ++e) blk[f][e] = 0.0f;
#pragma unroll 2
        for (long long c = base + lane; c < cend; c += 32) {
            const int2 ss = cslot[c];
            const long long a = sg0 + ss.x, bb = sh0 + ss.y;
            const float vv = vslot[a];
            float xg[NF], xh[NF];
            load_slot<NF>(sval32 + a * 8, xg);
            load_slot<NF>(sval32 + bb * 8, xh);
#pragma unroll
            for (int e = 0; e < NF; ++e) xh[e] *= vv;
#pragma unroll
            for (int f = 0; f < NF; ++f)
#pragma unroll
                for (int e = 0; e < NF; ++e) blk[f][e] = fmaf(xg[f], xh[e], blk[f][e]);
        }
        // one row at a time (the compiler would otherwise hoist all 36 loads)
#pragma unroll
        for (int f = 0; f < NF; ++f) {
#pragma unroll
            for (int e = 0; e < NF; ++e) {
                float2 a = acc_s[f * NF + e][t];
                two_sum_acc(a.x, a.y, blk[f][e]);
                acc_s[f * NF + e][t] = a;
            }
            asm volatile("" ::: "memory");
        }
    }
    // the lanes' pairs of element k reduced by a butterfly; lane k % 32 keeps the result, and
    // every lane then converts and stores its own elements (the FP64 instructions are issued
    // once or twice per warp, all lanes busy, rather than once per element)
    constexpr int kPer = (NF * NF + 31) / 32;
    float2 mine[kPer];
#pragma unroll
    for (int m = 0; m < kPer; ++m) mine[m] = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < NF * NF; ++k) {
        float2 a = acc_s[k][t];
#pragma unroll 1
        for (int s = 16; s; s >>= 1) {
            const float ohi = __shfl_xor_sync(0xffffffffu, a.x, s);
            const float olo = __shfl_xor_sync(0xffffffffu, a.y, s);
            // the same pair of operands in the same order on both lanes of a butterfly
            float hi = lane & s ? ohi : a.x, lo = lane & s ? olo : a.y;
            const float x = lane & s ? a.x : ohi, xlo = lane & s ? a.y : olo;
            two_sum_acc(hi, lo, x);
            a = make_float2(hi, lo + xlo);
        }
        if (k % 32 == lane) mine[k / 32] = a;
    }
    const long long o = boff[b];
    const long long ot = boff[btrans[b]];
#pragma unroll
    for (int m = 0; m < kPer; ++m) {
        const int k = lane + 32 * m;
        if (k >= NF * NF) break;
        const int f = k / NF, e = k % NF;
        if (f >= nfg || e >= nfh) continue;
        const double x = (double)mine[m].x + (double)mine[m].y;
        Hblk[o + f * nfh + e] = Tblk[o + f * nfh + e] + x * dV;
        if (h != g) Hblk[ot + e * nfg + f] = Tblk[ot + e * nfg + f] + x * dV;
    }
}

bool assemble_h32_supported(const BlockPattern& bp) { return bp.nfmax <= 6; }

int assemble_h32(const BlockPattern& bp, const Supports& sp, const double* Tblk, const double* v, double dV,
                 double* Hblk, cudaStream_t s) {
    if (!sp.sval32 || !sp.vslot || bp.nfmax > 6) {
        lres_set_error("FP32 H(v) assembly needs the FP32 basis values and at most 6 functions per atom");
        return LRES_ESTATE;
    }
    if (!bp.npair) return LRES_OK;
    if (sp.nslot)
        slot_potential_kernel<<<(unsigned)((sp.nslot + 255) / 256), 256, 0, s>>>(sp.nslot, sp.sgrid, v, sp.vslot);
    LRES_CUDA_TRY(cudaGetLastError());
    const int threads = kAsmThreads;
    const int blocks = (int)(((long long)bp.npair * 32 + threads - 1) / threads);
    assemble_h32_kernel<6><<<blocks, threads, 0, s>>>(bp.npair, bp.pair_blk, bp.brow, bp.bcol, bp.boff, bp.btrans,
                                                      bp.gptr, sp.soff, sp.sval32, sp.vslot, sp.coff, sp.cslot, Tblk,
                                                      dV, Hblk);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// dense window blocks from the block-sparse storage
// ---------------------------------------------------------------------------

// Every element of every dense window block, column-major, from the atom-pair blocks:
// thread = row, a warp = 32 consecutive rows of one column (coalesced stores).  H is
// symmetric, so element (i, j) with i in atom g, j in atom h is read from the stored block
// (h, g) at [e][f] (e, f the functions of j in h and of i in g): consecutive rows of one atom
// read consecutive values.  fn[i] = (local atom << 12) | (f << 6) | nf_g; btab[lg_i * nlg +
// lg_j] = value offset of block (h, g), -1 where the atoms do not overlap.  With F32, the same
// element of the FP32 copy of the blocks (blk32) is written to dense32 as well: the FP32
// standard form then reads FP32 windows (the blocks are converted once, not every window
// element once per GEMM tile).
constexpr int kGatherCols = 32;

template <bool F32>
__global__ void __launch_bounds__(256) gather_windows_kernel(const int* fn, const long long* fnoff, const int* btab,
                                                             const long long* btoff, const int* nlg,
                                                             const long long* offC, const int* n_w, const double* blk,
                                                             double* dense, const float* blk32, float* dense32) {
    const int w = blockIdx.y;
    const int n = n_w[w];
    const int j0 = blockIdx.x * kGatherCols;
    if (j0 >= n) return;
    const int* fw = fn + fnoff[w];
    const int* bt = btab + btoff[w];
    const int L = nlg[w];
    double* D = dense + offC[w];
    float* D32 = F32 ? dense32 + offC[w] : nullptr;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j1 = min(n, j0 + kGatherCols);
    for (int j = j0 + warp; j < j1; j += 8) {
        const int mj = fw[j];
        const int lgj = mj >> 12, e = (mj >> 6) & 63;
        for (int i = lane; i < n; i += 32) {
            const int mi = fw[i];
            const int lgi = mi >> 12, f = (mi >> 6) & 63, nfg = mi & 63;
            const int off = bt[lgi * L + lgj];
            D[i + (long long)j * n] = off >= 0 ? blk[off + e * nfg + f] : 0.0;
            if constexpr (F32) D32[i + (long long)j * n] = off >= 0 ? blk32[off + e * nfg + f] : 0.0f;
        }
    }
}

int gather_windows(int nwin, int nmax, const int* fn, const long long* fnoff, const int* btab, const long long* btoff,
                   const int* nlg, const long long* offC, const int* n_w, const double* blk, double* dense,
                   const float* blk32, float* dense32, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    if (nwin > 65535) {
        lres_set_error("window gather supports at most 65535 windows (got %d)", nwin);
        return LRES_EINVAL;
    }
    const dim3 grid((unsigned)((nmax + kGatherCols - 1) / kGatherCols), (unsigned)nwin);
    if (blk32 && dense32)
        gather_windows_kernel<true><<<grid, 256, 0, s>>>(fn, fnoff, btab, btoff, nlg, offC, n_w, blk, dense, blk32,
                                                         dense32);
    else
        gather_windows_kernel<false><<<grid, 256, 0, s>>>(fn, fnoff, btab, btoff, nlg, offC, n_w, blk, dense, nullptr,
                                                          nullptr);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// F_W[r + a*m] = X[own_w[r], W[a]]
// ---------------------------------------------------------------------------

__global__ void build_F_kernel(const long long* Xp, const int* Xi, const double* Xv, const int* group_of_fn,
                               const int* gptr, const int* gloc, int ngroups, const long long* Ooff,
                               const long long* Oflat, const long long* offF, const int* m_w, double* F) {
    const int w = blockIdx.x;
    const int m = m_w[w];
    const int* gl = gloc + (long long)w * ngroups;
    double* Fw = F + offF[w];
    for (int r = threadIdx.x; r < m; r += blockDim.x) {
        const long long gpt = Oflat[Ooff[w] + r];
        for (long long pidx = Xp[gpt]; pidx < Xp[gpt + 1]; ++pidx) {
            const int f = Xi[pidx];
            const int g = group_of_fn[f];
            const int lo = gl[g];
            if (lo < 0) continue;
            Fw[r + (long long)(lo + f - gptr[g]) * m] = Xv[pidx];
        }
    }
}

int build_F(int nwin, const long long* Xp, const int* Xi, const double* Xv, const int* group_of_fn,
            const int* gptr, const int* gloc, int ngroups, const long long* Ooff, const long long* Oflat,
            const long long* offF, const int* m_w, int mmax, double* F, cudaStream_t s) {
    (void)mmax;
    if (!nwin) return LRES_OK;
    build_F_kernel<<<nwin, 256, 0, s>>>(Xp, Xi, Xv, group_of_fn, gptr, gloc, ngroups, Ooff, Oflat, offF, m_w, F);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// batched FP64 GEMM  C_w = op(A_w) B_w  (n_w x n_w, column-major, same offsets)
// ---------------------------------------------------------------------------

// KLIM = 0: full product.  KLIM = 1: B upper triangular (k <= column).  KLIM = 2: op(A)
// lower triangular (k <= row) and only the lower triangle of C is needed.  TB: C = op(A) B^T.
template <bool TA, int KLIM, bool TB = false>
__global__ void __launch_bounds__(256) gemm_f64_kernel(const int* n_w, const long long* off, const double* A,
                                                       const double* B, double* C) {
    constexpr int BM = 64, BN = 64, BK = 16;
    const int w = blockIdx.z;
    const int n = n_w[w];
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (m0 >= n || n0 >= n) return;
    if (KLIM == 2 && m0 + BM - 1 < n0) return;
    const int kend = KLIM == 1 ? min(n, n0 + BN) : KLIM == 2 ? min(n, m0 + BM) : n;
    const double* Aw = A + off[w];
    const double* Bw = B + off[w];
    double* Cw = C + off[w];
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;   // 16 x 16 threads, 4 x 4 outputs each
    double acc[4][4] = {};
    for (int k0 = 0; k0 < kend; k0 += BK) {
        for (int idx = tid; idx < BK * BM; idx += 256) {
            const int kk = idx / BM, i = idx % BM;
            const int gi = m0 + i, gk = k0 + kk;
            double a = 0.0;
            if (gi < n && gk < n) a = TA ? Aw[gk + (long long)gi * n] : Aw[gi + (long long)gk * n];
            As[kk][i] = a;
        }
        for (int idx = tid; idx < BK * BN; idx += 256) {
            const int j = TB ? idx % BN : idx / BK, kk = TB ? idx / BN : idx % BK;
            const int gj = n0 + j, gk = k0 + kk;
            Bs[kk][j] = (gj < n && gk < n) ? (TB ? Bw[gj + (long long)gk * n] : Bw[gk + (long long)gj * n]) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[kk][tx + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) b[v] = Bs[kk][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int gi = m0 + tx + 16 * u, gj = n0 + ty + 16 * v;
            if (gi < n && gj < n) Cw[gi + (long long)gj * n] = acc[u][v];
        }
}

// C_w = A_w U_w with A_w m_w x n_w (column-major, leading dimension m_w, offsets offA) and
// U_w n_w x n_w upper triangular (column-major, offsets offU): the owned-point rows in the
// standard form, F^ = F L^-T.
__global__ void __launch_bounds__(256) gemm_rect_upper_kernel(const int* n_w, const int* m_w, const long long* offA,
                                                              const long long* offU, const double* A,
                                                              const double* U, double* C) {
    constexpr int BM = 64, BN = 64, BK = 16;
    const int w = blockIdx.z;
    const int n = n_w[w], m = m_w[w];
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (m0 >= m || n0 >= n) return;
    const int kend = min(n, n0 + BN);
    const double* Aw = A + offA[w];
    const double* Uw = U + offU[w];
    double* Cw = C + offA[w];
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < kend; k0 += BK) {
        for (int idx = tid; idx < BK * BM; idx += 256) {
            const int kk = idx / BM, i = idx % BM;
            const int gi = m0 + i, gk = k0 + kk;
            As[kk][i] = (gi < m && gk < n) ? Aw[gi + (long long)gk * m] : 0.0;
        }
        for (int idx = tid; idx < BK * BN; idx += 256) {
            const int j = idx / BK, kk = idx % BK;
            const int gj = n0 + j, gk = k0 + kk;
            Bs[kk][j] = (gj < n && gk <= gj) ? Uw[gk + (long long)gj * n] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[kk][tx + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) b[v] = Bs[kk][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int gi = m0 + tx + 16 * u, gj = n0 + ty + 16 * v;
            if (gi < m && gj < n) Cw[gi + (long long)gj * m] = acc[u][v];
        }
}

// K_w = F_w^T F_w (n_w x n_w, column-major at offK) from the owned-point rows F_w (m_w x n_w,
// leading dimension m_w at offF); lower-triangle tiles computed, mirrored.
__global__ void __launch_bounds__(256) gram_kernel(const int* n_w, const int* m_w, const long long* offF,
                                                   const long long* offK, const double* F, double* K) {
    constexpr int BM = 64, BK = 16;
    const int w = blockIdx.z;
    const int n = n_w[w], m = m_w[w];
    const int a0 = blockIdx.x * BM, b0 = blockIdx.y * BM;
    if (a0 >= n || b0 >= n || a0 < b0) return;
    const double* Fw = F + offF[w];
    double* Kw = K + offK[w];
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BM + 1];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    double acc[4][4] = {};
    for (int r0 = 0; r0 < m; r0 += BK) {
        for (int idx = tid; idx < BK * BM; idx += 256) {
            const int kk = idx % BK, i = idx / BK;         // rows contiguous
            const int r = r0 + kk;
            As[kk][i] = (r < m && a0 + i < n) ? Fw[r + (long long)(a0 + i) * m] : 0.0;
            Bs[kk][i] = (r < m && b0 + i < n) ? Fw[r + (long long)(b0 + i) * m] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[kk][tx + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) b[v] = Bs[kk][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int a = a0 + tx + 16 * u, b = b0 + ty + 16 * v;
            if (a < n && b < n) {
                Kw[a + (long long)b * n] = acc[u][v];
                Kw[b + (long long)a * n] = acc[u][v];
            }
        }
}

int batched_gram(int nwin, const int* n_w, const int* m_w, const long long* offF, const long long* offK, int nmax,
                 const double* F, double* K, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    dim3 grid((nmax + 63) / 64, (nmax + 63) / 64, nwin);
    gram_kernel<<<grid, 256, 0, s>>>(n_w, m_w, offF, offK, F, K);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int batched_gemm_rect_upper(int nwin, const int* n_w, const int* m_w, const long long* offA, const long long* offU,
                            int nmax, int mmax, const double* A, const double* U, double* C, cudaStream_t s) {
    if (!nwin || !mmax) return LRES_OK;
    dim3 grid((mmax + 63) / 64, (nmax + 63) / 64, nwin);
    gemm_rect_upper_kernel<<<grid, 256, 0, s>>>(n_w, m_w, offA, offU, A, U, C);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int batched_gemm(int nwin, const int* n_w, const long long* offA, int nmax, bool transA, const double* A,
                 const double* B, double* C, cudaStream_t s, int klim, bool transB) {
    if (!nwin) return LRES_OK;
    dim3 grid((nmax + 63) / 64, (nmax + 63) / 64, nwin);
    if (transB) {
        if (transA || klim) {
            lres_set_error("unsupported FP64 GEMM variant");
            return LRES_EINVAL;
        }
        gemm_f64_kernel<false, 0, true><<<grid, 256, 0, s>>>(n_w, offA, A, B, C);
    } else if (transA) {
        if (klim == 2) gemm_f64_kernel<true, 2><<<grid, 256, 0, s>>>(n_w, offA, A, B, C);
        else gemm_f64_kernel<true, 0><<<grid, 256, 0, s>>>(n_w, offA, A, B, C);
    } else {
        if (klim == 1) gemm_f64_kernel<false, 1><<<grid, 256, 0, s>>>(n_w, offA, A, B, C);
        else gemm_f64_kernel<false, 0><<<grid, 256, 0, s>>>(n_w, offA, A, B, C);
    }
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

__global__ void convert_kernel(const double* a, float* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

int convert_f64_f32(const double* a, float* b, long long n, cudaStream_t s) {
    if (n <= 0) return LRES_OK;
    convert_kernel<<<1216, 256, 0, s>>>(a, b, n);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// pole sums: n(r) = 4 Re sum_k w_k q_k(r),  e(r) = 4 Re sum_k w_k z_k q_k(r)
// (factor 2 for the conjugate half-plane, 2 for spin); one CTA per window,
// fixed summation order (bitwise reproducible)
// ---------------------------------------------------------------------------

template <class T>
__global__ void __launch_bounds__(256) pole_sum_kernel(const long long* offQ, const int* m_w, const long long* Oflat,
                                                       const T* q, long long qstride, int npoles, const double2* wq,
                                                       const double2* wzq, double dV, double* dens, double* n_out,
                                                       double* e_out) {
    const int w = blockIdx.x;
    const int m = m_w[w];
    const long long base = offQ[w];
    double sn = 0.0, se = 0.0;
    for (int r = threadIdx.x; r < m; r += blockDim.x) {
        double an = 0.0, ae = 0.0;
        for (int k = 0; k < npoles; ++k) {
            const T x = q[(long long)k * qstride + base + r];
            const double qx = (double)x.x, qy = (double)x.y;
            const double2 a = wq[k], b = wzq[k];
            an += a.x * qx - a.y * qy;
            ae += b.x * qx - b.y * qy;
        }
        const double nr = 4.0 * an, er = 4.0 * ae;
        if (dens) dens[Oflat[base + r]] = nr;
        sn += nr;
        se += er;
    }
    __shared__ double red[2][256];
    red[0][threadIdx.x] = sn;
    red[1][threadIdx.x] = se;
    __syncthreads();
    for (int o = 128; o; o >>= 1) {
        if (threadIdx.x < o) {
            red[0][threadIdx.x] += red[0][threadIdx.x + o];
            red[1][threadIdx.x] += red[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        n_out[w] = red[0][0] * dV;
        e_out[w] = red[1][0] * dV;
    }
}

int pole_sums(int nwin, const long long* offQ, const int* m_w, const long long* Oflat, bool fp32, const void* q,
              long long qstride, int npoles, const double2* wq, const double2* wzq, double dV, double* dens,
              double* n_w, double* e_w, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    if (fp32)
        pole_sum_kernel<float2><<<nwin, 256, 0, s>>>(offQ, m_w, Oflat, (const float2*)q, qstride, npoles, wq, wzq, dV,
                                                     dens, n_w, e_w);
    else
        pole_sum_kernel<double2><<<nwin, 256, 0, s>>>(offQ, m_w, Oflat, (const double2*)q, qstride, npoles, wq, wzq,
                                                      dV, dens, n_w, e_w);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}



// ---------------------------------------------------------------------------
// Standard-form transform in double-float arithmetic on the FP32 pipes.
// Every FP64 operand x is carried as an unevaluated pair (hi, lo) of floats with
// hi = fl32(x), lo = fl32(x - hi) (about 48 significant bits); products use the exact
// FMA residual of hi*hi plus the two cross terms, sums use Knuth's TwoSum, so the
// accumulated result keeps ~1e-14 relative accuracy — far below the FP32 rounding of
// the final H^ — at ~11 FP32 operations per multiply-add instead of one FP64 FMA.
// ---------------------------------------------------------------------------

__global__ void split_f64_kernel(const double* a, float2* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double x = a[i];
        const float hi = (float)x;
        b[i] = make_float2(hi, (float)(x - (double)hi));
    }
}

int split_f64(const double* a, float2* b, long long n, cudaStream_t s) {
    if (n <= 0) return LRES_OK;
    split_f64_kernel<<<1216, 256, 0, s>>>(a, b, n);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// Explicitly rounded operations keep the compiler from contracting the error-free
// transformations into fused multiply-adds.
__device__ __forceinline__ void df_mac(float2 a, float2 b, float& sh, float& sl) {
    const float ph = __fmul_rn(a.x, b.x);
    float pl = fmaf(a.x, b.x, -ph);          // exact residual of the leading product
    pl = fmaf(a.x, b.y, pl);
    pl = fmaf(a.y, b.x, pl);
    const float t = __fadd_rn(sh, ph);       // TwoSum(sh, ph)
    const float v = __fsub_rn(t, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, v)), __fsub_rn(ph, v));
    sl = __fadd_rn(sl, __fadd_rn(e, pl));
    sh = t;
}

// KLIM as gemm_f64_kernel.  OUT32: write fl32(hi + lo) to a float array, else (hi, lo).
template <bool TA, int KLIM, bool OUT32>
__global__ void __launch_bounds__(256) gemm_df64_kernel(const int* n_w, const long long* off, const float2* A,
                                                        const float2* B, float2* C, float* C32) {
    constexpr int BM = 64, BN = 64, BK = 16;
    const int w = blockIdx.z;
    const int n = n_w[w];
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (m0 >= n || n0 >= n) return;
    if (KLIM == 2 && m0 + BM - 1 < n0) return;
    const int kend = KLIM == 1 ? min(n, n0 + BN) : KLIM == 2 ? min(n, m0 + BM) : n;
    const float2* Aw = A + off[w];
    const float2* Bw = B + off[w];
    __shared__ float2 As[BK][BM + 1];
    __shared__ float2 Bs[BK][BN + 1];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    float sh[4][4], sl[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) sh[u][v] = sl[u][v] = 0.f;
    for (int k0 = 0; k0 < kend; k0 += BK) {
        for (int idx = tid; idx < BK * BM; idx += 256) {
            const int kk = idx / BM, i = idx % BM;
            const int gi = m0 + i, gk = k0 + kk;
            float2 a = make_float2(0.f, 0.f);
            if (gi < n && gk < n) a = TA ? Aw[gk + (long long)gi * n] : Aw[gi + (long long)gk * n];
            As[kk][i] = a;
        }
        for (int idx = tid; idx < BK * BN; idx += 256) {
            const int j = idx / BK, kk = idx % BK;
            const int gj = n0 + j, gk = k0 + kk;
            Bs[kk][j] = (gj < n && gk < n) ? Bw[gk + (long long)gj * n] : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < BK; ++kk) {
            float2 a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[kk][tx + 16 * u];
#pragma unroll
            for (int v = 0; v < 4; ++v) b[v] = Bs[kk][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) df_mac(a[u], b[v], sh[u][v], sl[u][v]);
        }
        __syncthreads();
    }
    float* C32w = OUT32 ? C32 + off[w] : nullptr;
    float2* Cw = OUT32 ? nullptr : C + off[w];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int gi = m0 + tx + 16 * u, gj = n0 + ty + 16 * v;
            if (gi >= n || gj >= n) continue;
            const float hi = __fadd_rn(sh[u][v], sl[u][v]);          // renormalise (fast TwoSum)
            const float lo = __fsub_rn(sl[u][v], __fsub_rn(hi, sh[u][v]));
            if (OUT32) C32w[gi + (long long)gj * n] = hi;
            else Cw[gi + (long long)gj * n] = make_float2(hi, lo);
        }
}

// ---------------------------------------------------------------------------
// batched FP32 GEMM with blocked sums  C_w = A_w B_w  (n_w x n_w, offsets off)
// ---------------------------------------------------------------------------
// KLIM as gemm_f64_kernel (1: B upper triangular, k <= column; 2: A lower triangular, k <= row,
// lower triangle of C only).  A is column-major, FP64 (converted on load) or FP32; B is given
// k-major (Bt[j + k n] = B[k][j], i.e. B stored row-major), so that both operand tiles are
// staged with coalesced loads and conflict-free stores and read as 16-byte vectors; C is
// written column-major or (CROW) row-major, the k-major layout of the next product.  Each
// 32-term block of the k sum is formed from zero and added to the running value, so the
// rounding grows with the number of blocks rather than the number of terms.  64 x 64 tiles,
// 128 threads, 8 x 4 outputs per thread (rows 4tx..4tx+3 and 32+4tx..; columns 4ty..4ty+3:
// per k two 16-byte loads of A and one of B feed 32 FMAs); the next k tile is loaded into
// registers while the current one is multiplied (two shared-memory buffers).
template <int KLIM, bool AF64, bool CROW>
__global__ void __launch_bounds__(128, 3) gemm_f32blk_kernel(const int* n_w, const long long* off, const void* Av,
                                                          const float* Bt, float* C) {
    constexpr int BM = 64, BN = 64, BK = 32, NT = 128, PER = BK * BM / NT;     // 16 staged values each
    const int w = blockIdx.z;
    const int n = n_w[w];
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    if (m0 >= n || n0 >= n) return;
    if (KLIM == 2 && m0 + BM - 1 < n0) return;
    const int kend = KLIM == 1 ? min(n, n0 + BN) : KLIM == 2 ? min(n, m0 + BM) : n;
    const double* A64 = AF64 ? static_cast<const double*>(Av) + off[w] : nullptr;
    const float* A32 = AF64 ? nullptr : static_cast<const float*>(Av) + off[w];
    const float* Bw = Bt + off[w];
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Bs[2][BK][BN];
    const int tid = threadIdx.x;
    const int tx = tid & 7, ty = tid >> 3;
    // the next tile is held in registers as loaded (FP64 values converted only when stored,
    // so that the loads stay in flight during the multiplication)
    using AT = typename std::conditional<AF64, double, float>::type;
    AT ra[PER];
    float rb[PER];
    auto load = [&](int k0) {
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = tid + q * NT, kk = idx / BM, x = idx % BM;
            const int gk = k0 + kk;
            const int gi = m0 + x, gj = n0 + x;
            AT a = AT(0);
            float b = 0.f;
            if (gi < n && gk < n) {
                if constexpr (AF64) a = A64[gi + (long long)gk * n];
                else a = A32[gi + (long long)gk * n];
            }
            if (gj < n && gk < n) b = Bw[gj + (long long)gk * n];
            ra[q] = a;
            rb[q] = b;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int idx = tid + q * NT, kk = idx / BM, x = idx % BM;
            As[buf][kk][x] = (float)ra[q];
            Bs[buf][kk][x] = rb[q];
        }
    };
    float acc[8][4];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
    load(0);
    store(0);
    __syncthreads();
    int buf = 0;
    for (int k0 = 0; k0 < kend; k0 += BK) {
        const bool more = k0 + BK < kend;
        if (more) load(k0 + BK);
        float blk[8][4];
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) blk[u][v] = 0.f;
#pragma unroll 8
        for (int kk = 0; kk < BK; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][4 * tx]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][32 + 4 * tx]);
            const float4 b = *reinterpret_cast<const float4*>(&Bs[buf][kk][4 * ty]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) blk[u][v] = fmaf(av[u], bv[v], blk[u][v]);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] += blk[u][v];
        if (more) {
            store(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }
    float* Cw = C + off[w];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int gi = m0 + (u < 4 ? 4 * tx + u : 32 + 4 * tx + u - 4), gj = n0 + 4 * ty + v;
            if (gi < n && gj < n) {
                if (CROW) Cw[(long long)gi * n + gj] = acc[u][v];
                else Cw[gi + (long long)gj * n] = acc[u][v];
            }
        }
}

int batched_gemm_f32(int nwin, const int* n_w, const long long* off, int nmax, int klim, const void* A, bool a_f64,
                     const float* Bt, float* C, bool c_rowmajor, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    if (nwin > 65535) {
        lres_set_error("FP32 GEMM supports at most 65535 windows (got %d)", nwin);
        return LRES_EINVAL;
    }
    dim3 grid((nmax + 63) / 64, (nmax + 63) / 64, nwin);
    if (klim == 1 && a_f64 && c_rowmajor) gemm_f32blk_kernel<1, true, true><<<grid, 128, 0, s>>>(n_w, off, A, Bt, C);
    else if (klim == 1 && !a_f64 && c_rowmajor)
        gemm_f32blk_kernel<1, false, true><<<grid, 128, 0, s>>>(n_w, off, A, Bt, C);
    else if (klim == 2 && !a_f64 && !c_rowmajor)
        gemm_f32blk_kernel<2, false, false><<<grid, 128, 0, s>>>(n_w, off, A, Bt, C);
    else {
        lres_set_error("unsupported FP32 GEMM variant");
        return LRES_EINVAL;
    }
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// B_w = A_w^T for every window block (FP32, one 32 x 32 tile per CTA through shared memory).
__global__ void transpose_f32_kernel(const int* n_w, const long long* off, const float* A, float* B) {
    __shared__ float t[32][33];
    const int w = blockIdx.z, n = n_w[w];
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    if (i0 >= n || j0 >= n) return;
    const float* Aw = A + off[w];
    float* Bw = B + off[w];
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        const int i = i0 + threadIdx.x, j = j0 + c;
        t[c][threadIdx.x] = (i < n && j < n) ? Aw[i + (long long)j * n] : 0.f;
    }
    __syncthreads();
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        const int j = j0 + threadIdx.x, i = i0 + c;     // B[j, i] = A[i, j]
        if (i < n && j < n) Bw[j + (long long)i * n] = t[threadIdx.x][c];
    }
}

int batched_transpose_f32(int nwin, const int* n_w, const long long* off, int nmax, const float* A, float* B,
                          cudaStream_t s) {
    if (!nwin) return LRES_OK;
    dim3 grid((nmax + 31) / 32, (nmax + 31) / 32, nwin);
    transpose_f32_kernel<<<grid, dim3(32, 8), 0, s>>>(n_w, off, A, B);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

int batched_gemm_df64(int nwin, const int* n_w, const long long* off, int nmax, bool transA, int klim,
                      const float2* A, const float2* B, float2* C, float* C32, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    dim3 grid((nmax + 63) / 64, (nmax + 63) / 64, nwin);
    if (!transA && klim == 1 && C)
        gemm_df64_kernel<false, 1, false><<<grid, 256, 0, s>>>(n_w, off, A, B, C, nullptr);
    else if (transA && klim == 2 && C32)
        gemm_df64_kernel<true, 2, true><<<grid, 256, 0, s>>>(n_w, off, A, B, nullptr, C32);
    else {
        lres_set_error("unsupported double-float GEMM variant");
        return LRES_EINVAL;
    }
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

}  // namespace lres

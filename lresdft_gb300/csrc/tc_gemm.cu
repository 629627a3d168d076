// The standard-form products of the mixed tridiagonal route on the 5th-generation tensor
// cores: Y = H L^-T and A^ = lower(L^-1 Y) for every window, C_w = A_w B_w (n_w x n_w), as
// batched_gemm_f32 computes them on the SIMT pipes (same operand layouts: A column-major,
// FP64 or FP32; B k-major; C row- or column-major; the same triangular limits).
//
// A CTA computes a 128 x 64 tile of C: 128 threads, thread = row = TMEM lane.  The K sum runs
// in chunks of 32: each chunk's operands are split into TF32 pairs x = hi + lo and staged in
// shared memory (K-major, 8 x 16-byte core matrices, no swizzle); one thread issues the 3xTF32
// products hi.hi + hi.lo + lo.hi of the chunk (12 tcgen05.mma.kind::tf32, K = 8 each) into a
// 64-column TMEM accumulator that starts from zero, commits them to an mbarrier, and the
// threads add the chunk's sums (tcgen05.ld) to their rows' running values in registers, so
// the K sum is blocked in 32-term chunks as on the SIMT path.  Two shared-memory stages and
// two accumulators: chunk c+1 is staged and its MMAs issued before chunk c is read back, and
// the global loads of chunk c+2 are in flight meanwhile.  Every mbarrier wait is bounded: on a
// timeout the kernel sets ST_TIMEOUT in *status, waits (bounded) for its MMAs in flight,
// frees its tensor memory and returns.
#include "common.cuh"
#include "launch.cuh"
#include "lres_internal.h"

#include <type_traits>

namespace lres {
namespace {

namespace tg {
constexpr int M = 128, N = 64, KR = 32;
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
// kind::tf32: D f32, A and B tf32, N and M
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
// 64 consecutive columns of this thread's TMEM lane, added to acc
__device__ __forceinline__ void ld64_add(uint32_t taddr, float* acc) {
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
    for (int j = 0; j < 64; ++j) acc[j] += __uint_as_float(r[j]);
}
// bounded wait on an mbarrier phase; true when it completed
__device__ __forceinline__ bool wait_phase(uint32_t mbar, uint32_t phase) {
    uint32_t done = 0;
    for (int spin = 0; spin < (1 << 24) && !done; ++spin)
        asm volatile("{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n"
                     "selp.u32 %0, 1, 0, q; }" : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
    return done != 0;
}
}  // namespace tg

template <int KLIM, bool AF64, bool CROW>
__global__ void __launch_bounds__(128, 2) gemm_tc_kernel(const int* n_w, const long long* off, const void* Av,
                                                         const float* Bt, float* C, int* status) {
    using AT = typename std::conditional<AF64, double, float>::type;
    extern __shared__ __align__(128) unsigned char smem_g[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int bail_sh;
    const int w = blockIdx.z;
    const int n = n_w[w];
    const int m0 = blockIdx.x * tg::M, n0 = blockIdx.y * tg::N;
    // whole-CTA exits only (before any barrier or tensor-memory allocation)
    if (m0 >= n || n0 >= n) return;
    if (KLIM == 2 && m0 + tg::M - 1 < n0) return;
    const int kend = KLIM == 1 ? min(n, n0 + tg::N) : KLIM == 2 ? min(n, m0 + tg::M) : n;
    const int nch = (kend + tg::KR - 1) / tg::KR;
    const AT* A = static_cast<const AT*>(Av) + off[w];
    const float* Bw = Bt + off[w];
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t mb0 = (uint32_t)__cvta_generic_to_shared(&mbar[0]);
    const uint32_t mb1 = (uint32_t)__cvta_generic_to_shared(&mbar[1]);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem_g);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb0));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb1));
        bail_sh = 0;
    }
    if (warp == 0) {
        const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "n"(tg::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    const uint32_t my_lane = (uint32_t)(warp * 32) << 16;
    uint32_t ph[2] = {0u, 0u};
    int pend[2] = {0, 0};

    // operands of one chunk in registers: row tid of A (32 k), 16 (column, k) entries of B
    AT ar[tg::KR];
    float br[16];
    const int row = m0 + tid;
    const int bj = tid & 63, bk0 = (tid >> 6) * 16;
    auto load = [&](int c) {
        const int k0 = c * tg::KR;
#pragma unroll
        for (int kk = 0; kk < tg::KR; ++kk) {
            const int k = k0 + kk;
            ar[kk] = (row < n && k < kend) ? A[row + (long long)k * n] : AT(0);
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int k = k0 + bk0 + q, j = n0 + bj;
            br[q] = (j < n && k < kend) ? Bw[j + (long long)k * n] : 0.0f;
        }
    };
    auto stage = [&](int st) {
        float* Ahi = reinterpret_cast<float*>(smem_g + st * tg::STAGE_BYTES);
        float* Alo = reinterpret_cast<float*>(smem_g + st * tg::STAGE_BYTES + tg::A_BYTES);
        float* Bhi = reinterpret_cast<float*>(smem_g + st * tg::STAGE_BYTES + 2 * tg::A_BYTES);
        float* Blo = reinterpret_cast<float*>(smem_g + st * tg::STAGE_BYTES + 2 * tg::A_BYTES + tg::B_BYTES);
#pragma unroll
        for (int kk = 0; kk < tg::KR; kk += 4) {
            float h[4], l[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) tg::split((float)ar[kk + u], h[u], l[u]);
            *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(Ahi) + tg::off(tid, kk)) =
                make_float4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(Alo) + tg::off(tid, kk)) =
                make_float4(l[0], l[1], l[2], l[3]);
        }
#pragma unroll
        for (int q = 0; q < 16; q += 4) {
            float h[4], l[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) tg::split(br[q + u], h[u], l[u]);
            *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(Bhi) + tg::off(bj, bk0 + q)) =
                make_float4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(Blo) + tg::off(bj, bk0 + q)) =
                make_float4(l[0], l[1], l[2], l[3]);
        }
    };
    auto issue = [&](int st) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (tid == 0) {
            const uint32_t aH = sbase + st * tg::STAGE_BYTES, aL = aH + tg::A_BYTES;
            const uint32_t bH = aH + 2 * tg::A_BYTES, bL = bH + tg::B_BYTES;
            const uint32_t acc_t = tmem + (uint32_t)(st * 64);
#pragma unroll
            for (int kb = 0; kb < tg::KR / 8; ++kb)
                tg::mma(acc_t, tg::desc(aH + kb * 2 * tg::LBO), tg::desc(bH + kb * 2 * tg::LBO), kb > 0);
#pragma unroll
            for (int kb = 0; kb < tg::KR / 8; ++kb)
                tg::mma(acc_t, tg::desc(aH + kb * 2 * tg::LBO), tg::desc(bL + kb * 2 * tg::LBO), 1);
#pragma unroll
            for (int kb = 0; kb < tg::KR / 8; ++kb)
                tg::mma(acc_t, tg::desc(aL + kb * 2 * tg::LBO), tg::desc(bH + kb * 2 * tg::LBO), 1);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(st ? mb1 : mb0));
        }
        pend[st] = 1;
    };
    float acc[64];
#pragma unroll
    for (int j = 0; j < 64; ++j) acc[j] = 0.0f;
    auto finish = [&](int st) -> bool {
        bool ok = tg::wait_phase(st ? mb1 : mb0, ph[st]);
        if (ok) {
            ph[st] ^= 1u;
            pend[st] = 0;
        } else {
            atomicOr(status, ST_TIMEOUT);
            atomicOr(&bail_sh, 1);
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        ok = __all_sync(0xffffffffu, ok);                 // tcgen05.ld is warp-collective
        if (ok) tg::ld64_add(tmem + my_lane + (uint32_t)(st * 64), acc);
        return ok;
    };

    load(0);
    stage(0);
    issue(0);
    if (nch > 1) load(1);
    bool ok = true;
    for (int c = 0; c < nch && ok; ++c) {
        if (c + 1 < nch) {
            stage((c + 1) & 1);
            issue((c + 1) & 1);
            if (c + 2 < nch) load(c + 2);
        }
        ok = finish(c & 1);
        __syncthreads();                                  // every thread's read-back before reuse
        if (bail_sh) ok = false;
    }
    if (ok) {
        float* Cw = C + off[w];
        if (row < n) {
#pragma unroll
            for (int j = 0; j < 64; ++j) {
                const int col = n0 + j;
                if (col < n) {
                    if (CROW) Cw[(long long)row * n + col] = acc[j];
                    else Cw[row + (long long)col * n] = acc[j];
                }
            }
        }
    }
    // MMAs still in flight after a timeout: bounded wait before the tensor memory is released
    if (pend[0]) (void)tg::wait_phase(mb0, ph[0]);
    if (pend[1]) (void)tg::wait_phase(mb1, ph[1]);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(tg::TMEM_COLS));
}

template <int KLIM, bool AF64, bool CROW>
int launch_tc(int nwin, const int* n_w, const long long* off, int nmax, const void* A, const float* Bt, float* C,
              int* status, cudaStream_t s) {
    const size_t smem = 2 * (size_t)tg::STAGE_BYTES;
    int per_sm = 0;
    if (int rc = prepare_kernel<gemm_tc_kernel<KLIM, AF64, CROW>>(128, smem, &per_sm)) return rc;
    const dim3 grid((unsigned)((nmax + tg::M - 1) / tg::M), (unsigned)((nmax + tg::N - 1) / tg::N), (unsigned)nwin);
    gemm_tc_kernel<KLIM, AF64, CROW><<<grid, 128, smem, s>>>(n_w, off, A, Bt, C, status);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

}  // namespace

int batched_gemm_tc(int nwin, const int* n_w, const long long* off, int nmax, int klim, const void* A, bool a_f64,
                    const float* Bt, float* C, bool c_rowmajor, int* status, cudaStream_t s) {
    if (!nwin) return LRES_OK;
    if (nwin > 65535) {
        lres_set_error("tensor-core GEMM supports at most 65535 windows (got %d)", nwin);
        return LRES_EINVAL;
    }
    if (klim == 1 && a_f64 && c_rowmajor) return launch_tc<1, true, true>(nwin, n_w, off, nmax, A, Bt, C, status, s);
    if (klim == 2 && !a_f64 && !c_rowmajor)
        return launch_tc<2, false, false>(nwin, n_w, off, nmax, A, Bt, C, status, s);
    lres_set_error("unsupported tensor-core GEMM variant");
    return LRES_EINVAL;
}

}  // namespace lres

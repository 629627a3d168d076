// Dense Kohn-Sham LCAO on the GPU (ks_lcao, lrft/lcao3d.py:110-117; ks_density,
// src/lrft_cpp.cpp:235-284): the lowest nocc + 1 eigenpairs of the generalised problem
// H C = S C diag(w) for the whole cell, the density n(r) = 2 sum_{i < nocc} (X[r,:] C_i)^2 and
// the band energy 2 sum_{i < nocc} w_i.  This is the oracle side of the identity
// LRes(R_w >= cell) = KS, not the window solve.
//
// The dense symmetric-definite eigensolver is LAPACK's in the reference (dsygvx); here it is
// cuSOLVER's dsygvd (Cholesky, reduction to standard form, divide and conquer), opened at
// run time with dlopen so that the library does not depend on it.  The kernels around it are
// this file's: H and S densified from CSR, C transposed to rows, and the density as one warp
// per grid point over the sparse row of X (lanes over the occupied states, a fixed butterfly
// for the sum of squares, so the result does not depend on the schedule).
#include "common.cuh"
#include "lres_internal.h"

#include <cusolverDn.h>
#include <dlfcn.h>

#include <vector>

namespace lres {
namespace {

__global__ void csr_to_dense_kernel(long long n, const long long* p, const long long* idx, const double* v,
                                    double* A) {
    const long long r = (long long)blockIdx.x * blockDim.y + threadIdx.y;
    if (r >= n) return;
    for (long long k = p[r] + threadIdx.x; k < p[r + 1]; k += blockDim.x) A[idx[k] * n + r] = v[k];
}

// Ct[mu * nocc + i] = C[i * n + mu] (C column-major, eigenvector i in column i)
__global__ void transpose_occ_kernel(long long n, int nocc, const double* C, double* Ct) {
    __shared__ double tile[32][33];
    const long long mu0 = (long long)blockIdx.x * 32, i0 = (long long)blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const long long i = i0 + y, mu = mu0 + threadIdx.x;
        tile[y][threadIdx.x] = (i < nocc && mu < n) ? C[i * n + mu] : 0.0;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const long long mu = mu0 + y, i = i0 + threadIdx.x;
        if (mu < n && i < nocc) Ct[mu * nocc + i] = tile[threadIdx.x][y];
    }
}

// n(r) = 2 sum_i (sum_p Xv[p] Ct[Xi[p], i])^2, one warp per grid point
__global__ void ks_density_kernel(long long ng, int nocc, const long long* Xp, const long long* Xi, const double* Xv,
                                  const double* Ct, double* dens) {
    const long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= ng) return;
    double s = 0.0;
    for (int i0 = 0; i0 < nocc; i0 += 32) {
        const int i = i0 + lane;
        double t = 0.0;
        if (i < nocc)
            for (long long p = Xp[r]; p < Xp[r + 1]; ++p) t += Xv[p] * Ct[Xi[p] * nocc + i];
        s += t * t;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) dens[r] = 2.0 * s;
}

// cuSOLVER entry points, resolved once
struct Solver {
    bool tried = false, ok = false;
    decltype(&cusolverDnCreate) create = nullptr;
    decltype(&cusolverDnDestroy) destroy = nullptr;
    decltype(&cusolverDnDsygvd_bufferSize) sygvd_buffer = nullptr;
    decltype(&cusolverDnDsygvd) sygvd = nullptr;
};

Solver& solver() {
    static Solver s;
    if (s.tried) return s;
    s.tried = true;
    void* h = nullptr;
    for (const char* name : {"libcusolver.so.12", "libcusolver.so.11", "libcusolver.so"})
        if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return s;
    s.create = reinterpret_cast<decltype(s.create)>(dlsym(h, "cusolverDnCreate"));
    s.destroy = reinterpret_cast<decltype(s.destroy)>(dlsym(h, "cusolverDnDestroy"));
    s.sygvd_buffer = reinterpret_cast<decltype(s.sygvd_buffer)>(dlsym(h, "cusolverDnDsygvd_bufferSize"));
    s.sygvd = reinterpret_cast<decltype(s.sygvd)>(dlsym(h, "cusolverDnDsygvd"));
    s.ok = s.create && s.destroy && s.sygvd_buffer && s.sygvd;
    return s;
}

template <class T>
int up(T** d, const T* h, long long n) {
    LRES_CUDA_TRY(cudaMalloc(d, sizeof(T) * (size_t)std::max<long long>(n, 1)));
    if (n) LRES_CUDA_TRY(cudaMemcpy(*d, h, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice));
    return LRES_OK;
}

}  // namespace
}  // namespace lres

using namespace lres;

extern "C" int lres_ks_density(int64_t nb, const int64_t* Hp, const int64_t* Hi, const double* Hv, const int64_t* Sp,
                               const int64_t* Si, const double* Sv, int64_t ng, const int64_t* Xp, const int64_t* Xi,
                               const double* Xv, int32_t nocc, double* dens, double* w, double* e_band) {
    if (nb <= 0 || ng <= 0 || nocc < 0 || nocc >= nb || !Hp || !Hi || !Hv || !Sp || !Si || !Sv || !Xp || !Xi ||
        !Xv || !dens || !w || !e_band) {
        lres_set_error("lres_ks_density: bad arguments (0 <= nocc < nb)");
        return LRES_EINVAL;
    }
    if (nb > 46340) {                                   // nb^2 within 2^31 (cuSOLVER's int sizes)
        lres_set_error("lres_ks_density: nb = %lld too large for the dense solve", (long long)nb);
        return LRES_EINVAL;
    }
    Solver& sv = solver();
    if (!sv.ok) {
        lres_set_error("lres_ks_density: cuSOLVER (libcusolver) not found");
        return LRES_ESTATE;
    }
    const long long n = nb, nnzH = Hp[nb], nnzS = Sp[nb], nnzX = Xp[ng];
    long long *dHp = nullptr, *dHi = nullptr, *dSp = nullptr, *dSi = nullptr, *dXp = nullptr, *dXi = nullptr;
    double *dHv = nullptr, *dSv = nullptr, *dXv = nullptr, *A = nullptr, *B = nullptr, *W = nullptr, *work = nullptr,
           *Ct = nullptr, *dd = nullptr;
    int* info = nullptr;
    cusolverDnHandle_t h = nullptr;
    auto run = [&]() -> int {
        if (int e = up(&dHp, (const long long*)Hp, n + 1)) return e;
        if (int e = up(&dHi, (const long long*)Hi, nnzH)) return e;
        if (int e = up(&dHv, Hv, nnzH)) return e;
        if (int e = up(&dSp, (const long long*)Sp, n + 1)) return e;
        if (int e = up(&dSi, (const long long*)Si, nnzS)) return e;
        if (int e = up(&dSv, Sv, nnzS)) return e;
        LRES_CUDA_TRY(cudaMalloc(&A, sizeof(double) * n * n));
        LRES_CUDA_TRY(cudaMalloc(&B, sizeof(double) * n * n));
        LRES_CUDA_TRY(cudaMalloc(&W, sizeof(double) * n));
        LRES_CUDA_TRY(cudaMalloc(&info, sizeof(int)));
        LRES_CUDA_TRY(cudaMemset(A, 0, sizeof(double) * n * n));
        LRES_CUDA_TRY(cudaMemset(B, 0, sizeof(double) * n * n));
        const dim3 blk(32, 8);
        const unsigned g = (unsigned)((n + 7) / 8);
        csr_to_dense_kernel<<<g, blk>>>(n, dHp, dHi, dHv, A);
        csr_to_dense_kernel<<<g, blk>>>(n, dSp, dSi, dSv, B);
        LRES_CUDA_TRY(cudaGetLastError());
        if (sv.create(&h) != CUSOLVER_STATUS_SUCCESS) {
            lres_set_error("lres_ks_density: cusolverDnCreate failed");
            return LRES_ECUDA;
        }
        int lwork = 0;
        if (sv.sygvd_buffer(h, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)n, A,
                            (int)n, B, (int)n, W, &lwork) != CUSOLVER_STATUS_SUCCESS) {
            lres_set_error("lres_ks_density: dsygvd workspace query failed");
            return LRES_ECUDA;
        }
        LRES_CUDA_TRY(cudaMalloc(&work, sizeof(double) * (size_t)std::max(lwork, 1)));
        if (sv.sygvd(h, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)n, A, (int)n, B,
                     (int)n, W, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) {
            lres_set_error("lres_ks_density: dsygvd failed");
            return LRES_ECUDA;
        }
        int hinfo = 0;
        LRES_CUDA_TRY(cudaMemcpy(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost));
        if (hinfo) {
            lres_set_error("lres_ks_density: dsygvd info %d (S not positive definite or no convergence)", hinfo);
            return LRES_ENUMERIC;
        }
        std::vector<double> hw(n);
        LRES_CUDA_TRY(cudaMemcpy(hw.data(), W, sizeof(double) * n, cudaMemcpyDeviceToHost));
        double eb = 0.0;
        for (int i = 0; i < nocc; ++i) eb += hw[i];
        *e_band = 2.0 * eb;
        for (int i = 0; i <= nocc; ++i) w[i] = hw[i];
        if (int e = up(&dXp, (const long long*)Xp, ng + 1)) return e;
        if (int e = up(&dXi, (const long long*)Xi, nnzX)) return e;
        if (int e = up(&dXv, Xv, nnzX)) return e;
        LRES_CUDA_TRY(cudaMalloc(&Ct, sizeof(double) * (size_t)std::max<long long>(n * nocc, 1)));
        LRES_CUDA_TRY(cudaMalloc(&dd, sizeof(double) * ng));
        if (nocc) {
            const dim3 tg((unsigned)((n + 31) / 32), (unsigned)((nocc + 31) / 32));
            transpose_occ_kernel<<<tg, dim3(32, 8)>>>(n, nocc, A, Ct);
            LRES_CUDA_TRY(cudaGetLastError());
        }
        ks_density_kernel<<<(unsigned)((ng * 32 + 255) / 256), 256>>>(ng, nocc, dXp, dXi, dXv, Ct, dd);
        LRES_CUDA_TRY(cudaGetLastError());
        LRES_CUDA_TRY(cudaMemcpy(dens, dd, sizeof(double) * ng, cudaMemcpyDeviceToHost));
        return LRES_OK;
    };
    const int rc = run();
    if (h) sv.destroy(h);
    for (void* q : {(void*)dHp, (void*)dHi, (void*)dHv, (void*)dSp, (void*)dSi, (void*)dSv, (void*)dXp, (void*)dXi,
                    (void*)dXv, (void*)A, (void*)B, (void*)W, (void*)work, (void*)Ct, (void*)dd, (void*)info})
        if (q) cudaFree(q);
    return rc;
}

// Grid kernels of the SCF step: a hand-written mixed-radix complex FFT (3-D, FP64),
// FFT Hartree, LDA exchange-correlation, the ion potential and Voronoi ownership.
// All are HBM-bandwidth bound.
//
// FFT: three passes of batched 1-D transforms.  Each CTA loads a pencil of B lines
// (coalesced along the contiguous axis) into shared memory and runs a Stockham
// autosort transform over the factorisation of the line length (radix 4, 2, 3, 5,
// then any remaining prime by a direct DFT), ping-ponging between two shared
// buffers.  Bytes per 3-D transform: 3 passes x (read + write) x 16 B per point.
#include "common.cuh"
#include "lres_internal.h"

#include <vector>

namespace lres {

struct FFT3 {
    int64_t shape[3];
    std::vector<int> fac[3];
    int* d_fac = nullptr;     // [3][16] radices, 0-terminated
};

static std::vector<int> factorise(int n) {
    std::vector<int> f;
    while (n % 4 == 0) { f.push_back(4); n /= 4; }
    while (n % 2 == 0) { f.push_back(2); n /= 2; }
    for (int p = 3; p * p <= n; p += 2)
        while (n % p == 0) { f.push_back(p); n /= p; }
    if (n > 1) f.push_back(n);
    return f;
}

int fft3_create(FFT3** out, const int64_t shape[3]) {
    FFT3* f = new FFT3();
    std::vector<int> flat(48, 0);
    for (int a = 0; a < 3; ++a) {
        f->shape[a] = shape[a];
        f->fac[a] = factorise((int)shape[a]);
        if (f->fac[a].size() > 15 || shape[a] > 4096) {
            delete f;
            lres_set_error("grid axis of length %lld not supported by the FFT", (long long)shape[a]);
            return LRES_EINVAL;
        }
        for (size_t i = 0; i < f->fac[a].size(); ++i) flat[a * 16 + i] = f->fac[a][i];
    }
    if (cudaMalloc(&f->d_fac, sizeof(int) * 48) != cudaSuccess ||
        cudaMemcpy(f->d_fac, flat.data(), sizeof(int) * 48, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(f->d_fac);
        delete f;
        lres_set_error("FFT plan allocation failed");
        return LRES_ENOMEM;
    }
    *out = f;
    return LRES_OK;
}

void fft3_destroy(FFT3* f) {
    if (!f) return;
    cudaFree(f->d_fac);
    delete f;
}

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One pass of 1-D transforms of length L along one axis.  Element t of line (base, b)
// lives at data[base + t*tstride + b*bstride]; the CTA owns lines b in [b0, b0+B).
__global__ void fft_pass_kernel(double2* data, int L, long long tstride, long long bstride, int nb_lines,
                                int lines_per_base, long long base_stride_a, long long base_stride_b, int nbase_b,
                                const int* fac, double sign, int B) {
    extern __shared__ __align__(16) unsigned char smraw[];
    double2* x = reinterpret_cast<double2*>(smraw);      // L x B
    double2* y = x + (size_t)L * B;
    const int tid = threadIdx.x;
    // which lines: blockIdx.x enumerates (base, group of B lines)
    const int groups = (lines_per_base + B - 1) / B;
    const int gidx = blockIdx.x % groups;
    const int base = blockIdx.x / groups;
    const long long off = (long long)(base / nbase_b) * base_stride_a + (long long)(base % nbase_b) * base_stride_b;
    const int b0 = gidx * B;
    const int nbl = min(B, lines_per_base - b0);
    (void)nb_lines;
    // load (contiguous axis fastest)
    if (tstride == 1) {
        for (int idx = tid; idx < L * nbl; idx += blockDim.x) {
            const int t = idx % L, b = idx / L;
            x[t * B + b] = data[off + t + (long long)(b0 + b) * bstride];
        }
    } else {
        for (int idx = tid; idx < L * nbl; idx += blockDim.x) {
            const int b = idx % nbl, t = idx / nbl;
            x[t * B + b] = data[off + (long long)t * tstride + (long long)(b0 + b) * bstride];
        }
    }
    __syncthreads();
    int n = L, s = 1;
    for (int fi = 0; fac[fi]; ++fi) {
        const int r = fac[fi];
        const int m = n / r;
        // butterflies: (p, q, b) with p < m, q < s
        const int nbf = m * s * nbl;
        for (int idx = tid; idx < nbf; idx += blockDim.x) {
            const int b = idx % nbl;
            const int pq = idx / nbl;
            const int q = pq % s, p = pq / s;
            double2 a[16];
            double2 buf[16];
            if (r <= 16) {
                for (int j = 0; j < r; ++j) a[j] = x[(q + s * (p + j * m)) * B + b];
                // small DFT: buf[t] = sum_j a_j exp(sign 2 pi i j t / r)
                if (r == 2) {
                    buf[0] = cadd(a[0], a[1]);
                    buf[1] = make_double2(a[0].x - a[1].x, a[0].y - a[1].y);
                } else if (r == 4) {
                    const double2 t0 = cadd(a[0], a[2]), t1 = make_double2(a[0].x - a[2].x, a[0].y - a[2].y);
                    const double2 t2 = cadd(a[1], a[3]), t3 = make_double2(a[1].x - a[3].x, a[1].y - a[3].y);
                    // multiply t3 by (sign * i)
                    const double2 t3i = make_double2(-sign * t3.y, sign * t3.x);
                    buf[0] = cadd(t0, t2);
                    buf[1] = cadd(t1, t3i);
                    buf[2] = make_double2(t0.x - t2.x, t0.y - t2.y);
                    buf[3] = make_double2(t1.x - t3i.x, t1.y - t3i.y);
                } else {
                    for (int t = 0; t < r; ++t) {
                        double2 acc = make_double2(0.0, 0.0);
                        for (int j = 0; j < r; ++j) {
                            double sn, cs;
                            sincospi(sign * 2.0 * (double)((j * t) % r) / (double)r, &sn, &cs);
                            acc = cadd(acc, cmulc(a[j], make_double2(cs, sn)));
                        }
                        buf[t] = acc;
                    }
                }
                for (int t = 0; t < r; ++t) {
                    double2 v = buf[t];
                    if (p && t) {
                        double sn, cs;
                        sincospi(sign * 2.0 * (double)(p * t) / (double)n, &sn, &cs);
                        v = cmulc(v, make_double2(cs, sn));
                    }
                    y[(q + s * (r * p + t)) * B + b] = v;
                }
            } else {
                // large prime radix: direct DFT from shared memory
                for (int t = 0; t < r; ++t) {
                    double2 acc = make_double2(0.0, 0.0);
                    for (int j = 0; j < r; ++j) {
                        double sn, cs;
                        sincospi(sign * 2.0 * (double)((long long)j * t % r) / (double)r, &sn, &cs);
                        acc = cadd(acc, cmulc(x[(q + s * (p + j * m)) * B + b], make_double2(cs, sn)));
                    }
                    if (p && t) {
                        double sn, cs;
                        sincospi(sign * 2.0 * (double)(p * t) / (double)n, &sn, &cs);
                        acc = cmulc(acc, make_double2(cs, sn));
                    }
                    y[(q + s * (r * p + t)) * B + b] = acc;
                }
            }
        }
        __syncthreads();
        double2* tmp = x;
        x = y;
        y = tmp;
        n = m;
        s *= r;
    }
    // store
    if (tstride == 1) {
        for (int idx = tid; idx < L * nbl; idx += blockDim.x) {
            const int t = idx % L, b = idx / L;
            data[off + t + (long long)(b0 + b) * bstride] = x[t * B + b];
        }
    } else {
        for (int idx = tid; idx < L * nbl; idx += blockDim.x) {
            const int b = idx % nbl, t = idx / nbl;
            data[off + (long long)t * tstride + (long long)(b0 + b) * bstride] = x[t * B + b];
        }
    }
}

int fft3_exec(FFT3* f, double2* data, int inverse, cudaStream_t s) {
    const long long n1 = f->shape[0], n2 = f->shape[1], n3 = f->shape[2];
    const double sign = inverse ? 1.0 : -1.0;
    const int B = 16;
    for (int axis = 2; axis >= 0; --axis) {
        const int L = (int)f->shape[axis];
        long long tstride, bstride, bsa, bsb;
        int lines_per_base, nbase, nbase_b;
        if (axis == 2) {        // lines along k, batched along j; bases = i
            tstride = 1; bstride = n3; lines_per_base = (int)n2; nbase = (int)n1; nbase_b = 1;
            bsa = n2 * n3; bsb = 0;
        } else if (axis == 1) { // lines along j, batched along k; bases = i
            tstride = n3; bstride = 1; lines_per_base = (int)n3; nbase = (int)n1; nbase_b = 1;
            bsa = n2 * n3; bsb = 0;
        } else {                // lines along i, batched along k; bases = j
            tstride = n2 * n3; bstride = 1; lines_per_base = (int)n3; nbase = (int)n2; nbase_b = 1;
            bsa = n3; bsb = 0;
        }
        const int groups = (lines_per_base + B - 1) / B;
        const size_t smem = sizeof(double2) * 2 * (size_t)L * B;
        LRES_CUDA_TRY(cudaFuncSetAttribute(fft_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        fft_pass_kernel<<<nbase * groups, 256, smem, s>>>(data, L, tstride, bstride, lines_per_base * nbase,
                                                        lines_per_base, bsa, bsb, nbase_b, f->d_fac + axis * 16,
                                                        sign, B);
        LRES_CUDA_TRY(cudaGetLastError());
    }
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// wave vectors as numpy: k = 2 pi * (f * (1 / (m * (L / m)))) with f the fftfreq index
// ---------------------------------------------------------------------------
__device__ __forceinline__ double kvec(int i, int m, double L) {
    const int f = (i < (m + 1) / 2) ? i : i - m;
    const double d = L / (double)m;
    const double val = 1.0 / ((double)m * d);
    return 2.0 * M_PI * ((double)f * val);
}

__global__ void real_to_complex(const double* a, double2* b, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = make_double2(a[i], 0.0);
}

__global__ void poisson_kernel(double2* w, int n1, int n2, int n3, double L1, double L2, double L3) {
    const long long n = (long long)n1 * n2 * n3;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx % n3), j = (int)((idx / n3) % n2), i = (int)(idx / ((long long)n2 * n3));
        const double kx = kvec(i, n1, L1), ky = kvec(j, n2, L2), kz = kvec(k, n3, L3);
        const double G2 = kx * kx + ky * ky + kz * kz;
        double2 v = w[idx];
        if (idx == 0) {
            v = make_double2(0.0, 0.0);
        } else {
            const double f = 4.0 * M_PI;
            v = make_double2(f * v.x / G2, f * v.y / G2);
        }
        w[idx] = v;
    }
}

__global__ void complex_real_part(const double2* a, double* b, long long n, double scale) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = a[i].x * scale;
}

int hartree_apply(FFT3* f, const int64_t shape[3], const double cell[3], const double* dens, double* vh,
                  double2* work, cudaStream_t s) {
    const long long n = shape[0] * shape[1] * shape[2];
    real_to_complex<<<1216, 256, 0, s>>>(dens, work, n);
    LRES_CUDA_TRY(cudaGetLastError());
    int rc = fft3_exec(f, work, 0, s);
    if (rc) return rc;
    poisson_kernel<<<1216, 256, 0, s>>>(work, (int)shape[0], (int)shape[1], (int)shape[2], cell[0], cell[1], cell[2]);
    LRES_CUDA_TRY(cudaGetLastError());
    rc = fft3_exec(f, work, 1, s);
    if (rc) return rc;
    complex_real_part<<<1216, 256, 0, s>>>(work, vh, n, 1.0 / (double)n);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// LDA: Slater exchange + Perdew-Zunger 1981 correlation (lrft/three_d.py:132-148)
// ---------------------------------------------------------------------------
__global__ void lda_kernel(const double* dens, double* exc, double* vxc, long long n) {
    const double third = 1.0 / 3.0;
    const double cx = -0.75 * pow(3.0 / M_PI, third);
    const double g = -0.1423, b1 = 1.0529, b2 = 0.3334;
    const double A = 0.0311, Bc = -0.048, C = 0.0020, D = -0.0116;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double nn = fmax(dens[i], 1e-14);
        const double rs = pow(3.0 / (4.0 * M_PI * nn), third);
        const double ex = cx * pow(nn, third);
        const double vx = 4.0 / 3.0 * ex;
        double ec, vc;
        if (rs >= 1.0) {
            const double sr = sqrt(rs);
            const double den = 1.0 + b1 * sr + b2 * rs;
            ec = g / den;
            vc = ec * (1.0 + 7.0 / 6.0 * b1 * sr + 4.0 / 3.0 * b2 * rs) / den;
        } else {
            const double lr = log(rs);
            ec = A * lr + Bc + C * rs * lr + D * rs;
            vc = A * lr + (Bc - A / 3.0) + 2.0 / 3.0 * C * rs * lr + (2.0 * D - C) / 3.0 * rs;
        }
        exc[i] = ex + ec;
        vxc[i] = vx + vc;
    }
}

int lda_apply(long long n, const double* dens, double* exc, double* vxc, cudaStream_t s) {
    lda_kernel<<<1216, 256, 0, s>>>(dens, exc, vxc, n);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// ion potential: v(G) = -4 pi / G^2 * sum_a Z_a exp(-i G.R_a - G^2 rc_a^2 / 4) / vol,
// G = 0 removed, then v(r) = IFFT(v(G)) * ng (lrft/three_d.py:102-112,119)
// ---------------------------------------------------------------------------
__global__ void ion_structure_kernel(double2* w, int n1, int n2, int n3, double L1, double L2, double L3, int natoms,
                                     const double* pos, const double* Z, const double* rc) {
    const long long n = (long long)n1 * n2 * n3;
    const double vol = L1 * L2 * L3;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx % n3), j = (int)((idx / n3) % n2), i = (int)(idx / ((long long)n2 * n3));
        const double kx = kvec(i, n1, L1), ky = kvec(j, n2, L2), kz = kvec(k, n3, L3);
        const double G2 = kx * kx + ky * ky + kz * kz;
        double sx = 0.0, sy = 0.0;
        for (int a = 0; a < natoms; ++a) {
            const double ph = kx * pos[3 * a] + ky * pos[3 * a + 1] + kz * pos[3 * a + 2];
            const double amp = Z[a] * exp(-G2 * rc[a] * rc[a] / 4.0);
            double sn, cs;
            sincos(ph, &sn, &cs);
            sx += amp * cs;
            sy -= amp * sn;
        }
        double2 v;
        if (idx == 0) v = make_double2(0.0, 0.0);
        else {
            const double f = -4.0 * M_PI / G2 / vol;
            v = make_double2(f * sx, f * sy);
        }
        w[idx] = v;
    }
}

int ion_apply(FFT3* f, const int64_t shape[3], const double cell[3], int natoms, const double* pos, const double* Z,
              const double* rc, double* vion, double2* work, cudaStream_t s) {
    const long long n = shape[0] * shape[1] * shape[2];
    ion_structure_kernel<<<1216, 256, 0, s>>>(work, (int)shape[0], (int)shape[1], (int)shape[2], cell[0], cell[1],
                                              cell[2], natoms, pos, Z, rc);
    LRES_CUDA_TRY(cudaGetLastError());
    int r = fft3_exec(f, work, 1, s);
    if (r) return r;
    // ifftn scales by 1/ng and the reference multiplies by ng again
    complex_real_part<<<1216, 256, 0, s>>>(work, vion, n, 1.0);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// Voronoi ownership with the reference's operation order (lrft/lcao3d.py:141-150):
// r = index * dx; dd = (r - c) - L * rint((r - c) / L); d2 = (dd0^2 + dd2^2) + dd1^2
// (numpy's einsum order for 3-vectors); strict '<' keeps the lowest centre index.
// Intrinsics with explicit rounding keep the compiler from fusing multiply-adds.
// ---------------------------------------------------------------------------
__global__ void voronoi_kernel(int n1, int n2, int n3, double dx, double L0, double L1, double L2, int ncent,
                               const double* cen, int* owner) {
    __shared__ double cs[3 * 256];
    const long long n = (long long)n1 * n2 * n3;
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int k = (int)(idx % n3), j = (int)((idx / n3) % n2), i = (int)(idx / ((long long)n2 * n3));
    const double r0 = __dmul_rn((double)i, dx), r1 = __dmul_rn((double)j, dx), r2 = __dmul_rn((double)k, dx);
    double best = INFINITY;
    int who = 0;
    for (int c0 = 0; c0 < ncent; c0 += 256) {
        __syncthreads();
        for (int t = threadIdx.x; t < 3 * 256 && 3 * c0 + t < 3 * ncent; t += blockDim.x) cs[t] = cen[3 * c0 + t];
        __syncthreads();
        const int cend = min(256, ncent - c0);
        if (idx < n) {
            for (int c = 0; c < cend; ++c) {
                double d0 = __dsub_rn(r0, cs[3 * c]), d1 = __dsub_rn(r1, cs[3 * c + 1]), d2 = __dsub_rn(r2, cs[3 * c + 2]);
                d0 = __dsub_rn(d0, __dmul_rn(L0, rint(__ddiv_rn(d0, L0))));
                d1 = __dsub_rn(d1, __dmul_rn(L1, rint(__ddiv_rn(d1, L1))));
                d2 = __dsub_rn(d2, __dmul_rn(L2, rint(__ddiv_rn(d2, L2))));
                const double q = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d2, d2)), __dmul_rn(d1, d1));
                if (q < best) {
                    best = q;
                    who = c0 + c;
                }
            }
        }
    }
    if (idx < n) owner[idx] = who;
}

int voronoi_apply(const int64_t shape[3], const double cell[3], int ncent, const double* centres, int* owner,
                  cudaStream_t s) {
    const long long n = shape[0] * shape[1] * shape[2];
    const double dx = cell[0] / (double)shape[0];
    const int blocks = (int)((n + 255) / 256);
    voronoi_kernel<<<blocks, 256, 0, s>>>((int)shape[0], (int)shape[1], (int)shape[2], dx, cell[0], cell[1], cell[2],
                                          ncent, centres, owner);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

}  // namespace lres

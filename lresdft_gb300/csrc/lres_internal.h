// Internal declarations shared by the translation units of liblres_gb300.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>
#include "../../include/lres_gb300.h"

namespace lres {

// One launch of the fused window LDL^T kernel (window_ldl.cu).
struct LdlJob {
    enum Kind { C128, C64, R64 } kind;
    int nitems = 0;
    const int2* items = nullptr;
    int* counter = nullptr;
    const int* n_w = nullptr;
    const int* m_w = nullptr;
    const long long* offC = nullptr;
    const long long* offF = nullptr;
    const long long* offQ = nullptr;
    const void* C = nullptr;
    const void* B = nullptr;
    const void* F = nullptr;
    const void* shifts = nullptr;
    void* q = nullptr;
    long long qstride = 0;
    double* mult = nullptr;
    int* npos = nullptr;
    int* status = nullptr;
    void* ws = nullptr;
    long long ws_stride = 0;
    int ldp = 0, nmax = 0, mmax = 0;
    int grid = 0;
    size_t smem_budget = 0;
    int config = 0;                 // complex kernels: tile configuration (see lres_tune)
    int keep = 0;                   // complex kernels: keep every item's factor (slot = item index)
    const int* c0 = nullptr;        // per window: the F rows are zero in the columns before c0[w]
};

// Panel width of the factor kept for the adjoint (the window is padded to a multiple).
constexpr int kKeepNB64 = 32, kKeepNB128 = 16;

// Tile configurations of the complex pole kernel, index = LdlJob::config:
//   0: NB 32 (c64) / 16 (c128), 256 threads, k-chunk 32     1: 128 threads
//   2: k-chunk 16                                           3: NB 16 (c64) / 8 (c128)
//   4: c64: chunk products on the tensor cores (tcgen05, 3xTF32); c128: NB 8, 128 threads
//   5: operands of every chunk brought in by bulk asynchronous copies, 128 threads
constexpr int kLeftConfigs = 6;

int run_ldl(const LdlJob& j, cudaStream_t s);
size_t ldl_smem_bytes(int elem_bytes, int nb, int ldp, int mmax);

// Block-sparse (atom-pair) storage of the nb x nb matrices S, T, H.
struct BlockPattern {
    int ngroups = 0;
    int nblk = 0;                     // stored blocks (both triangles)
    int npair = 0;                    // blocks with g <= h (assembled by the H(v) kernel)
    int nfmax = 0;                    // largest group (functions per atom)
    // device arrays
    int* gptr = nullptr;              // [ngroups+1] first function of each group
    int* bptr = nullptr;              // [ngroups+1] blocks of block-row g: [bptr[g], bptr[g+1])
    int* bcol = nullptr;              // [nblk] column group
    int* brow = nullptr;              // [nblk] row group
    long long* boff = nullptr;        // [nblk] value offset (nf_g * nf_h values, row-major)
    int* btrans = nullptr;            // [nblk] index of the transposed block
    int* pair_blk = nullptr;          // [npair] block index of pair p (g <= h)
    long long nval = 0;
};

// Group supports on the grid and common-point lists of overlapping pairs.
struct Supports {
    long long nslot = 0;
    long long* soff = nullptr;        // [ngroups+1] slot range of each group
    int* sgrid = nullptr;             // [nslot] grid index of each slot
    double* sval = nullptr;           // [nslot * 8] basis values, 8 per slot (zero padded)
    float* sval32 = nullptr;          // the same in FP32 (mixed precision only)
    float* vslot = nullptr;           // [nslot] FP32 potential at each slot (mixed H(v) scratch)
    long long ncommon = 0;
    long long* coff = nullptr;        // [npair+1] common-point range of each pair
    int2* cslot = nullptr;            // [ncommon] (slot in g, slot in h)
};

// Kernel launchers implemented in hamiltonian.cu / grid.cu / dense.cu
int pair_common_points(const BlockPattern& bp, Supports& sp, int ngroups, const std::vector<int>& pair_g,
                       const std::vector<int>& pair_h, cudaStream_t s);
int assemble_h(const BlockPattern& bp, const Supports& sp, const double* Tblk, const double* v, double dV,
               double* Hblk, cudaStream_t s);
bool assemble_h32_supported(const BlockPattern& bp);
int assemble_h32(const BlockPattern& bp, const Supports& sp, const double* Tblk, const double* v, double dV,
                 double* Hblk, cudaStream_t s);
// Dense window blocks (column-major, every element written) from the atom-pair blocks; with
// blk32 and dense32, also the FP32 windows from the FP32 copy of the blocks.
int gather_windows(int nwin, int nmax, const int* fn, const long long* fnoff, const int* btab, const long long* btoff,
                   const int* nlg, const long long* offC, const int* n_w, const double* blk, double* dense,
                   const float* blk32, float* dense32, cudaStream_t s);
int build_F(int nwin, const long long* Xp, const int* Xi, const double* Xv, const int* group_of_fn,
            const int* gptr, const int* gloc, int ngroups, const long long* Ooff, const long long* Oflat,
            const long long* offF, const int* m_w, int mmax, double* F, cudaStream_t s);
int batched_gemm(int nwin, const int* n_w, const long long* offA, int nmax, bool transA, const double* A,
                 const double* B, double* C, cudaStream_t s, int klim = 0, bool transB = false);
int batched_gram(int nwin, const int* n_w, const int* m_w, const long long* offF, const long long* offK, int nmax,
                 const double* F, double* K, cudaStream_t s);
int batched_gemm_rect_upper(int nwin, const int* n_w, const int* m_w, const long long* offA, const long long* offU,
                            int nmax, int mmax, const double* A, const double* U, double* C, cudaStream_t s);
int convert_f64_f32(const double* a, float* b, long long n, cudaStream_t s);
int split_f64(const double* a, float2* b, long long n, cudaStream_t s);
int batched_gemm_df64(int nwin, const int* n_w, const long long* off, int nmax, bool transA, int klim,
                      const float2* A, const float2* B, float2* C, float* C32, cudaStream_t s);
// C = A B for every window block: A column-major (FP64 or FP32), B k-major (Bt[j + k n] =
// B[k][j]), C column-major or row-major (c_rowmajor); klim as batched_gemm.
int batched_gemm_f32(int nwin, const int* n_w, const long long* off, int nmax, int klim, const void* A, bool a_f64,
                     const float* Bt, float* C, bool c_rowmajor, cudaStream_t s);
// batched_gemm_f32's products on the tensor cores (tcgen05, 3xTF32, 32-term chunks); a timed-out
// completion wait sets ST_TIMEOUT in *status (device)
int batched_gemm_tc(int nwin, const int* n_w, const long long* off, int nmax, int klim, const void* A, bool a_f64,
                    const float* Bt, float* C, bool c_rowmajor, int* status, cudaStream_t s);
int batched_transpose_f32(int nwin, const int* n_w, const long long* off, int nmax, const float* A, float* B,
                          cudaStream_t s);
int pole_sums(int nwin, const long long* offQ, const int* m_w, const long long* Oflat, bool fp32,
              const void* q, long long qstride, int npoles, const double2* wq, const double2* wzq, double dV,
              double* dens, double* n_w, double* e_w, cudaStream_t s);

// Multi-shift tridiagonal route (tridiag.cu): R = float (fp32) or double.
// Tile configuration of the tridiagonal route for windows of at most nmax functions.
struct TriPick {
    int nb = 0, nt = 0;        // reduction panel width and threads
    int rres = 0;              // 1: the reduction holds each window in shared memory (FP32)
    int nb_apply = 0;          // row application panel width
    int rpt = 1;               // rows per thread of the row-per-thread application; 0: resident rows
    int arows = 0;             // rows per application item
    int ldv = 0;               // shared vector length (multiple of 32, >= nmax)
    long long tstride = 0;     // T-factor elements per window (resident application)
};
int tri_pick(bool fp32, int nmax, size_t smem_budget, int cfg, TriPick* out);
int tri_reduce(bool fp32, int nwin, const int* order, int* counter, const int* n_w, const long long* offC,
               const long long* offA, const long long* offN, const void* H, void* A, void* d, void* e, void* tau,
               int* status, const TriPick& pk, int nmax, size_t smem_budget, cudaStream_t s);
// tfactors: form the T factors of every (window, panel) first (once per Hamiltonian)
int tri_apply(bool fp32, int nitems, const int4* items, const int* n_w, const int* m_w, const long long* offA,
              const long long* offN, const long long* offF, const void* A, const void* tau, const void* F, void* Y,
              const TriPick& pk, int nwin, bool tfactors, void* T, size_t smem_budget, cudaStream_t s);
int tri_rows_per_item(bool fp32, int P);
int tri_pass(bool fp32, int nitems, const int4* items, int* counter, const int* n_w, const int* m_w,
             const long long* offN, const long long* offF, const long long* offQ, const long long* Oflat,
             const void* Y, const void* d, const void* e, int P, const void* shifts, const double2* wq,
             const double2* wzq, double* dens, double* part, int* status, int ldv, size_t smem_budget,
             cudaStream_t s);
int tri_window_sums(int nwin, const int* first, const int* count, const double* part, double dV, double* nw,
                    double* ew, cudaStream_t s);
int tri_sturm(bool fp32, int nwin, const int* n_w, const long long* offN, const void* d, const void* e,
              double sigma, int* below, cudaStream_t s);
int tri_min_eig(bool fp32, int nwin, const int* n_w, const long long* offN, const void* d, const void* e,
                double tol, double* lam, cudaStream_t s);

// Adjoint of the window solve (adjoint.cu)
int adj_backsolve(bool fp32, const int2* items, int nitems, const int* n_w, const int* m_w, void* ws,
                  long long ws_stride, int* status, cudaStream_t s);
int adj_accumulate(bool fp32, const int* wins, int nwin_batch, int P, int nmax, const int* n_w, const int* m_w,
                   const long long* offC, const void* ws, long long ws_stride, const double2* cw, double* A0,
                   double* A1, double* A2, cudaStream_t s);
int adj_weights(int P, int M, double mu, double e_lo, double2* cw, cudaStream_t s);
int adj_inner(int nwin, const int* n_w, const long long* offC, const double* S, const double* A0, const double* A1,
              const double* A2, double* u, cudaStream_t s);
int adj_combine(long long nval, const double* A0, const double* A1, const double* A2, double kappa, double a,
                double b, double* X, double* Y, cudaStream_t s);
int adj_block_gather(const BlockPattern& bp, const long long* eoff, const int4* ent, const int* n_w,
                     const long long* offC, const double* dHW, double* gH, cudaStream_t s);
int adj_point(long long ng, const long long* poff, const int2* pent, const Supports& sp, const BlockPattern& bp,
              const double* gH, double dV, double* dv, cudaStream_t s);

struct FFT3;
int fft3_create(FFT3** out, const int64_t shape[3]);
void fft3_destroy(FFT3* f);
int fft3_exec(FFT3* f, double2* data, int inverse, cudaStream_t s);
int hartree_apply(FFT3* f, const int64_t shape[3], const double cell[3], const double* dens, double* vh,
                  double2* work, cudaStream_t s);
int lda_apply(long long n, const double* dens, double* exc, double* vxc, cudaStream_t s);
int ion_apply(FFT3* f, const int64_t shape[3], const double cell[3], int natoms, const double* pos,
              const double* Z, const double* rc, double* vion, double2* work, cudaStream_t s);
int voronoi_apply(const int64_t shape[3], const double cell[3], int ncent, const double* centres, int* owner,
                  cudaStream_t s);

}  // namespace lres

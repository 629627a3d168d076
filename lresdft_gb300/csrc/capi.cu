// C ABI of liblres_gb300: context set-up, Hamiltonian updates, pole passes,
// inertia counts and the grid kernels of the SCF step.  See include/lres_gb300.h.
#include "common.cuh"
#include "lres_internal.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <complex>
#include <memory>
#include <cstdarg>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

static thread_local char g_err[1024] = "";

extern "C" void lres_set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" const char* lres_last_error(void) { return g_err; }
extern "C" const char* lres_version(void) { return "lres_gb300 0.1 (sm_103a)"; }

using namespace lres;

namespace {

template <class T>
int dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e != cudaSuccess) {
        lres_set_error("cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(e));
        return LRES_ENOMEM;
    }
    return LRES_OK;
}

template <class T>
int upload(T** p, const std::vector<T>& v, cudaStream_t s) {
    int rc = dalloc(p, v.size());
    if (rc) return rc;
    if (!v.empty()) LRES_CUDA_TRY(cudaMemcpyAsync(*p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    return LRES_OK;
}

#define TRY(x)                 \
    do {                       \
        int _rc = (x);         \
        if (_rc) return _rc;   \
    } while (0)

}  // namespace

struct lres_ctx {
    int device = 0, precision = 0, M = 0, npoles = 0;
    int64_t nb = 0, ng = 0, shape[3] = {0, 0, 0};
    double cell[3] = {0, 0, 0}, dV = 0;
    int nwin = 0, ngroups = 0, nmax = 0, mmax = 0, nsm = 0;
    long long npts = 0;
    bool have_T = false, have_h = false;
    int config = 0;                      // tile configuration of the complex pole kernel
    size_t smem_budget = 0;
    // host copies
    std::vector<int> n_w, m_w, gptr_h, order;
    std::vector<long long> offC, offF, offQ;
    // device: windows
    int *d_n = nullptr, *d_m = nullptr;
    int* d_c0 = nullptr;                 // per window: first local column any owned point touches
    bool skip_rows = false;              // owned-point rows start late enough to skip panels
    long long *d_offC = nullptr, *d_offF = nullptr, *d_offQ = nullptr, *d_Oflat = nullptr;
    int *d_wgrp_off = nullptr, *d_wgrp = nullptr, *d_wgrp_lo = nullptr, *d_gloc = nullptr;
    // gather tables: per window function (local atom, function in atom, atom size), per
    // window pair of local atoms the value offset of the stored block (h, g) or -1
    int *d_gfn = nullptr, *d_gbtab = nullptr, *d_gnlg = nullptr;
    long long *d_gfnoff = nullptr, *d_gbtoff = nullptr;
    // block storage
    BlockPattern bp;
    Supports sp;
    double *d_Sblk = nullptr, *d_Tblk = nullptr, *d_Hblk = nullptr;
    float* d_Hblk32 = nullptr;           // FP32 copy of the H blocks (mixed precision)
    bool h32_dense = false;              // the FP32 H_W of the current H sits in the second standard-form slot
    std::vector<int> bptr_h, bcol_h;
    std::vector<long long> boff_h;
    // dense windows
    double *d_SW = nullptr, *d_HW = nullptr, *d_F = nullptr;
    double *d_LinvT = nullptr, *d_Y = nullptr, *d_Hhat = nullptr;
    float2 *d_LinvT_df = nullptr, *d_H_df = nullptr, *d_Y_df = nullptr;   // double-float operands
    float *d_Hhat32 = nullptr, *d_Fhat32 = nullptr;
    float *d_LinvT32 = nullptr, *d_Linv32 = nullptr;   // L^-T and L^-1 in FP32 (mixed tridiagonal route)
    bool hhat_df = false;                // d_Hhat32 holds the double-float transform of the current H_W
    double *d_Fhat64 = nullptr, *d_FhatT64 = nullptr;   // FP64 standard-form rows (FP64 tridiagonal route)
    long long sizeC = 0, sizeF = 0;
    // multi-shift tridiagonal route (tridiag.cu): T = Q^T H^ Q per window once per Hamiltonian,
    // rows Y = F^ Q, then each pass is one fused shifted-solve + pole-sum kernel
    int route = LRES_ROUTE_LDL;
    bool tri_alloc = false, tri_ready = false;
    TriPick tri;                                 // tile configuration (tri_pick)
    int sf_kind = LRES_SF_SIMT;                  // kernel of the FP32 standard form
    int tri_cfg = 0;
    float* d_triT = nullptr;                     // T factors of the resident row application
    long long triT_size = 0;
    std::vector<long long> offN;                 // window vectors (sum of n)
    long long sizeN = 0, sizeA = 0;
    long long* d_offN = nullptr;
    long long* d_offA = nullptr;                 // working blocks: leading dimension n rounded up to 4
    int* d_order_w = nullptr;                    // windows, most expensive first
    int* d_tstatus = nullptr;                    // status of the reduction (kept across passes)
    void *d_triA = nullptr, *d_trid = nullptr, *d_trie = nullptr, *d_tritau = nullptr;
    void *d_Yown = nullptr, *d_Ytr = nullptr;
    double* d_lam = nullptr;                     // per-window smallest eigenvalue
    struct RowItems {                            // work items over the rows of every window
        int4* apply = nullptr;                   // (window, first row, rows <= rows per application item)
        int arows = 0;                           // rows per application item the items were built for
        int napply = 0;
        int4* pass = nullptr;                    // (window, first row, rows <= rows per pass item)
        int npass = 0;
        int *first = nullptr, *count = nullptr;  // pass items of each window (contiguous)
        double* part = nullptr;                  // per pass item: sums of n(r), e(r)
        void release() {
            for (void* q : {(void*)apply, (void*)pass, (void*)first, (void*)count, (void*)part})
                if (q) cudaFree(q);
            *this = RowItems{};
        }
    };
    RowItems ri_own, ri_tr;
    // pole work
    int2 *d_items = nullptr, *d_items_win = nullptr, *d_items_sub = nullptr;
    int nitems = 0;
    int *d_counter = nullptr, *d_status = nullptr, *d_npos = nullptr;
    void* d_ws = nullptr;
    size_t ws_bytes = 0;
    void* d_shifts = nullptr;
    double2 *d_wq = nullptr, *d_wzq = nullptr;
    void* d_q = nullptr;
    double *d_dens = nullptr, *d_nw = nullptr, *d_ew = nullptr, *d_v = nullptr;
    std::vector<double> nw_h, ew_h;
    // trace rows: r_w x n_w factors R_W with R_W^T R_W = F_W^T F_W, used by passes that need
    // N and E_band only (no density) and by the adjoint
    bool have_trace = false;
    int mmaxT = 0;
    long long nptsT = 0, sizeFT = 0;
    int *d_mT = nullptr;
    long long *d_offFT = nullptr, *d_offQT = nullptr;
    double* d_FT = nullptr;
    float* d_FhatT32 = nullptr;
    void* d_qT = nullptr;
    // host copies kept for the adjoint's inverse maps
    std::vector<long long> soff_h;
    std::vector<int> sgrid_h, wgrp_off_h, wgrp_h, wgrp_lo_h, gloc_h;
    // adjoint (allocated on first use)
    bool adj_ready = false;
    double *d_adjA[3] = {nullptr, nullptr, nullptr}, *d_dHW = nullptr, *d_dSW = nullptr, *d_gH = nullptr;
    double *d_adjdv = nullptr, *d_adju = nullptr;
    double2* d_cw = nullptr;
    int* d_order = nullptr;
    long long *d_eoff = nullptr, *d_poff = nullptr;
    int4* d_ent = nullptr;
    int2* d_pent = nullptr;
    void* d_adjws = nullptr;
    size_t adjws_bytes = 0;
    std::vector<double> adju_h;
    // grid
    FFT3* fft = nullptr;
    double2* d_fftwork = nullptr;
    // CUDA events bracketing the launches, for lres_timings: pairs (begin, end) of
    // 0 pole kernel, 1 pole sums, 2 H(v) assembly, 3 window gather, 4 standard-form transform, 5 inertia kernel
    // 6 tridiagonal reduction, 7 rows through the reflectors
    cudaEvent_t ev[16] = {};
    bool ev_used[8] = {};
    ~lres_ctx();
};

lres_ctx::~lres_ctx() {
    void* ptrs[] = {d_n, d_m, d_c0, d_offC, d_offF, d_offQ, d_Oflat, d_wgrp_off, d_wgrp, d_wgrp_lo, d_gloc,
                    d_gfn, d_gbtab, d_gnlg, d_gfnoff, d_gbtoff,
                    bp.gptr, bp.bptr, bp.bcol, bp.brow, bp.boff, bp.btrans, bp.pair_blk, sp.soff, sp.sgrid,
                    sp.sval, sp.sval32, sp.vslot, sp.coff, sp.cslot, d_Sblk, d_Tblk, d_Hblk, d_Hblk32, d_SW, d_HW, d_F, d_LinvT, d_Y, d_Hhat,
                    d_Hhat32, d_Fhat32, d_LinvT_df, d_H_df, d_Y_df, d_items, d_items_win, d_items_sub, d_counter, d_status, d_npos, d_ws, d_shifts,
                    d_wq, d_wzq, d_q, d_dens, d_nw, d_ew, d_v, d_fftwork, d_adjA[0], d_adjA[1], d_adjA[2],
                    d_dHW, d_dSW, d_gH, d_adjdv, d_adju, d_cw, d_order, d_eoff, d_poff, d_ent, d_pent, d_adjws,
                    d_mT, d_offFT, d_offQT, d_FT, d_FhatT32, d_qT, d_Fhat64, d_FhatT64, d_offN, d_offA, d_order_w, d_LinvT32, d_Linv32,
                    d_tstatus, d_triA, d_trid, d_trie, d_tritau, d_Yown, d_Ytr, d_lam, d_triT};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    ri_own.release();
    ri_tr.release();
    if (fft) fft3_destroy(fft);
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
}

namespace {

// Runs the fused LDL^T kernel over `items` (device) with the given operands.
int ldl_launch(lres_ctx* c, LdlJob::Kind kind, int nitems, const int2* items, const void* C, const void* B,
               const void* F, const int* m_w, const long long* offF, const void* shifts, void* q, double* mult,
               int ldp, int mmax, cudaStream_t s, const long long* offQ = nullptr, long long qstride = -1) {
    LdlJob j{};
    j.kind = kind;
    j.nitems = nitems;
    j.items = items;
    j.counter = c->d_counter;
    j.n_w = c->d_n;
    j.m_w = m_w;
    j.offC = c->d_offC;
    j.offF = offF;
    j.offQ = offQ ? offQ : c->d_offQ;
    j.C = C;
    j.B = B;
    j.F = F;
    j.shifts = shifts;
    j.q = q;
    j.qstride = qstride >= 0 ? qstride : c->npts;
    j.mult = mult;
    j.npos = c->d_npos;
    j.status = c->d_status;
    j.ldp = ldp;
    j.nmax = c->nmax;
    j.mmax = mmax;
    const size_t el = kind == LdlJob::C128 ? 16 : 8;
    // one workspace slot per resident CTA (complex: up to 4 per SM), never more than items;
    // slots start 16-byte aligned (bulk copies) and hold (n_pad + m + 1) x n_pad complex
    const int slots = std::max(1, std::min(nitems, kind == LdlJob::R64 ? c->nsm : 4 * c->nsm));
    const long long nmaxp = (c->nmax + 31) / 32 * 32;   // padded window dimension (complex kernel)
    const long long need = kind == LdlJob::R64 ? (long long)ldp * c->nmax : (nmaxp + mmax + 1) * nmaxp;
    j.ws_stride = (need + 15) / 16 * 16;
    const size_t bytes = (size_t)j.ws_stride * el * slots;
    if (bytes > c->ws_bytes) {            // grows on demand (an eager call precedes any capture)
        if (c->d_ws) cudaFree(c->d_ws);
        c->d_ws = nullptr;
        c->ws_bytes = 0;
        TRY(dalloc((char**)&c->d_ws, bytes));
        c->ws_bytes = bytes;
    }
    j.ws = c->d_ws;
    j.grid = slots;
    j.smem_budget = c->smem_budget;
    j.config = c->config;
    j.c0 = (kind == LdlJob::R64 || !c->skip_rows) ? nullptr : c->d_c0;
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_counter, 0, sizeof(int), s));
    return run_ldl(j, s);
}

// The owned-row set of a pass: the grid's owned points (density) or the trace rows.
struct Rows {
    const int* m;
    const long long *offF, *offQ, *Oflat;
    const void* F;            // FP64 rows (LRES_FP64) or standard-form FP32 rows (LRES_MIXED)
    void* q;
    long long npts;
    int mmax;
    double* dens;
};

Rows select_rows(lres_ctx* c, bool trace) {
    const bool mixed = c->precision == LRES_MIXED;
    if (trace)
        return Rows{c->d_mT, c->d_offFT, c->d_offQT, nullptr,
                    mixed ? (const void*)c->d_FhatT32 : (const void*)c->d_FT, c->d_qT, c->nptsT, c->mmaxT, nullptr};
    return Rows{c->d_m, c->d_offF, c->d_offQ, c->d_Oflat,
                mixed ? (const void*)c->d_Fhat32 : (const void*)c->d_F, c->d_q, c->npts, c->mmax, c->d_dens};
}

int read_status(lres_ctx* c, cudaStream_t s, int* st) {
    LRES_CUDA_TRY(cudaMemcpyAsync(st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    return LRES_OK;
}

// Status of the last pass: its kernels, and on the tridiagonal route the reduction of the
// current Hamiltonian.
int read_pass_status(lres_ctx* c, cudaStream_t s, int* st) {
    int v[2] = {0, 0};
    LRES_CUDA_TRY(cudaMemcpyAsync(&v[0], c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (c->route == LRES_ROUTE_TRIDIAG && c->d_tstatus)
        LRES_CUDA_TRY(cudaMemcpyAsync(&v[1], c->d_tstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    *st = v[0] | v[1];
    return LRES_OK;
}

__global__ void identity_kernel(const int* n_w, const long long* off, double* I, int nwin) {
    const int w = blockIdx.x;
    if (w >= nwin) return;
    const int n = n_w[w];
    double* D = I + off[w];
    for (int i = threadIdx.x; i < n; i += blockDim.x) D[i + (long long)i * n] = 1.0;
}

// Pole nodes and weights on the device (a capturable pass takes mu, e_lo by value):
// z_k = c + R e^{i pi (2k+1)/M}, w_k = R e^{i pi (2k+1)/M} / M  (lrft/core.py:130-139)
__global__ void poles_kernel(int P, int M, double mu, double e_lo, int fp32, void* shifts, double2* wq, double2* wzq) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P) return;
    const double cc = 0.5 * (mu + e_lo), R = 0.5 * (mu - e_lo);
    double sn, cs;
    sincospi((double)(2 * k + 1) / (double)M, &sn, &cs);
    const double zr = cc + R * cs, zi = R * sn;
    const double wr = R * cs / M, wi = R * sn / M;
    if (fp32) reinterpret_cast<float2*>(shifts)[k] = make_float2((float)zr, (float)zi);
    else reinterpret_cast<double2*>(shifts)[k] = make_double2(zr, zi);
    wq[k] = make_double2(wr, wi);
    wzq[k] = make_double2(wr * zr - wi * zi, wr * zi + wi * zr);
}

// N and E_band from the per-window sums, fixed order (one thread).
__global__ void window_total_kernel(int nwin, const double* nw, const double* ew, double* out) {
    if (blockIdx.x || threadIdx.x) return;
    double N = 0.0, E = 0.0;
    for (int w = 0; w < nwin; ++w) {
        N += nw[w];
        E += ew[w];
    }
    out[0] = N;
    out[1] = E;
}

// H^_W = L^-1 H_W L^-T with LinvT = L^-T (upper triangular) stored column-major:
// Y = H LinvT (k <= column), then the lower triangle of H^ = LinvT^T Y (k <= row).

// Double-float arithmetic on the FP32 pipes, H^ rounded to FP32 at the end (the mixed LDL^T
// route and the mixed adjoint, whose FP32 factorisations are more accurate than FP32 input).
int transform_df64(lres_ctx* c, cudaStream_t s) {
    TRY(split_f64(c->d_HW, c->d_H_df, c->sizeC, s));
    TRY(batched_gemm_df64(c->nwin, c->d_n, c->d_offC, c->nmax, false, 1, c->d_H_df, c->d_LinvT_df, c->d_Y_df,
                          nullptr, s));
    TRY(batched_gemm_df64(c->nwin, c->d_n, c->d_offC, c->nmax, true, 2, c->d_LinvT_df, c->d_Y_df, nullptr,
                          c->d_Hhat32, s));
    c->hhat_df = true;
    return LRES_OK;
}

// Standard form of the mixed tridiagonal route: FP32 with blocked sums (measured as accurate
// as the double-float form there, whose FP32 Householder reduction sets the error).  Both
// products live in the double-float scratch: Y in its first sizeC floats, H^ in the next.
float* tri_hhat32(lres_ctx* c) { return reinterpret_cast<float*>(c->d_Y_df) + c->sizeC; }

int transform_f32(lres_ctx* c, cudaStream_t s) {
    // Y = H L^-T (B = L^-T given k-major: its transpose L^-1), written row-major (k-major for
    // the next product); A^ = lower(L^-1 Y)
    float* Y = reinterpret_cast<float*>(c->d_Y_df);
    const bool h32 = c->h32_dense;       // consumed here, whatever the outcome
    c->h32_dense = false;
    if (c->sf_kind == LRES_SF_TENSOR && c->d_tstatus) {
        TRY(batched_gemm_tc(c->nwin, c->d_n, c->d_offC, c->nmax, 1, c->d_HW, true, c->d_Linv32, Y, true, c->d_tstatus,
                            s));
        TRY(batched_gemm_tc(c->nwin, c->d_n, c->d_offC, c->nmax, 2, c->d_Linv32, false, Y, tri_hhat32(c), false,
                            c->d_tstatus, s));
    } else if (h32) {
        TRY(batched_gemm_f32(c->nwin, c->d_n, c->d_offC, c->nmax, 1, tri_hhat32(c), false, c->d_Linv32, Y, true, s));
        TRY(batched_gemm_f32(c->nwin, c->d_n, c->d_offC, c->nmax, 2, c->d_Linv32, false, Y, tri_hhat32(c), false, s));
    } else {
        TRY(batched_gemm_f32(c->nwin, c->d_n, c->d_offC, c->nmax, 1, c->d_HW, true, c->d_Linv32, Y, true, s));
        TRY(batched_gemm_f32(c->nwin, c->d_n, c->d_offC, c->nmax, 2, c->d_Linv32, false, Y, tri_hhat32(c), false, s));
    }
    c->hhat_df = false;                  // d_Hhat32 no longer follows H_W
    return LRES_OK;
}

// FP64 (the FP64 tridiagonal route); the product H LinvT lives in the working blocks of the
// reduction (at least sizeC elements), which the reduction overwrites afterwards.
int transform_fp64(lres_ctx* c, cudaStream_t s) {
    double* Y = static_cast<double*>(c->d_triA);
    if (!Y || c->sizeA < c->sizeC) {
        lres_set_error("FP64 standard form without the tridiagonal buffers");
        return LRES_ESTATE;
    }
    TRY(batched_gemm(c->nwin, c->d_n, c->d_offC, c->nmax, false, c->d_HW, c->d_LinvT, Y, s, 1));
    TRY(batched_gemm(c->nwin, c->d_n, c->d_offC, c->nmax, true, c->d_LinvT, Y, c->d_Hhat, s, 2));
    return LRES_OK;
}

int window_transform(lres_ctx* c, cudaStream_t s) {
    if (c->precision == LRES_MIXED)
        return c->route == LRES_ROUTE_TRIDIAG ? transform_f32(c, s) : transform_df64(c, s);
    return transform_fp64(c, s);
}

// The double-float standard form for the LDL^T consumers (passes on that route, the adjoint).
int ensure_hhat_df(lres_ctx* c, cudaStream_t s) {
    if (c->precision == LRES_MIXED && !c->hhat_df) return transform_df64(c, s);
    return LRES_OK;
}

// The standard form is used by the mixed path (both routes) and by the FP64 tridiagonal route.
bool needs_standard_form(const lres_ctx* c) {
    return c->precision == LRES_MIXED || c->route == LRES_ROUTE_TRIDIAG;
}

int mark(lres_ctx* c, int which, int end, cudaStream_t s) {
    // a stream being captured into a graph records no timing events
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    LRES_CUDA_TRY(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return LRES_OK;
    LRES_CUDA_TRY(cudaEventRecord(c->ev[2 * which + end], s));
    c->ev_used[which] = true;
    return LRES_OK;
}

int tri_prepare(lres_ctx* c, cudaStream_t s);

int after_h_blocks(lres_ctx* c, cudaStream_t s) {
    TRY(mark(c, 3, 0, s));
    // the FP32 standard form on the SIMT pipes reads FP32 windows, gathered beside the FP64 ones
    // from FP32 blocks into the slot its second product overwrites
    const bool h32 = c->precision == LRES_MIXED && c->route == LRES_ROUTE_TRIDIAG && c->sf_kind == LRES_SF_SIMT &&
                     c->d_Hblk32 && c->d_Y_df;
    if (h32) TRY(convert_f64_f32(c->d_Hblk, c->d_Hblk32, c->bp.nval, s));
    TRY(gather_windows(c->nwin, c->nmax, c->d_gfn, c->d_gfnoff, c->d_gbtab, c->d_gbtoff, c->d_gnlg, c->d_offC,
                       c->d_n, c->d_Hblk, c->d_HW, h32 ? c->d_Hblk32 : nullptr, h32 ? tri_hhat32(c) : nullptr, s));
    c->h32_dense = h32;
    TRY(mark(c, 3, 1, s));
    if (needs_standard_form(c)) {
        TRY(mark(c, 4, 0, s));
        TRY(window_transform(c, s));
        TRY(mark(c, 4, 1, s));
    }
    if (c->route == LRES_ROUTE_TRIDIAG) TRY(tri_prepare(c, s));
    c->have_h = true;
    return LRES_OK;
}

// Trace rows in the standard form: R^ = R L^-T (FP32 for the mixed path, FP64 otherwise).
int trace_standard_form(lres_ctx* c, cudaStream_t s) {
    const bool mixed = c->precision == LRES_MIXED;
    double* out = mixed ? nullptr : c->d_FhatT64;
    double* tmp = nullptr;
    if (mixed) TRY(dalloc(&tmp, c->sizeFT));
    int rc = batched_gemm_rect_upper(c->nwin, c->d_n, c->d_mT, c->d_offFT, c->d_offC, c->nmax, c->mmaxT, c->d_FT,
                                     c->d_LinvT, mixed ? tmp : out, s);
    if (!rc && mixed) rc = convert_f64_f32(tmp, c->d_FhatT32, c->sizeFT, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (tmp) cudaFree(tmp);
    if (rc) return rc;
    LRES_CUDA_TRY(e);
    return LRES_OK;
}

// Every window overlap S_W positive definite: all n_w pivots of its LDL^T positive (the
// factorisation that filled d_npos, one item per window).  The reference's dsygvx reports the
// same failure as info > n (src/lrft_cpp.cpp:94,110).
int check_positive_pivots(lres_ctx* c, cudaStream_t s) {
    std::vector<int> npos(c->nwin);
    LRES_CUDA_TRY(cudaMemcpyAsync(npos.data(), c->d_npos, sizeof(int) * c->nwin, cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    for (int w = 0; w < c->nwin; ++w)
        if (npos[w] != c->n_w[w]) {
            lres_set_error("overlap S_W of window %d is not positive definite (%d of %d pivots positive)", w,
                           npos[w], c->n_w[w]);
            return LRES_ENUMERIC;
        }
    return LRES_OK;
}

// Positive definiteness of the current S_W alone (the FP64 LDL^T route has no standard form).
int check_overlaps(lres_ctx* c, cudaStream_t s) {
    double* one = nullptr;
    TRY(dalloc(&one, 1));
    const double h_one = 1.0;
    int rc = LRES_OK;
    cudaError_t e = cudaMemcpyAsync(one, &h_one, sizeof(double), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = LRES_ECUDA;
    if (!rc) rc = ldl_launch(c, LdlJob::R64, c->nwin, c->d_items_win, nullptr, c->d_SW, nullptr, c->d_m, c->d_offF,
                             one, nullptr, nullptr, c->nmax, 0, s);
    if (!rc) rc = check_positive_pivots(c, s);
    cudaFree(one);
    return rc;
}

// Standard form from the current S_W: L_c^-1 (stored as L^-T in FP64; for the mixed path also
// as double-float pairs) and F^ = L_c^-1 F (FP32 for the mixed path, FP64 for the FP64
// tridiagonal route).  Allocates on the first call.
int setup_standard_form(lres_ctx* c, cudaStream_t s) {
    const bool mixed = c->precision == LRES_MIXED;
    if (!c->d_LinvT) {
        TRY(dalloc(&c->d_LinvT, c->sizeC));
        if (mixed) {
            TRY(dalloc(&c->d_LinvT_df, c->sizeC));
            TRY(dalloc(&c->d_H_df, c->sizeC));
            TRY(dalloc(&c->d_Y_df, c->sizeC));
            TRY(dalloc(&c->d_Hhat32, c->sizeC));
            TRY(dalloc(&c->d_Fhat32, c->sizeF));
            TRY(dalloc(&c->d_LinvT32, c->sizeC));
            TRY(dalloc(&c->d_Linv32, c->sizeC));
        } else {
            TRY(dalloc(&c->d_Hhat, c->sizeC));
            TRY(dalloc(&c->d_Fhat64, c->sizeF));
        }
    }
    if (!mixed && c->have_trace && !c->d_FhatT64) TRY(dalloc(&c->d_FhatT64, c->sizeFT));
    double* I = nullptr;
    double* Fhat = nullptr;
    double* one = nullptr;
    TRY(dalloc(&I, c->sizeC));
    if (mixed) TRY(dalloc(&Fhat, c->sizeF));
    TRY(dalloc(&one, 1));
    const double h_one = 1.0;
    LRES_CUDA_TRY(cudaMemcpyAsync(one, &h_one, sizeof(double), cudaMemcpyHostToDevice, s));
    LRES_CUDA_TRY(cudaMemsetAsync(I, 0, sizeof(double) * c->sizeC, s));
    identity_kernel<<<c->nwin, 128, 0, s>>>(c->d_n, c->d_offC, I, c->nwin);
    LRES_CUDA_TRY(cudaGetLastError());
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
    // A = 1*S - 0 with identity rows: multipliers sqrt(D) D^-1 L^-1 e_r = (L_c^-1)_{:,r}
    int rc = ldl_launch(c, LdlJob::R64, c->nwin, c->d_items_win, nullptr, c->d_SW, I, c->d_n, c->d_offC, one,
                        nullptr, c->d_LinvT, 2 * c->nmax, c->nmax, s);
    // F^ = F L^-T (owned-point rows in the standard form), any number of rows
    if (!rc)
        rc = batched_gemm_rect_upper(c->nwin, c->d_n, c->d_m, c->d_offF, c->d_offC, c->nmax, c->mmax, c->d_F,
                                     c->d_LinvT, mixed ? Fhat : c->d_Fhat64, s);
    if (!rc && mixed) rc = convert_f64_f32(Fhat, c->d_Fhat32, c->sizeF, s);
    if (!rc && c->have_trace) rc = trace_standard_form(c, s);
    if (!rc && mixed) rc = split_f64(c->d_LinvT, c->d_LinvT_df, c->sizeC, s);
    if (!rc && mixed) rc = convert_f64_f32(c->d_LinvT, c->d_LinvT32, c->sizeC, s);
    if (!rc && mixed) rc = batched_transpose_f32(c->nwin, c->d_n, c->d_offC, c->nmax, c->d_LinvT32, c->d_Linv32, s);
    c->hhat_df = false;                  // the standard form changed
    int st = 0;
    if (!rc) rc = read_status(c, s, &st);
    cudaFree(I);
    if (Fhat) cudaFree(Fhat);
    cudaFree(one);
    if (rc) return rc;
    if (st) {
        lres_set_error("Cholesky of a window overlap S_W failed (status %d)", st);
        return LRES_ENUMERIC;
    }
    return check_positive_pivots(c, s);
}

// Work items over the rows of every window, windows in the order of c->order (most
// expensive first): blocks of the application's rows per item for the reflector application,
// batches of the pass kernel's rows per item for the pole passes (each window's batches
// contiguous).
int build_row_items(lres_ctx* c, const std::vector<int>& m, lres_ctx::RowItems& ri, cudaStream_t s) {
    ri.release();
    const int rb = tri_rows_per_item(c->precision == LRES_MIXED, c->npoles);
    const int ar = c->tri.arows;
    std::vector<int4> ap, pa;
    std::vector<int> first(c->nwin, 0), count(c->nwin, 0);
    for (int w : c->order) {
        for (int r0 = 0; r0 < m[w]; r0 += ar) ap.push_back(make_int4(w, r0, std::min(ar, m[w] - r0), 0));
        first[w] = (int)pa.size();
        for (int r0 = 0; r0 < m[w]; r0 += rb) pa.push_back(make_int4(w, r0, std::min(rb, m[w] - r0), 0));
        count[w] = (int)pa.size() - first[w];
    }
    ri.napply = (int)ap.size();
    ri.arows = ar;
    ri.npass = (int)pa.size();
    TRY(upload(&ri.apply, ap, s));
    TRY(upload(&ri.pass, pa, s));
    TRY(upload(&ri.first, first, s));
    TRY(upload(&ri.count, count, s));
    TRY(dalloc(&ri.part, 2 * (size_t)std::max(ri.npass, 1)));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));     // the host vectors go out of scope
    return LRES_OK;
}

// T-factor buffer of the resident row application (grown on a configuration change).
int ensure_tfactors(lres_ctx* c) {
    const long long need = (long long)c->nwin * c->tri.tstride;
    if (need <= c->triT_size) return LRES_OK;
    if (c->d_triT) cudaFree(c->d_triT);
    c->d_triT = nullptr;
    c->triT_size = 0;
    TRY(dalloc(&c->d_triT, need));
    c->triT_size = need;
    return LRES_OK;
}

// Buffers of the tridiagonal route (once per context).
int tri_setup(lres_ctx* c, cudaStream_t s) {
    if (c->tri_alloc) return LRES_OK;
    const bool fp32 = c->precision == LRES_MIXED;
    const size_t el = fp32 ? sizeof(float) : sizeof(double);
    TRY(tri_pick(fp32, c->nmax, c->smem_budget, c->tri_cfg, &c->tri));
    TRY(ensure_tfactors(c));
    TRY(dalloc((char**)&c->d_triA, el * (size_t)c->sizeA));
    TRY(dalloc((char**)&c->d_trid, el * (size_t)c->sizeN));
    TRY(dalloc((char**)&c->d_trie, el * (size_t)c->sizeN));
    TRY(dalloc((char**)&c->d_tritau, el * (size_t)c->sizeN));
    TRY(dalloc((char**)&c->d_Yown, el * (size_t)std::max<long long>(c->sizeF, 1)));
    TRY(dalloc(&c->d_lam, c->nwin));
    TRY(dalloc(&c->d_tstatus, 1));
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_tstatus, 0, sizeof(int), s));
    TRY(build_row_items(c, c->m_w, c->ri_own, s));
    if (c->have_trace) {
        std::vector<int> mT(c->nwin);
        LRES_CUDA_TRY(cudaMemcpy(mT.data(), c->d_mT, sizeof(int) * c->nwin, cudaMemcpyDeviceToHost));
        TRY(build_row_items(c, mT, c->ri_tr, s));
        TRY(dalloc((char**)&c->d_Ytr, el * (size_t)std::max<long long>(c->sizeFT, 1)));
    }
    c->tri_alloc = true;
    return LRES_OK;
}

// Rows of one row set (owned points or trace rows) through the reflectors.
int tri_rows(lres_ctx* c, bool trace, cudaStream_t s) {
    const bool fp32 = c->precision == LRES_MIXED;
    const lres_ctx::RowItems& ri = trace ? c->ri_tr : c->ri_own;
    const void* F = trace ? (fp32 ? (const void*)c->d_FhatT32 : (const void*)c->d_FhatT64)
                          : (fp32 ? (const void*)c->d_Fhat32 : (const void*)c->d_Fhat64);
    // the T factors depend on the reflectors only: formed with the owned rows
    return tri_apply(fp32, ri.napply, ri.apply, c->d_n, trace ? c->d_mT : c->d_m, c->d_offA, c->d_offN,
                     trace ? c->d_offFT : c->d_offF, c->d_triA, c->d_tritau, F, trace ? c->d_Ytr : c->d_Yown,
                     c->tri, c->nwin, !trace, c->d_triT, c->smem_budget, s);
}

// Tridiagonal form of the current standard-form windows and the rows through its reflectors
// (kernels and memsets only).
int tri_prepare(lres_ctx* c, cudaStream_t s) {
    const bool fp32 = c->precision == LRES_MIXED;
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_tstatus, 0, sizeof(int), s));
    TRY(mark(c, 6, 0, s));
    TRY(tri_reduce(fp32, c->nwin, c->d_order_w, c->d_counter, c->d_n, c->d_offC, c->d_offA, c->d_offN,
                   fp32 ? (const void*)tri_hhat32(c) : (const void*)c->d_Hhat, c->d_triA, c->d_trid, c->d_trie,
                   c->d_tritau, c->d_tstatus, c->tri, c->nmax, c->smem_budget, s));
    TRY(mark(c, 6, 1, s));
    TRY(mark(c, 7, 0, s));
    TRY(tri_rows(c, false, s));
    if (c->have_trace) TRY(tri_rows(c, true, s));
    TRY(mark(c, 7, 1, s));
    c->tri_ready = true;
    return LRES_OK;
}

// Standard form and tridiagonal form of the current H_W (when the route was switched after it
// was set).
int tri_refresh(lres_ctx* c, cudaStream_t s) {
    TRY(window_transform(c, s));
    return tri_prepare(c, s);
}

// The pole pass of the tridiagonal route over one row set (nodes and weights already set):
// per-window N and E_band into d_nw / d_ew, the density into d_dens for the owned points.
int tri_run_pass(lres_ctx* c, bool trace, cudaStream_t s) {
    const bool fp32 = c->precision == LRES_MIXED;
    const lres_ctx::RowItems& ri = trace ? c->ri_tr : c->ri_own;
    TRY(mark(c, 0, 0, s));
    TRY(tri_pass(fp32, ri.npass, ri.pass, c->d_counter, c->d_n, trace ? c->d_mT : c->d_m, c->d_offN,
                 trace ? c->d_offFT : c->d_offF, trace ? c->d_offQT : c->d_offQ, trace ? nullptr : c->d_Oflat,
                 trace ? c->d_Ytr : c->d_Yown, c->d_trid, c->d_trie, c->npoles, c->d_shifts, c->d_wq, c->d_wzq,
                 trace ? nullptr : c->d_dens, ri.part, c->d_status, c->tri.ldv, c->smem_budget, s));
    TRY(mark(c, 0, 1, s));
    TRY(mark(c, 1, 0, s));
    TRY(tri_window_sums(c->nwin, ri.first, ri.count, ri.part, c->dV, c->d_nw, c->d_ew, s));
    TRY(mark(c, 1, 1, s));
    return LRES_OK;
}

int find_block(const std::vector<int>& bptr, const std::vector<int>& bcol, int g, int h) {
    auto b0 = bcol.begin() + bptr[g], b1 = bcol.begin() + bptr[g + 1];
    auto it = std::lower_bound(b0, b1, h);
    if (it == b1 || *it != h) return -1;
    return (int)(it - bcol.begin());
}

int scatter_csr(const lres_ctx* c, const std::vector<int>& group_of_fn, const int64_t* Ap, const int64_t* Ai,
                const double* Av, std::vector<double>& blk) {
    blk.assign(c->bp.nval, 0.0);
    for (int64_t a = 0; a < c->nb; ++a) {
        const int g = group_of_fn[a];
        const int fa = (int)(a - c->gptr_h[g]);
        for (int64_t p = Ap[a]; p < Ap[a + 1]; ++p) {
            const int64_t b = Ai[p];
            if (b < 0 || b >= c->nb) {
                lres_set_error("CSR column index %lld out of range", (long long)b);
                return LRES_EINVAL;
            }
            const int h = group_of_fn[b];
            const int blkid = find_block(c->bptr_h, c->bcol_h, g, h);
            if (blkid < 0) {
                lres_set_error("CSR entry (%lld,%lld) outside the atom-pair pattern", (long long)a, (long long)b);
                return LRES_EINVAL;
            }
            const int nfh = c->gptr_h[h + 1] - c->gptr_h[h];
            blk[c->boff_h[blkid] + fa * nfh + (b - c->gptr_h[h])] = Av[p];
        }
    }
    return LRES_OK;
}

}  // namespace

extern "C" int lres_ctx_create(lres_ctx** out, const lres_system_desc* d, int precision, int M, void* stream) {
    if (!out || !d) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    *out = nullptr;
    if (precision != LRES_FP64 && precision != LRES_MIXED) {
        lres_set_error("precision must be LRES_FP64 or LRES_MIXED");
        return LRES_EINVAL;
    }
    if (M < 2 || M % 2) {
        lres_set_error("M must be even and >= 2 (got %d)", M);
        return LRES_EINVAL;
    }
    if (!d->Xp || !d->Xi || !d->Xv || !d->Sp || !d->Si || !d->Sv || !d->gptr || !d->Wflat || !d->Woff ||
        !d->Oflat || !d->Ooff || d->nb <= 0 || d->ngroups <= 0 || d->nwin <= 0) {
        lres_set_error("incomplete system description");
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    auto c = std::make_unique<lres_ctx>();
    LRES_CUDA_TRY(cudaGetDevice(&c->device));
    LRES_CUDA_TRY(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device));
    int optin = 0;
    LRES_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    c->smem_budget = (size_t)optin - 1024;
    for (cudaEvent_t& e : c->ev) LRES_CUDA_TRY(cudaEventCreate(&e));
    c->precision = precision;
    c->M = M;
    c->npoles = M / 2;
    c->nb = d->nb;
    for (int i = 0; i < 3; ++i) {
        c->shape[i] = d->shape[i];
        c->cell[i] = d->cell[i];
    }
    c->ng = d->shape[0] * d->shape[1] * d->shape[2];
    c->dV = d->dV;
    c->nwin = (int)d->nwin;
    c->ngroups = (int)d->ngroups;
    c->have_T = d->Tp && d->Ti && d->Tv;
    const int64_t nb = c->nb, ng = c->ng;

    // ---- groups
    c->gptr_h.resize(c->ngroups + 1);
    for (int g = 0; g <= c->ngroups; ++g) c->gptr_h[g] = (int)d->gptr[g];
    if (c->gptr_h[0] != 0 || c->gptr_h[c->ngroups] != nb) {
        lres_set_error("gptr must start at 0 and end at nb");
        return LRES_EINVAL;
    }
    std::vector<int> group_of_fn(nb);
    int nfmax = 0;
    for (int g = 0; g < c->ngroups; ++g) {
        const int nf = c->gptr_h[g + 1] - c->gptr_h[g];
        if (nf <= 0 || nf > 8) {
            lres_set_error("group %d has %d functions (1..8 supported)", g, nf);
            return LRES_EINVAL;
        }
        nfmax = std::max(nfmax, nf);
        for (int f = c->gptr_h[g]; f < c->gptr_h[g + 1]; ++f) group_of_fn[f] = g;
    }
    c->bp.nfmax = nfmax;

    // ---- supports of each group from the CSR rows of X (rows ascending -> slots sorted)
    std::vector<long long> scount(c->ngroups + 1, 0);
    std::vector<long long> last(c->ngroups, -1);
    for (int64_t r = 0; r < ng; ++r)
        for (int64_t p = d->Xp[r]; p < d->Xp[r + 1]; ++p) {
            const int64_t f = d->Xi[p];
            if (f < 0 || f >= nb) {
                lres_set_error("X column index out of range");
                return LRES_EINVAL;
            }
            const int g = group_of_fn[f];
            if (last[g] != r) {
                last[g] = r;
                ++scount[g + 1];
            }
        }
    std::vector<long long> soff(c->ngroups + 1, 0);
    for (int g = 0; g < c->ngroups; ++g) soff[g + 1] = soff[g] + scount[g + 1];
    const long long nslot = soff[c->ngroups];
    std::vector<int> sgrid(nslot);
    std::vector<double> sval((size_t)nslot * 8, 0.0);
    std::vector<long long> cur(soff.begin(), soff.end() - 1);
    std::fill(last.begin(), last.end(), -1);
    for (int64_t r = 0; r < ng; ++r)
        for (int64_t p = d->Xp[r]; p < d->Xp[r + 1]; ++p) {
            const int f = (int)d->Xi[p];
            const int g = group_of_fn[f];
            if (last[g] != r) {
                last[g] = r;
                sgrid[cur[g]++] = (int)r;
            }
            sval[(size_t)(cur[g] - 1) * 8 + (f - c->gptr_h[g])] = d->Xv[p];
        }
    c->sp.nslot = nslot;

    // ---- atom-pair block pattern: union of the S and T patterns, made symmetric
    std::vector<std::vector<int>> nbr(c->ngroups);
    {
        std::vector<int> mark(c->ngroups, -1);
        for (int g = 0; g < c->ngroups; ++g) {
            nbr[g].push_back(g);
            mark[g] = g;
            for (int f = c->gptr_h[g]; f < c->gptr_h[g + 1]; ++f) {
                for (int pass = 0; pass < 2; ++pass) {
                    const int64_t* Ap = pass ? d->Tp : d->Sp;
                    const int64_t* Ai = pass ? d->Ti : d->Si;
                    if (!Ap) continue;
                    for (int64_t p = Ap[f]; p < Ap[f + 1]; ++p) {
                        const int64_t b = Ai[p];
                        if (b < 0 || b >= nb) {
                            lres_set_error("S/T column index out of range");
                            return LRES_EINVAL;
                        }
                        const int h = group_of_fn[b];
                        if (mark[h] != g) {
                            mark[h] = g;
                            nbr[g].push_back(h);
                        }
                    }
                }
            }
        }
        // symmetrise
        std::vector<std::vector<int>> extra(c->ngroups);
        for (int g = 0; g < c->ngroups; ++g)
            for (int h : nbr[g]) extra[h].push_back(g);
        for (int g = 0; g < c->ngroups; ++g) {
            auto& v = nbr[g];
            v.insert(v.end(), extra[g].begin(), extra[g].end());
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
        }
    }
    c->bptr_h.assign(c->ngroups + 1, 0);
    for (int g = 0; g < c->ngroups; ++g) c->bptr_h[g + 1] = c->bptr_h[g] + (int)nbr[g].size();
    const int nblk = c->bptr_h[c->ngroups];
    c->bcol_h.resize(nblk);
    std::vector<int> brow(nblk), btrans(nblk);
    c->boff_h.resize(nblk);
    long long nval = 0;
    for (int g = 0; g < c->ngroups; ++g)
        for (int i = 0; i < (int)nbr[g].size(); ++i) {
            const int b = c->bptr_h[g] + i, h = nbr[g][i];
            c->bcol_h[b] = h;
            brow[b] = g;
            c->boff_h[b] = nval;
            nval += (long long)(c->gptr_h[g + 1] - c->gptr_h[g]) * (c->gptr_h[h + 1] - c->gptr_h[h]);
        }
    std::vector<int> pair_blk, pair_g, pair_h;
    for (int b = 0; b < nblk; ++b) {
        btrans[b] = find_block(c->bptr_h, c->bcol_h, c->bcol_h[b], brow[b]);
        if (brow[b] <= c->bcol_h[b]) {
            pair_blk.push_back(b);
            pair_g.push_back(brow[b]);
            pair_h.push_back(c->bcol_h[b]);
        }
    }
    c->bp.ngroups = c->ngroups;
    c->bp.nblk = nblk;
    c->bp.npair = (int)pair_blk.size();
    c->bp.nval = nval;

    // ---- windows: unions of whole groups, local offsets, group -> local map
    c->n_w.resize(c->nwin);
    c->m_w.resize(c->nwin);
    c->offC.assign(c->nwin + 1, 0);
    c->offF.assign(c->nwin + 1, 0);
    c->offQ.assign(c->nwin + 1, 0);
    std::vector<int> wgrp_off(c->nwin + 1, 0), wgrp, wgrp_lo;
    std::vector<int> gloc((size_t)c->nwin * c->ngroups, -1);
    for (int w = 0; w < c->nwin; ++w) {
        const int64_t a0 = d->Woff[w], a1 = d->Woff[w + 1];
        const int64_t o0 = d->Ooff[w], o1 = d->Ooff[w + 1];
        if (a1 < a0 || o1 < o0 || (w == 0 && (a0 != 0 || o0 != 0))) {
            lres_set_error("bad window / ownership offsets at window %d", w);
            return LRES_EINVAL;
        }
        int64_t a = a0;
        int lo = 0;
        while (a < a1) {
            const int64_t f = d->Wflat[a];
            if (f < 0 || f >= nb) {
                lres_set_error("window function index out of range");
                return LRES_EINVAL;
            }
            const int g = group_of_fn[f];
            const int nf = c->gptr_h[g + 1] - c->gptr_h[g];
            if (f != c->gptr_h[g] || a + nf > a1) {
                lres_set_error("window %d is not a union of whole atoms (function %lld)", w, (long long)f);
                return LRES_EINVAL;
            }
            for (int k = 0; k < nf; ++k)
                if (d->Wflat[a + k] != f + k) {
                    lres_set_error("window %d lists the functions of atom %d out of order", w, g);
                    return LRES_EINVAL;
                }
            if (gloc[(size_t)w * c->ngroups + g] >= 0) {
                lres_set_error("window %d lists atom %d twice", w, g);
                return LRES_EINVAL;
            }
            gloc[(size_t)w * c->ngroups + g] = lo;
            wgrp.push_back(g);
            wgrp_lo.push_back(lo);
            lo += nf;
            a += nf;
        }
        wgrp_off[w + 1] = (int)wgrp.size();
        c->n_w[w] = (int)(a1 - a0);
        c->m_w[w] = (int)(o1 - o0);
        c->offC[w + 1] = c->offC[w] + (long long)c->n_w[w] * c->n_w[w];
        c->offF[w + 1] = c->offF[w] + (long long)c->n_w[w] * c->m_w[w];
        c->offQ[w] = o0;
        c->offQ[w + 1] = o1;
        c->nmax = std::max(c->nmax, c->n_w[w]);
        c->mmax = std::max(c->mmax, c->m_w[w]);
    }
    c->npts = d->Ooff[c->nwin];
    for (int64_t p = 0; p < c->npts; ++p)
        if (d->Oflat[p] < 0 || d->Oflat[p] >= ng) {
            lres_set_error("owned grid index out of range");
            return LRES_EINVAL;
        }
    c->sizeC = c->offC[c->nwin];
    c->sizeF = c->offF[c->nwin];

    // ---- block values of S and T
    std::vector<double> Sblk, Tblk;
    TRY(scatter_csr(c.get(), group_of_fn, d->Sp, d->Si, d->Sv, Sblk));
    if (c->have_T) TRY(scatter_csr(c.get(), group_of_fn, d->Tp, d->Ti, d->Tv, Tblk));
    else Tblk.assign(nval, 0.0);

    // ---- uploads
    TRY(upload(&c->bp.gptr, c->gptr_h, s));
    TRY(upload(&c->bp.bptr, c->bptr_h, s));
    TRY(upload(&c->bp.bcol, c->bcol_h, s));
    TRY(upload(&c->bp.brow, brow, s));
    TRY(upload(&c->bp.boff, c->boff_h, s));
    TRY(upload(&c->bp.btrans, btrans, s));
    TRY(upload(&c->bp.pair_blk, pair_blk, s));
    TRY(upload(&c->sp.soff, soff, s));
    TRY(upload(&c->sp.sgrid, sgrid, s));
    TRY(upload(&c->sp.sval, sval, s));
    if (c->precision == LRES_MIXED && assemble_h32_supported(c->bp)) {
        // the mixed H(v) assembly reads FP32 basis values and an FP32 potential per slot
        std::vector<float> sval32(sval.begin(), sval.end());
        TRY(upload(&c->sp.sval32, sval32, s));
        TRY(dalloc(&c->sp.vslot, std::max<long long>(nslot, 1)));
    }
    TRY(upload(&c->d_Sblk, Sblk, s));
    TRY(upload(&c->d_Tblk, Tblk, s));
    TRY(dalloc(&c->d_Hblk, nval));
    if (c->precision == LRES_MIXED) TRY(dalloc(&c->d_Hblk32, nval));
    TRY(upload(&c->d_n, c->n_w, s));
    TRY(upload(&c->d_m, c->m_w, s));
    {
        // first window column with a nonzero owned-point value: the owned rows F_W (and the
        // standard-form and trace rows derived from it) are zero before it
        std::vector<int> c0(c->nwin);
        for (int w = 0; w < c->nwin; ++w) {
            int lo = c->n_w[w];
            for (int64_t pp = d->Ooff[w]; pp < d->Ooff[w + 1]; ++pp) {
                const int64_t r = d->Oflat[pp];
                for (int64_t q = d->Xp[r]; q < d->Xp[r + 1]; ++q) {
                    if (d->Xv[q] == 0.0) continue;
                    const int f = (int)d->Xi[q];
                    const int g = group_of_fn[f];
                    const int l = gloc[(size_t)w * c->ngroups + g];
                    if (l >= 0) lo = std::min(lo, l + f - c->gptr_h[g]);
                }
            }
            c0[w] = lo;
        }
        TRY(upload(&c->d_c0, c0, s));
        // the skipping kernel pays when windows skip a good share of their columns (cell
        // windows with a large R_w); with ~10% the extra partial row batches cost more
        double frac = 0.0;
        for (int w = 0; w < c->nwin; ++w) frac += c->n_w[w] ? (double)c0[w] / c->n_w[w] : 0.0;
        c->skip_rows = frac >= 0.25 * c->nwin;
    }
    TRY(upload(&c->d_offC, c->offC, s));
    TRY(upload(&c->d_offF, c->offF, s));
    TRY(upload(&c->d_offQ, c->offQ, s));
    TRY(upload(&c->d_wgrp_off, wgrp_off, s));
    TRY(upload(&c->d_wgrp, wgrp, s));
    TRY(upload(&c->d_wgrp_lo, wgrp_lo, s));
    TRY(upload(&c->d_gloc, gloc, s));
    {
        // gather tables
        std::vector<int> gfn, gbtab, gnlg(c->nwin);
        std::vector<long long> gfnoff(c->nwin + 1, 0), gbtoff(c->nwin + 1, 0);
        for (int w = 0; w < c->nwin; ++w) {
            const int i0 = wgrp_off[w], L = wgrp_off[w + 1] - i0;
            gnlg[w] = L;
            for (int a = 0; a < L; ++a) {
                const int g = wgrp[i0 + a], nf = c->gptr_h[g + 1] - c->gptr_h[g];
                if (nf > 63 || a >= (1 << 19)) {
                    lres_set_error("window gather: atoms of at most 63 functions (got %d)", nf);
                    return LRES_EINVAL;
                }
                for (int f = 0; f < nf; ++f) gfn.push_back((a << 12) | (f << 6) | nf);
            }
            gfnoff[w + 1] = (long long)gfn.size();
            for (int a = 0; a < L; ++a)
                for (int b = 0; b < L; ++b) {
                    const int blkid = find_block(c->bptr_h, c->bcol_h, wgrp[i0 + b], wgrp[i0 + a]);
                    if (blkid >= 0 && c->boff_h[blkid] > INT_MAX - 4096) {
                        lres_set_error("window gather: block storage beyond 2^31 values");
                        return LRES_EINVAL;
                    }
                    gbtab.push_back(blkid < 0 ? -1 : (int)c->boff_h[blkid]);
                }
            gbtoff[w + 1] = (long long)gbtab.size();
        }
        TRY(upload(&c->d_gfn, gfn, s));
        TRY(upload(&c->d_gfnoff, gfnoff, s));
        TRY(upload(&c->d_gbtab, gbtab, s));
        TRY(upload(&c->d_gbtoff, gbtoff, s));
        TRY(upload(&c->d_gnlg, gnlg, s));
        LRES_CUDA_TRY(cudaStreamSynchronize(s));
    }
    {
        std::vector<long long> Oflat(d->Oflat, d->Oflat + c->npts);
        TRY(upload(&c->d_Oflat, Oflat, s));
    }
    TRY(pair_common_points(c->bp, c->sp, c->ngroups, pair_g, pair_h, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));   // the uploads above read the host vectors moved below
    c->soff_h = std::move(soff);
    c->sgrid_h = std::move(sgrid);
    c->wgrp_off_h = std::move(wgrp_off);
    c->wgrp_h = std::move(wgrp);
    c->wgrp_lo_h = std::move(wgrp_lo);
    c->gloc_h = std::move(gloc);

    // ---- dense window overlaps and owned-point blocks
    TRY(dalloc(&c->d_SW, c->sizeC));
    TRY(dalloc(&c->d_HW, c->sizeC));
    TRY(gather_windows(c->nwin, c->nmax, c->d_gfn, c->d_gfnoff, c->d_gbtab, c->d_gbtoff, c->d_gnlg, c->d_offC,
                       c->d_n, c->d_Sblk, c->d_SW, nullptr, nullptr, s));
    TRY(dalloc(&c->d_F, c->sizeF));
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_F, 0, sizeof(double) * c->sizeF, s));
    {
        long long* dXp = nullptr;
        int* dXi = nullptr;
        double* dXv = nullptr;
        int* dgof = nullptr;
        const int64_t nnz = d->Xp[ng];
        std::vector<long long> Xp(d->Xp, d->Xp + ng + 1);
        std::vector<int> Xi(nnz);
        for (int64_t p = 0; p < nnz; ++p) Xi[p] = (int)d->Xi[p];
        std::vector<double> Xv(d->Xv, d->Xv + nnz);
        std::vector<long long> Ooff(d->Ooff, d->Ooff + c->nwin + 1);
        long long* dOoff = nullptr;
        TRY(upload(&dXp, Xp, s));
        TRY(upload(&dXi, Xi, s));
        TRY(upload(&dXv, Xv, s));
        TRY(upload(&dgof, group_of_fn, s));
        TRY(upload(&dOoff, Ooff, s));
        int rc = build_F(c->nwin, dXp, dXi, dXv, dgof, c->bp.gptr, c->d_gloc, c->ngroups, dOoff, c->d_Oflat,
                         c->d_offF, c->d_m, c->mmax, c->d_F, s);
        LRES_CUDA_TRY(cudaStreamSynchronize(s));
        cudaFree(dXp);
        cudaFree(dXi);
        cudaFree(dXv);
        cudaFree(dgof);
        cudaFree(dOoff);
        if (rc) return rc;
    }

    // ---- work queue: windows by decreasing size (LPT), poles inner
    c->order.resize(c->nwin);
    std::iota(c->order.begin(), c->order.end(), 0);
    std::stable_sort(c->order.begin(), c->order.end(), [&](int a, int b) {
        const long long ca = (long long)c->n_w[a] * c->n_w[a] * (c->n_w[a] + 3 * c->m_w[a]);
        const long long cb = (long long)c->n_w[b] * c->n_w[b] * (c->n_w[b] + 3 * c->m_w[b]);
        return ca > cb;
    });
    std::vector<int2> items;
    items.reserve((size_t)c->nwin * c->npoles);
    for (int w : c->order)
        for (int k = 0; k < c->npoles; ++k) items.push_back(make_int2(w, k));
    c->nitems = (int)items.size();
    TRY(upload(&c->d_items, items, s));
    std::vector<int2> witems(c->nwin);
    for (int w = 0; w < c->nwin; ++w) witems[w] = make_int2(w, 0);
    TRY(upload(&c->d_items_win, witems, s));
    TRY(dalloc(&c->d_items_sub, c->nwin));
    TRY(dalloc(&c->d_counter, 1));
    TRY(dalloc(&c->d_status, 1));
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
    TRY(dalloc(&c->d_npos, std::max(c->nitems, c->nwin)));

    // workspace of the window kernels: allocated by the first launch that needs it

    // ---- route of the pole solves: tridiagonal unless the windows are too few to fill the
    //      GPU with one CTA each, or too large for the reduction's shared-memory panels
    c->offN.assign(c->nwin + 1, 0);
    for (int w = 0; w < c->nwin; ++w) c->offN[w + 1] = c->offN[w] + c->n_w[w];
    c->sizeN = c->offN[c->nwin];
    TRY(upload(&c->d_offN, c->offN, s));
    {
        std::vector<long long> offA(c->nwin + 1, 0);
        for (int w = 0; w < c->nwin; ++w) offA[w + 1] = offA[w] + (long long)((c->n_w[w] + 3) & ~3) * c->n_w[w];
        c->sizeA = offA[c->nwin];
        TRY(upload(&c->d_offA, offA, s));
        LRES_CUDA_TRY(cudaStreamSynchronize(s));
    }
    TRY(upload(&c->d_order_w, c->order, s));
    {
        TriPick pk;
        const bool fits = tri_pick(precision == LRES_MIXED, c->nmax, c->smem_budget, 0, &pk) == LRES_OK;
        lres_set_error("");
        c->route = (fits && c->nwin >= 4) ? LRES_ROUTE_TRIDIAG : LRES_ROUTE_LDL;
    }

    // ---- standard form (mixed path; FP64 tridiagonal route)
    if (needs_standard_form(c.get())) TRY(setup_standard_form(c.get(), s));
    if (c->route == LRES_ROUTE_TRIDIAG) TRY(tri_setup(c.get(), s));

    // ---- pass buffers
    TRY(dalloc((char**)&c->d_shifts, (size_t)c->npoles * 16));
    TRY(dalloc(&c->d_wq, c->npoles));
    TRY(dalloc(&c->d_wzq, c->npoles));
    TRY(dalloc((char**)&c->d_q, (size_t)c->npoles * c->npts * (precision == LRES_MIXED ? 8 : 16)));
    TRY(dalloc(&c->d_dens, ng));
    TRY(dalloc(&c->d_v, ng));
    TRY(dalloc(&c->d_nw, c->nwin));
    TRY(dalloc(&c->d_ew, c->nwin));
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_dens, 0, sizeof(double) * ng, s));
    c->nw_h.resize(c->nwin);
    c->ew_h.resize(c->nwin);
    TRY(fft3_create(&c->fft, c->shape));
    TRY(dalloc(&c->d_fftwork, ng));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    *out = c.release();
    return LRES_OK;
}

extern "C" int lres_ctx_destroy(lres_ctx* c) {
    if (!c) return LRES_OK;
    cudaDeviceSynchronize();
    delete c;
    return LRES_OK;
}

extern "C" int lres_set_potential(lres_ctx* c, const double* v, int v_on_device, void* stream) {
    if (!c || !v) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (!c->have_T) {
        lres_set_error("lres_set_potential needs the kinetic matrix T in the system description");
        return LRES_ESTATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const double* dv = v;
    if (!v_on_device) {
        LRES_CUDA_TRY(cudaMemcpyAsync(c->d_v, v, sizeof(double) * c->ng, cudaMemcpyHostToDevice, s));
        dv = c->d_v;
    }
    TRY(mark(c, 2, 0, s));
    if (c->sp.sval32)
        TRY(assemble_h32(c->bp, c->sp, c->d_Tblk, dv, c->dV, c->d_Hblk, s));
    else
        TRY(assemble_h(c->bp, c->sp, c->d_Tblk, dv, c->dV, c->d_Hblk, s));
    TRY(mark(c, 2, 1, s));
    return after_h_blocks(c, s);
}

extern "C" int lres_set_hamiltonian_csr(lres_ctx* c, const int64_t* Hp, const int64_t* Hi, const double* Hv,
                                        void* stream) {
    if (!c || !Hp || !Hi || !Hv) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<int> group_of_fn(c->nb);
    for (int g = 0; g < c->ngroups; ++g)
        for (int f = c->gptr_h[g]; f < c->gptr_h[g + 1]; ++f) group_of_fn[f] = g;
    std::vector<double> blk;
    TRY(scatter_csr(c, group_of_fn, Hp, Hi, Hv, blk));
    LRES_CUDA_TRY(cudaMemcpyAsync(c->d_Hblk, blk.data(), sizeof(double) * blk.size(), cudaMemcpyHostToDevice, s));
    TRY(after_h_blocks(c, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));   // blk is a host temporary
    return LRES_OK;
}

extern "C" int lres_pass(lres_ctx* c, double mu, double e_lo, double* dens, int dens_on_device, double* out,
                         void* stream) {
    if (!c || !out) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (!c->have_h) {
        lres_set_error("lres_pass before a Hamiltonian was set");
        return LRES_ESTATE;
    }
    if (!(mu > e_lo) || !std::isfinite(mu) || !std::isfinite(e_lo)) {
        lres_set_error("need finite e_lo < mu (got mu=%g, e_lo=%g)", mu, e_lo);
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int P = c->npoles;
    const bool mixed = c->precision == LRES_MIXED;
    // nodes and weights on the device, the same kernel as the capturable pass (bitwise equal results)
    poles_kernel<<<(P + 63) / 64, 64, 0, s>>>(P, c->M, mu, e_lo, mixed ? 1 : 0, c->d_shifts, c->d_wq, c->d_wzq);
    LRES_CUDA_TRY(cudaGetLastError());
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_counter, 0, sizeof(int), s));
    // no density requested and trace rows installed: the pass over the trace rows
    const bool trace = !dens && c->have_trace;
    if (c->route == LRES_ROUTE_TRIDIAG) {
        if (!c->tri_ready) TRY(tri_refresh(c, s));
        TRY(tri_run_pass(c, trace, s));
    } else {
        const Rows rw = select_rows(c, trace);
        TRY(ensure_hhat_df(c, s));
        TRY(mark(c, 0, 0, s));
        if (mixed)
            TRY(ldl_launch(c, LdlJob::C64, c->nitems, c->d_items, c->d_Hhat32, nullptr, rw.F, rw.m, rw.offF,
                           c->d_shifts, rw.q, nullptr, c->nmax + rw.mmax, rw.mmax, s, rw.offQ, rw.npts));
        else
            TRY(ldl_launch(c, LdlJob::C128, c->nitems, c->d_items, c->d_HW, c->d_SW, rw.F, rw.m, rw.offF,
                           c->d_shifts, rw.q, nullptr, c->nmax + rw.mmax, rw.mmax, s, rw.offQ, rw.npts));
        TRY(mark(c, 0, 1, s));
        TRY(mark(c, 1, 0, s));
        TRY(pole_sums(c->nwin, rw.offQ, rw.m, rw.Oflat, mixed, rw.q, rw.npts, P, c->d_wq, c->d_wzq, c->dV,
                      rw.dens, c->d_nw, c->d_ew, s));
        TRY(mark(c, 1, 1, s));
    }
    LRES_CUDA_TRY(cudaMemcpyAsync(c->nw_h.data(), c->d_nw, sizeof(double) * c->nwin, cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(c->ew_h.data(), c->d_ew, sizeof(double) * c->nwin, cudaMemcpyDeviceToHost, s));
    if (dens)
        LRES_CUDA_TRY(cudaMemcpyAsync(dens, c->d_dens, sizeof(double) * c->ng,
                                      dens_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    int st = 0;
    TRY(read_pass_status(c, s, &st));
    double N = 0.0, E = 0.0;
    for (int w = 0; w < c->nwin; ++w) {
        N += c->nw_h[w];
        E += c->ew_h[w];
    }
    out[0] = N;
    out[1] = E;
    out[2] = (double)st;
    if (st & ST_ZERO_PIVOT) {
        lres_set_error("zero or non-finite pivot in a window factorisation");
        return LRES_ENUMERIC;
    }
    if (st) {
        lres_set_error("window kernel status %d", st);
        return LRES_EINVAL;
    }
    return LRES_OK;
}

extern "C" int lres_autotune(lres_ctx* c, double mu, double e_lo, int32_t force_config, int32_t* chosen,
                             double* ms_per_config, void* stream) {
    if (!c) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (force_config >= kLeftConfigs) {
        lres_set_error("configuration %d out of range (0..%d)", force_config, kLeftConfigs - 1);
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (c->route == LRES_ROUTE_TRIDIAG) {
        // panel widths of the reduction and the row application, timed on the current
        // Hamiltonian (reduction + rows per configuration)
        auto apply_cfg = [&](int cfg) -> int {
            TriPick pk;
            TRY(tri_pick(c->precision == LRES_MIXED, c->nmax, c->smem_budget, cfg, &pk));
            c->tri_cfg = cfg;
            c->tri = pk;
            if (c->tri_alloc) {
                TRY(ensure_tfactors(c));
                if (c->ri_own.arows != pk.arows) TRY(build_row_items(c, c->m_w, c->ri_own, s));
                if (c->have_trace && c->ri_tr.arows != pk.arows) {
                    std::vector<int> mT(c->nwin);
                    LRES_CUDA_TRY(cudaMemcpy(mT.data(), c->d_mT, sizeof(int) * c->nwin, cudaMemcpyDeviceToHost));
                    TRY(build_row_items(c, mT, c->ri_tr, s));
                }
            }
            if (c->have_h) TRY(tri_refresh(c, s));
            return LRES_OK;
        };
        if (force_config >= 0) {
            TRY(apply_cfg(force_config));
            if (chosen) *chosen = force_config;
            return LRES_OK;
        }
        if (!c->have_h) {
            lres_set_error("lres_autotune before a Hamiltonian was set");
            return LRES_ESTATE;
        }
        double best = 1e300;
        int arg = 0;
        for (int cfg = 0; cfg < kLeftConfigs; ++cfg) {
            double ms = 0.0;
            for (int rep = 0; rep < 2; ++rep) {          // first repetition warms up
                TRY(apply_cfg(cfg));
                double t[8];
                TRY(lres_timings(c, t, 8));
                ms = t[6] + t[7];
            }
            if (ms_per_config) ms_per_config[cfg] = ms;
            if (ms < best) {
                best = ms;
                arg = cfg;
            }
        }
        TRY(apply_cfg(arg));
        if (chosen) *chosen = arg;
        return LRES_OK;
    }
    if (force_config >= 0) {
        c->config = force_config;
        if (chosen) *chosen = force_config;
        return LRES_OK;
    }
    double out[3];
    double best = 1e300;
    int arg = 0;
    for (int cfg = 0; cfg < kLeftConfigs; ++cfg) {
        // the tensor-core variant (3xTF32) is timed but chosen only when forced: its
        // measured error is about 5x that of the FP32 SIMT configurations
        c->config = cfg;
        double ms = 0.0;
        for (int rep = 0; rep < 2; ++rep) {          // first repetition warms up
            TRY(lres_pass(c, mu, e_lo, nullptr, 0, out, stream));
            double t[1];
            TRY(lres_timings(c, t, 1));
            ms = t[0];
        }
        if (ms_per_config) ms_per_config[cfg] = ms;
        const bool eligible = !(cfg == 4 && c->precision == LRES_MIXED);
        if (eligible && ms < best) {
            best = ms;
            arg = cfg;
        }
    }
    c->config = arg;
    if (chosen) *chosen = arg;
    return LRES_OK;
}

extern "C" int lres_set_route(lres_ctx* c, int32_t route, void* stream) {
    if (!c || (route != LRES_ROUTE_LDL && route != LRES_ROUTE_TRIDIAG)) {
        lres_set_error("route must be LRES_ROUTE_LDL or LRES_ROUTE_TRIDIAG");
        return LRES_EINVAL;
    }
    if (route == c->route) return LRES_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (route == LRES_ROUTE_LDL) {
        c->route = route;
        c->tri_ready = false;               // T no longer follows the Hamiltonian
        return LRES_OK;
    }
    TriPick pk;
    TRY(tri_pick(c->precision == LRES_MIXED, c->nmax, c->smem_budget, c->tri_cfg, &pk));
    const int old = c->route;
    c->route = route;
    int rc = LRES_OK;
    if (c->precision != LRES_MIXED && !c->d_LinvT) rc = setup_standard_form(c, s);
    if (!rc) rc = tri_setup(c, s);
    if (!rc && c->have_h) {
        rc = window_transform(c, s);           // the route's standard form of the current H
        if (!rc) rc = tri_prepare(c, s);
    }
    if (rc) {
        c->route = old;
        c->tri_ready = false;
        return rc;
    }
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    return LRES_OK;
}

extern "C" int lres_set_standard_form_kernel(lres_ctx* c, int32_t kind) {
    if (!c || (kind != LRES_SF_SIMT && kind != LRES_SF_TENSOR)) {
        lres_set_error("standard-form kernel must be LRES_SF_SIMT or LRES_SF_TENSOR");
        return LRES_EINVAL;
    }
    c->sf_kind = kind;
    return LRES_OK;
}

extern "C" int lres_get_standard_form_kernel(lres_ctx* c, int32_t* kind) {
    if (!c || !kind) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    *kind = c->sf_kind;
    return LRES_OK;
}

extern "C" int lres_get_route(lres_ctx* c, int32_t* route) {
    if (!c || !route) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    *route = c->route;
    return LRES_OK;
}

extern "C" int lres_timings(lres_ctx* c, double* ms, int n) {
    if (!c || !ms || n < 0) {
        lres_set_error("bad arguments to lres_timings");
        return LRES_EINVAL;
    }
    for (int i = 0; i < n && i < 8; ++i) {
        ms[i] = -1.0;
        if (!c->ev_used[i]) continue;
        LRES_CUDA_TRY(cudaEventSynchronize(c->ev[2 * i + 1]));
        float t = 0.f;
        LRES_CUDA_TRY(cudaEventElapsedTime(&t, c->ev[2 * i], c->ev[2 * i + 1]));
        ms[i] = t;
    }
    for (int i = 8; i < n; ++i) ms[i] = -1.0;
    return LRES_OK;
}

extern "C" int lres_pass_async(lres_ctx* c, double mu, double e_lo, double* d_out, void* stream) {
    if (!c || !d_out) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (!c->have_h) {
        lres_set_error("lres_pass_async before a Hamiltonian was set");
        return LRES_ESTATE;
    }
    if (!(mu > e_lo) || !std::isfinite(mu) || !std::isfinite(e_lo)) {
        lres_set_error("need finite e_lo < mu (got mu=%g, e_lo=%g)", mu, e_lo);
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const bool mixed = c->precision == LRES_MIXED;
    const int P = c->npoles;
    poles_kernel<<<(P + 63) / 64, 64, 0, s>>>(P, c->M, mu, e_lo, mixed ? 1 : 0, c->d_shifts, c->d_wq, c->d_wzq);
    LRES_CUDA_TRY(cudaGetLastError());
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
    if (c->route == LRES_ROUTE_TRIDIAG) {
        if (!c->tri_ready) TRY(tri_refresh(c, s));
        TRY(tri_run_pass(c, false, s));
    } else {
        TRY(ensure_hhat_df(c, s));
        if (mixed)
            TRY(ldl_launch(c, LdlJob::C64, c->nitems, c->d_items, c->d_Hhat32, nullptr, c->d_Fhat32, c->d_m,
                           c->d_offF, c->d_shifts, c->d_q, nullptr, c->nmax + c->mmax, c->mmax, s));
        else
            TRY(ldl_launch(c, LdlJob::C128, c->nitems, c->d_items, c->d_HW, c->d_SW, c->d_F, c->d_m, c->d_offF,
                           c->d_shifts, c->d_q, nullptr, c->nmax + c->mmax, c->mmax, s));
        TRY(pole_sums(c->nwin, c->d_offQ, c->d_m, c->d_Oflat, mixed, c->d_q, c->npts, P, c->d_wq, c->d_wzq,
                      c->dV, c->d_dens, c->d_nw, c->d_ew, s));
    }
    window_total_kernel<<<1, 1, 0, s>>>(c->nwin, c->d_nw, c->d_ew, d_out);
    LRES_CUDA_TRY(cudaGetLastError());
    return LRES_OK;
}

extern "C" int lres_status(lres_ctx* c, int32_t* status, void* stream) {
    if (!c || !status) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    int st = 0;
    TRY(read_pass_status(c, (cudaStream_t)stream, &st));
    *status = st;
    return LRES_OK;
}

extern "C" int lres_density_ptr(lres_ctx* c, const double** d_dens) {
    if (!c || !d_dens) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    *d_dens = c->d_dens;
    return LRES_OK;
}

extern "C" int lres_window_sums(lres_ctx* c, double* n_w, double* e_w) {
    if (!c) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (n_w) std::copy(c->nw_h.begin(), c->nw_h.end(), n_w);
    if (e_w) std::copy(c->ew_h.begin(), c->ew_h.end(), e_w);
    return LRES_OK;
}

extern "C" int lres_inertia(lres_ctx* c, double sigma, int32_t* below, int64_t* total, void* stream) {
    if (!c) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (!c->have_h) {
        lres_set_error("lres_inertia before a Hamiltonian was set");
        return LRES_ESTATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (c->route == LRES_ROUTE_TRIDIAG) {
        // Sturm counts of T - sigma: T is congruent to the pencil (H_W, S_W)
        if (!c->tri_ready) TRY(tri_refresh(c, s));
        TRY(mark(c, 5, 0, s));
        TRY(tri_sturm(c->precision == LRES_MIXED, c->nwin, c->d_n, c->d_offN, c->d_trid, c->d_trie, sigma,
                      c->d_npos, s));
        TRY(mark(c, 5, 1, s));
    } else {
        LRES_CUDA_TRY(cudaMemcpyAsync(c->d_shifts, &sigma, sizeof(double), cudaMemcpyHostToDevice, s));
        LRES_CUDA_TRY(cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
        // positive pivots of (sigma S - H) = eigenvalues of (H, S) below sigma
        LRES_CUDA_TRY(cudaMemsetAsync(c->d_counter, 0, sizeof(int), s));
        TRY(mark(c, 5, 0, s));
        TRY(ldl_launch(c, LdlJob::R64, c->nwin, c->d_items_win, c->d_HW, c->d_SW, nullptr, c->d_m, c->d_offF,
                       c->d_shifts, nullptr, nullptr, c->nmax, 0, s));
        TRY(mark(c, 5, 1, s));
    }
    std::vector<int> cnt(c->nwin);
    LRES_CUDA_TRY(cudaMemcpyAsync(cnt.data(), c->d_npos, sizeof(int) * c->nwin, cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    int64_t t = 0;
    for (int w = 0; w < c->nwin; ++w) {
        t += cnt[w];
        if (below) below[w] = cnt[w];
    }
    if (total) *total = t;
    return LRES_OK;
}

// Inertia of the windows listed in `wins` (host), counts into cnt (host).
static int inertia_subset(lres_ctx* c, double sigma, const std::vector<int>& wins, std::vector<int>& cnt,
                          cudaStream_t s) {
    std::vector<int2> items(wins.size());
    for (size_t i = 0; i < wins.size(); ++i) items[i] = make_int2(wins[i], 0);
    LRES_CUDA_TRY(cudaMemcpyAsync(c->d_items_sub, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(c->d_shifts, &sigma, sizeof(double), cudaMemcpyHostToDevice, s));
    TRY(ldl_launch(c, LdlJob::R64, (int)wins.size(), c->d_items_sub, c->d_HW, c->d_SW, nullptr, c->d_m, c->d_offF,
                   c->d_shifts, nullptr, nullptr, c->nmax, 0, s));
    cnt.resize(wins.size());
    LRES_CUDA_TRY(cudaMemcpyAsync(cnt.data(), c->d_npos, sizeof(int) * wins.size(), cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    return LRES_OK;
}

extern "C" int lres_min_eig(lres_ctx* c, double lo, double hi, double tol, double* lam_min, void* stream) {
    if (!c || !lam_min || !(hi > lo) || !(tol > 0)) {
        lres_set_error("bad arguments to lres_min_eig");
        return LRES_EINVAL;
    }
    if (!c->have_h) {
        lres_set_error("lres_min_eig before a Hamiltonian was set");
        return LRES_ESTATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (c->route == LRES_ROUTE_TRIDIAG) {
        // every window's smallest eigenvalue by Sturm bisection on T, to width tol
        if (!c->tri_ready) TRY(tri_refresh(c, s));
        TRY(tri_min_eig(c->precision == LRES_MIXED, c->nwin, c->d_n, c->d_offN, c->d_trid, c->d_trie, tol,
                        c->d_lam, s));
        std::vector<double> lam(c->nwin);
        LRES_CUDA_TRY(cudaMemcpyAsync(lam.data(), c->d_lam, sizeof(double) * c->nwin, cudaMemcpyDeviceToHost, s));
        LRES_CUDA_TRY(cudaStreamSynchronize(s));
        *lam_min = *std::min_element(lam.begin(), lam.end());
        return LRES_OK;
    }
    std::vector<int> all(c->nwin), cnt;
    std::iota(all.begin(), all.end(), 0);
    auto any_below = [&](double sigma, const std::vector<int>& wins, std::vector<int>* keep) -> int {
        TRY(inertia_subset(c, sigma, wins, cnt, s));
        int found = 0;
        if (keep) keep->clear();
        for (size_t i = 0; i < wins.size(); ++i)
            if (cnt[i] > 0) {
                found = 1;
                if (keep) keep->push_back(wins[i]);
            }
        return found ? 1 : 0;
    };
    // lo must have no eigenvalue below it in any window
    for (int it = 0;; ++it) {
        const int r = any_below(lo, all, nullptr);
        if (r < 0) return r;
        if (r == 0) break;
        if (it == 59) {
            lres_set_error("no lower bound found for the window spectra");
            return LRES_ENUMERIC;
        }
        const double wdt = hi - lo;
        hi = lo;
        lo -= 2 * wdt;
    }
    // hi must have an eigenvalue below it; only windows with one can hold the minimum
    std::vector<int> cand;
    for (int it = 0;; ++it) {
        const int r = any_below(hi, all, &cand);
        if (r < 0) return r;
        if (r == 1) break;
        if (it == 59) {
            lres_set_error("no upper bound found for the smallest window eigenvalue");
            return LRES_ENUMERIC;
        }
        const double wdt = hi - lo;
        lo = hi;
        hi += 2 * wdt;
    }
    // bisection on the candidate windows, pruning those with no eigenvalue below hi
    std::vector<int> next;
    while (hi - lo > tol) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        const int r = any_below(mid, cand, &next);
        if (r < 0) return r;
        if (r == 1) {
            hi = mid;
            cand.swap(next);
        } else {
            lo = mid;
        }
    }
    *lam_min = 0.5 * (lo + hi);
    return LRES_OK;
}

extern "C" int lres_voronoi_owner(const int64_t shape[3], const double cell[3], int64_t ncent, const double* centres,
                                  int32_t* owner) {
    if (!shape || !cell || !centres || !owner || ncent <= 0) {
        lres_set_error("bad arguments to lres_voronoi_owner");
        return LRES_EINVAL;
    }
    const long long ng = shape[0] * shape[1] * shape[2];
    double* dc = nullptr;
    int* dow = nullptr;
    TRY(dalloc(&dc, 3 * ncent));
    int rc = dalloc(&dow, ng);
    if (rc) {
        cudaFree(dc);
        return rc;
    }
    cudaStream_t s = 0;
    rc = LRES_OK;
    if (cudaMemcpy(dc, centres, sizeof(double) * 3 * ncent, cudaMemcpyHostToDevice) != cudaSuccess) rc = LRES_ECUDA;
    if (!rc) rc = voronoi_apply(shape, cell, (int)ncent, dc, dow, s);
    if (!rc && cudaMemcpy(owner, dow, sizeof(int) * ng, cudaMemcpyDeviceToHost) != cudaSuccess) rc = LRES_ECUDA;
    if (rc == LRES_ECUDA) lres_set_error("voronoi: %s", cudaGetErrorString(cudaGetLastError()));
    cudaFree(dc);
    cudaFree(dow);
    return rc;
}

extern "C" int lres_lda_xc(lres_ctx* c, const double* dens, double* exc, double* vxc, void* stream) {
    if (!c || !dens || !exc || !vxc) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    return lda_apply(c->ng, dens, exc, vxc, (cudaStream_t)stream);
}

extern "C" int lres_hartree(lres_ctx* c, const double* dens, double* vh, void* stream) {
    if (!c || !dens || !vh) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    return hartree_apply(c->fft, c->shape, c->cell, dens, vh, c->d_fftwork, (cudaStream_t)stream);
}

extern "C" int lres_ion_potential(lres_ctx* c, int64_t natoms, const double* pos, const double* Z, const double* rc,
                                  double* vion, void* stream) {
    if (!c || !pos || !Z || !rc || !vion || natoms <= 0) {
        lres_set_error("bad arguments to lres_ion_potential");
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    double *dp = nullptr, *dz = nullptr, *dr = nullptr;
    TRY(dalloc(&dp, 3 * natoms));
    TRY(dalloc(&dz, natoms));
    TRY(dalloc(&dr, natoms));
    LRES_CUDA_TRY(cudaMemcpyAsync(dp, pos, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(dz, Z, sizeof(double) * natoms, cudaMemcpyHostToDevice, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(dr, rc, sizeof(double) * natoms, cudaMemcpyHostToDevice, s));
    int r = ion_apply(c->fft, c->shape, c->cell, (int)natoms, dp, dz, dr, vion, c->d_fftwork, s);
    cudaStreamSynchronize(s);
    cudaFree(dp);
    cudaFree(dz);
    cudaFree(dr);
    return r;
}

// ---------------------------------------------------------------------------
// window matrices set directly, and the adjoint of the band energy at fixed N
// ---------------------------------------------------------------------------

extern "C" int lres_set_windows(lres_ctx* c, const double* HW, const double* SW, int on_device, void* stream) {
    if (!c || (!HW && !SW)) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (!HW && !c->have_h) {
        lres_set_error("lres_set_windows without H_W before a Hamiltonian was set");
        return LRES_ESTATE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    c->h32_dense = false;                // the FP32 windows, if any, are of the previous H
    if (HW) LRES_CUDA_TRY(cudaMemcpyAsync(c->d_HW, HW, sizeof(double) * c->sizeC, kind, s));
    if (SW) {
        LRES_CUDA_TRY(cudaMemcpyAsync(c->d_SW, SW, sizeof(double) * c->sizeC, kind, s));
        if (needs_standard_form(c)) TRY(setup_standard_form(c, s));
        else TRY(check_overlaps(c, s));
    }
    if (needs_standard_form(c)) TRY(window_transform(c, s));
    if (c->route == LRES_ROUTE_TRIDIAG) TRY(tri_prepare(c, s));
    c->have_h = true;
    if (!on_device) LRES_CUDA_TRY(cudaStreamSynchronize(s));
    return LRES_OK;
}

extern "C" int lres_window_ptrs(lres_ctx* c, const double** d_HW, const double** d_SW) {
    if (!c || !d_HW || !d_SW) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    *d_HW = c->d_HW;
    *d_SW = c->d_SW;
    return LRES_OK;
}

namespace {

// Inverse maps of the adjoint (once per context): for every stored atom-pair block the
// windows holding both atoms with the atoms' local offsets (windows ascending), and for
// every grid point the atoms whose support covers it with their support slots.
int adj_prepare(lres_ctx* c, cudaStream_t s) {
    if (c->adj_ready) return LRES_OK;
    const int nblk = c->bp.nblk;
    std::vector<long long> eoff(nblk + 1, 0);
    for (int pass = 0; pass < 2; ++pass) {
        std::vector<long long> cur;
        std::vector<int4> ent;
        if (pass) {
            for (int b = 0; b < nblk; ++b) eoff[b + 1] += eoff[b];
            cur.assign(eoff.begin(), eoff.end() - 1);
            ent.resize(eoff[nblk]);
        }
        for (int w = 0; w < c->nwin; ++w)
            for (int gi = c->wgrp_off_h[w]; gi < c->wgrp_off_h[w + 1]; ++gi) {
                const int g = c->wgrp_h[gi], lg = c->wgrp_lo_h[gi];
                for (int b = c->bptr_h[g]; b < c->bptr_h[g + 1]; ++b) {
                    const int lh = c->gloc_h[(size_t)w * c->ngroups + c->bcol_h[b]];
                    if (lh < 0) continue;
                    if (pass) ent[cur[b]++] = make_int4(w, lg, lh, 0);
                    else ++eoff[b + 1];
                }
            }
        if (pass) {
            TRY(upload(&c->d_eoff, eoff, s));
            TRY(upload(&c->d_ent, ent, s));
            LRES_CUDA_TRY(cudaStreamSynchronize(s));
        }
    }
    std::vector<long long> poff(c->ng + 1, 0);
    for (long long sl = 0; sl < (long long)c->sgrid_h.size(); ++sl) ++poff[c->sgrid_h[sl] + 1];
    for (long long r = 0; r < c->ng; ++r) poff[r + 1] += poff[r];
    std::vector<int2> pent(poff[c->ng]);
    {
        std::vector<long long> cur(poff.begin(), poff.end() - 1);
        for (int g = 0; g < c->ngroups; ++g)
            for (long long sl = c->soff_h[g]; sl < c->soff_h[g + 1]; ++sl)
                pent[cur[c->sgrid_h[sl]]++] = make_int2(g, (int)sl);
    }
    TRY(upload(&c->d_poff, poff, s));
    TRY(upload(&c->d_pent, pent, s));
    TRY(upload(&c->d_order, c->order, s));
    for (double*& a : c->d_adjA) TRY(dalloc(&a, c->sizeC));
    TRY(dalloc(&c->d_dHW, c->sizeC));
    TRY(dalloc(&c->d_dSW, c->sizeC));
    TRY(dalloc(&c->d_gH, c->bp.nval));
    TRY(dalloc(&c->d_adjdv, c->ng));
    TRY(dalloc(&c->d_adju, 3 * (size_t)c->nwin));
    TRY(dalloc(&c->d_cw, 3 * (size_t)c->npoles));
    c->adju_h.resize(3 * (size_t)c->nwin);
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    c->adj_ready = true;
    return LRES_OK;
}

}  // namespace

extern "C" int lres_adjoint(lres_ctx* c, double mu, double e_lo, double* dv, int dv_on_device, double* dHW,
                            double* dSW, int dW_on_device, double* out, void* stream) {
    if (!c || !out) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    if (!c->have_h) {
        lres_set_error("lres_adjoint before a Hamiltonian was set");
        return LRES_ESTATE;
    }
    if (!(mu > e_lo) || !std::isfinite(mu) || !std::isfinite(e_lo)) {
        lres_set_error("need finite e_lo < mu (got mu=%g, e_lo=%g)", mu, e_lo);
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    TRY(ensure_hhat_df(c, s));                 // the adjoint factors the double-float standard form
    TRY(adj_prepare(c, s));
    const bool mixed = c->precision == LRES_MIXED;
    const int P = c->npoles;
    const size_t el = mixed ? 8 : 16;
    const int nbk = mixed ? kKeepNB64 : kKeepNB128;
    const long long npmax = (c->nmax + nbk - 1) / nbk * nbk;
    const int mrows = c->have_trace ? c->mmaxT : c->mmax;
    const long long stride = ((npmax + mrows + 1) * npmax + 15) / 16 * 16;   // elements per item slot
    const size_t item_bytes = (size_t)stride * el;
    // items per batch: whole windows (all poles), as many as the free device memory admits
    size_t freeb = 0, totalb = 0;
    LRES_CUDA_TRY(cudaMemGetInfo(&freeb, &totalb));
    size_t have = c->adjws_bytes + freeb;
    const size_t reserve = (size_t)4 << 30;
    size_t budget = have > reserve ? std::min(have - reserve, have / 4 * 3) : 0;
    long long win_per_batch = (long long)(budget / (item_bytes * P));
    if (win_per_batch < 1) {
        lres_set_error("adjoint: one window's %d pole factors (%zu bytes) do not fit in free device memory", P,
                       item_bytes * P);
        return LRES_ENOMEM;
    }
    win_per_batch = std::min<long long>(win_per_batch, c->nwin);
    const size_t need = item_bytes * P * (size_t)win_per_batch;
    if (c->adjws_bytes < need) {
        if (c->d_adjws) cudaFree(c->d_adjws);
        c->d_adjws = nullptr;
        c->adjws_bytes = 0;
        TRY(dalloc((char**)&c->d_adjws, need));
        c->adjws_bytes = need;
    }
    const Rows rw = select_rows(c, c->have_trace);
    poles_kernel<<<(P + 63) / 64, 64, 0, s>>>(P, c->M, mu, e_lo, mixed ? 1 : 0, c->d_shifts, c->d_wq, c->d_wzq);
    LRES_CUDA_TRY(cudaGetLastError());
    TRY(adj_weights(P, c->M, mu, e_lo, c->d_cw, s));
    LRES_CUDA_TRY(cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
    for (long long w0 = 0; w0 < c->nwin; w0 += win_per_batch) {
        const int nwb = (int)std::min<long long>(win_per_batch, c->nwin - w0);
        const int2* items = c->d_items + w0 * P;       // windows in work-queue order, poles inner
        const int nit = nwb * P;
        LdlJob j{};
        j.kind = mixed ? LdlJob::C64 : LdlJob::C128;
        j.nitems = nit;
        j.items = items;
        j.counter = c->d_counter;
        j.n_w = c->d_n;
        j.m_w = rw.m;
        j.offC = c->d_offC;
        j.offF = rw.offF;
        j.offQ = rw.offQ;
        j.C = mixed ? (const void*)c->d_Hhat32 : (const void*)c->d_HW;
        j.B = mixed ? nullptr : (const void*)c->d_SW;
        j.F = rw.F;
        j.shifts = c->d_shifts;
        j.q = rw.q;
        j.qstride = rw.npts;
        j.npos = c->d_npos;
        j.status = c->d_status;
        j.ws = c->d_adjws;
        j.ws_stride = stride;
        j.ldp = c->nmax + rw.mmax;
        j.nmax = c->nmax;
        j.mmax = rw.mmax;
        j.grid = nit;
        j.smem_budget = c->smem_budget;
        j.config = 0;
        j.keep = 1;
        LRES_CUDA_TRY(cudaMemsetAsync(c->d_counter, 0, sizeof(int), s));
        TRY(run_ldl(j, s));
        TRY(adj_backsolve(mixed, items, nit, c->d_n, rw.m, c->d_adjws, stride, c->d_status, s));
        TRY(adj_accumulate(mixed, c->d_order + w0, nwb, P, c->nmax, c->d_n, rw.m, c->d_offC, c->d_adjws, stride,
                           c->d_cw, c->d_adjA[0], c->d_adjA[1], c->d_adjA[2], s));
    }
    TRY(pole_sums(c->nwin, rw.offQ, rw.m, rw.Oflat, mixed, rw.q, rw.npts, P, c->d_wq, c->d_wzq, c->dV, rw.dens,
                  c->d_nw, c->d_ew, s));
    TRY(adj_inner(c->nwin, c->d_n, c->d_offC, mixed ? nullptr : c->d_SW, c->d_adjA[0], c->d_adjA[1], c->d_adjA[2],
                  c->d_adju, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(c->nw_h.data(), c->d_nw, sizeof(double) * c->nwin, cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(c->ew_h.data(), c->d_ew, sizeof(double) * c->nwin, cudaMemcpyDeviceToHost, s));
    LRES_CUDA_TRY(cudaMemcpyAsync(c->adju_h.data(), c->d_adju, sizeof(double) * 3 * c->nwin,
                                  cudaMemcpyDeviceToHost, s));
    int st = 0;
    TRY(read_status(c, s, &st));
    if (st) {
        lres_set_error(st & ST_ZERO_PIVOT ? "zero or non-finite pivot in a window factorisation (adjoint)"
                                          : "window kernel status %d (adjoint)", st);
        return st & ST_ZERO_PIVOT ? LRES_ENUMERIC : LRES_EINVAL;
    }
    double N = 0.0, E = 0.0, U[3] = {0.0, 0.0, 0.0};
    for (int w = 0; w < c->nwin; ++w) {
        N += c->nw_h[w];
        E += c->ew_h[w];
        for (int k = 0; k < 3; ++k) U[k] += c->adju_h[(size_t)k * c->nwin + w];
    }
    for (double& u : U) u *= 4.0 * c->dV;
    // z' = (1 + zeta)/2 = 1/2 + (z - cc)/(2R) and w' = w/(2R): every mu derivative is a real
    // combination of the three accumulations and of N, E
    const double cc = 0.5 * (mu + e_lo), R = 0.5 * (mu - e_lo);
    const double a0 = 0.5 - cc / (2.0 * R), a1 = 1.0 / (2.0 * R);
    const double dNdmu = N / (2.0 * R) - (a0 * U[0] + a1 * U[1]);
    const double dEdmu = E / R + 0.5 * N - cc * N / (2.0 * R) - (a0 * U[1] + a1 * U[2]);
    if (!(dNdmu != 0.0) || !std::isfinite(dNdmu) || !std::isfinite(dEdmu)) {
        lres_set_error("adjoint: dN/dmu = %g is not usable", dNdmu);
        return LRES_ENUMERIC;
    }
    const double kappa = dEdmu / dNdmu;
    const double sc = 4.0 * c->dV;
    if (mixed) {
        // B_H = 4dV (A1 - kappa A0) into A0, B_S = -4dV (A2 - kappa A1) into A2, then L^-T B L^-1
        TRY(adj_combine(c->sizeC, c->d_adjA[0], c->d_adjA[1], c->d_adjA[2], kappa, sc, -sc, c->d_adjA[0],
                        c->d_adjA[2], s));
        for (int which = 0; which < 2; ++which) {
            const double* B = which ? c->d_adjA[2] : c->d_adjA[0];
            double* D = which ? c->d_dSW : c->d_dHW;
            TRY(batched_gemm(c->nwin, c->d_n, c->d_offC, c->nmax, false, c->d_LinvT, B, c->d_adjA[1], s));
            TRY(batched_gemm(c->nwin, c->d_n, c->d_offC, c->nmax, false, c->d_adjA[1], c->d_LinvT, D, s, 0, true));
        }
    } else {
        TRY(adj_combine(c->sizeC, c->d_adjA[0], c->d_adjA[1], c->d_adjA[2], kappa, sc, -sc, c->d_dHW, c->d_dSW,
                        s));
    }
    TRY(adj_block_gather(c->bp, c->d_eoff, c->d_ent, c->d_n, c->d_offC, c->d_dHW, c->d_gH, s));
    TRY(adj_point(c->ng, c->d_poff, c->d_pent, c->sp, c->bp, c->d_gH, c->dV, c->d_adjdv, s));
    if (dv)
        LRES_CUDA_TRY(cudaMemcpyAsync(dv, c->d_adjdv, sizeof(double) * c->ng,
                                      dv_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    const cudaMemcpyKind wk = dW_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (dHW) LRES_CUDA_TRY(cudaMemcpyAsync(dHW, c->d_dHW, sizeof(double) * c->sizeC, wk, s));
    if (dSW) LRES_CUDA_TRY(cudaMemcpyAsync(dSW, c->d_dSW, sizeof(double) * c->sizeC, wk, s));
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    out[0] = N;
    out[1] = E;
    out[2] = dNdmu;
    out[3] = dEdmu;
    out[4] = kappa;
    out[5] = (double)st;
    return LRES_OK;
}

// ---------------------------------------------------------------------------
// trace rows: N and E_band (and the adjoint) depend on the owned-point rows F_W only
// through F_W^T F_W, so any R_W with R_W^T R_W = F_W^T F_W (rank <= n_W rows) gives the
// same sums with fewer rows when the grid is fine
// ---------------------------------------------------------------------------

extern "C" int lres_owned_gram(lres_ctx* c, double* K, int on_device, void* stream) {
    if (!c || !K) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    double* dK = K;
    if (!on_device) TRY(dalloc(&dK, c->sizeC));
    int rc = batched_gram(c->nwin, c->d_n, c->d_m, c->d_offF, c->d_offC, c->nmax, c->d_F, dK, s);
    if (!rc && !on_device) {
        cudaError_t e = cudaMemcpyAsync(K, dK, sizeof(double) * c->sizeC, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            lres_set_error("lres_owned_gram: %s", cudaGetErrorString(e));
            rc = LRES_ECUDA;
        }
    }
    if (!on_device) cudaFree(dK);
    return rc;
}

extern "C" int lres_set_trace_rows(lres_ctx* c, const int32_t* r_w, const double* R, void* stream) {
    if (!c) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    for (void* p : {(void*)c->d_mT, (void*)c->d_offFT, (void*)c->d_offQT, (void*)c->d_FT, (void*)c->d_FhatT32,
                    c->d_qT, (void*)c->d_FhatT64, c->d_Ytr})
        if (p) cudaFree(p);
    c->d_mT = nullptr;
    c->d_offFT = c->d_offQT = nullptr;
    c->d_FT = nullptr;
    c->d_FhatT32 = nullptr;
    c->d_FhatT64 = nullptr;
    c->d_qT = nullptr;
    c->d_Ytr = nullptr;
    c->ri_tr.release();
    c->have_trace = false;
    if (!r_w) return LRES_OK;                 // removed
    if (!R) {
        lres_set_error("null argument");
        return LRES_EINVAL;
    }
    std::vector<int> m(c->nwin);
    std::vector<long long> offF(c->nwin + 1, 0), offQ(c->nwin + 1, 0);
    int mmax = 0;
    for (int w = 0; w < c->nwin; ++w) {
        if (r_w[w] < 0 || r_w[w] > c->mmax) {
            lres_set_error("trace rows of window %d: %d (0..%d allowed)", w, r_w[w], c->mmax);
            return LRES_EINVAL;
        }
        m[w] = r_w[w];
        mmax = std::max(mmax, m[w]);
        offF[w + 1] = offF[w] + (long long)m[w] * c->n_w[w];
        offQ[w + 1] = offQ[w] + m[w];
    }
    c->mmaxT = mmax;
    c->sizeFT = offF[c->nwin];
    c->nptsT = offQ[c->nwin];
    std::vector<double> Rh(R, R + c->sizeFT);
    TRY(upload(&c->d_mT, m, s));
    TRY(upload(&c->d_offFT, offF, s));
    TRY(upload(&c->d_offQT, offQ, s));
    TRY(upload(&c->d_FT, Rh, s));
    const bool mixed = c->precision == LRES_MIXED;
    TRY(dalloc((char**)&c->d_qT, (size_t)c->npoles * std::max<long long>(c->nptsT, 1) * (mixed ? 8 : 16)));
    c->have_trace = true;
    if (mixed) {
        TRY(dalloc(&c->d_FhatT32, c->sizeFT));
        TRY(trace_standard_form(c, s));
    } else if (needs_standard_form(c)) {
        TRY(dalloc(&c->d_FhatT64, c->sizeFT));
        TRY(trace_standard_form(c, s));
    }
    if (c->tri_alloc) {
        TRY(build_row_items(c, m, c->ri_tr, s));
        TRY(dalloc((char**)&c->d_Ytr, (mixed ? sizeof(float) : sizeof(double)) * (size_t)std::max<long long>(c->sizeFT, 1)));
        if (c->tri_ready) TRY(tri_rows(c, true, s));
    }
    LRES_CUDA_TRY(cudaStreamSynchronize(s));
    return LRES_OK;
}

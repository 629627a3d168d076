/*
 * lres_gb300.h — C ABI of the GB300 (sm_103a) LRes-DFT LCAO window solve.
 *
 * Plain C: fixed-width integers, doubles and raw pointers; no C++ or torch types.
 * Every function returns 0 (LRES_OK) or a negative LRES_E* code; the message of the
 * last failure on the calling thread is available from lres_last_error().  No
 * exception crosses the ABI.  A context is bound to the CUDA device that was current
 * when it was created and is not thread-safe: calls on one context must not overlap.
 * `stream` arguments are cudaStream_t values passed as void* (NULL = legacy default
 * stream); every call is stream-ordered and returns after enqueueing its work, except
 * calls that hand results back in host memory, which synchronise that stream.
 *
 * Conventions of the data (all identical to the reference's):
 *   grid index    ravel of (i, j, k) with k fastest, shape (n1, n2, n3)
 *   CSR arrays    int64 indptr / indices (sorted within rows), float64 values
 *   windows       Wflat/Woff: basis functions of window w are Wflat[Woff[w]:Woff[w+1]] (ascending)
 *   ownership     Oflat/Ooff: grid points owned by window w (disjoint, covering the grid)
 *   density       electrons / bohr^3 with the spin factor 2 included (lrft/lcao3d.py:456)
 *
 * Reference interfaces replaced (albert-hzbn/LResDFT):
 *   lres_ctx_create + lres_set_potential + lres_pass   replace one call of
 *       _lrft_cpp.lrft_windows (src/lrft_cpp.cpp:129-233), bound at lrft/lcao3d.py:359-366,
 *       and the host H(v) assembly LCAOBasis.H (lrft/lcao3d.py:98-100).  The eigenpair
 *       outputs (lam, c, y2) of lrft_windows have no counterpart: the pole route yields the
 *       window density, electron count and band energy directly (see lres_pass).
 *   lres_set_hamiltonian_csr    the CSR H argument of lrft_windows (Hp, Hi, Hv).
 *   lres_inertia / lres_min_eig the role of lam.min() in the warm/cold decisions of
 *       LRFTLCAOCpp._density (lrft/lcao3d.py:420,450-451).
 *   lres_voronoi_owner          the ownership loop of LRFTLCAO.__init__ (lrft/lcao3d.py:139-151).
 *   lres_lda_xc                 lrft/three_d.py:132-148
 *   lres_hartree                lrft/three_d.py:122-129
 *   lres_ion_potential          lrft/three_d.py:102-112,119 (erf part; no GTH short-range term)
 *   lres_basis_build / _fetch   the sparse assembly of LCAOBasis (lrft/lcao3d.py:86-96), on the host
 *   lres_basis_tabulate         the tabulation loop of LCAOBasis.__init__ (lrft/lcao3d.py:61-84), on the GPU
 *   lres_ks_density             ks_density (src/lrft_cpp.cpp:235-284) / ks_lcao (lrft/lcao3d.py:110-117)
 */
#ifndef LRES_GB300_H
#define LRES_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    LRES_OK = 0,
    LRES_EINVAL = -22,     /* bad argument or inconsistent input */
    LRES_ENOMEM = -12,     /* allocation failed (device; host memory for lres_basis_build) */
    LRES_ECUDA = -5,       /* CUDA runtime error */
    LRES_ENUMERIC = -33,   /* a zero or non-finite pivot in some window (per-window status kept) */
    LRES_ESTATE = -71      /* call out of order (e.g. lres_pass before a Hamiltonian was set) */
};

enum { LRES_FP64 = 0, LRES_MIXED = 1 };

/* Routes of the pole solves (lres_set_route).
 *   LRES_ROUTE_LDL      one fused pivot-free LDL^T per (window, pole) of the augmented matrix
 *                       [[z S_W - H_W, F_W], [F_W^T, 0]] (window_ldl.cu): O(n^3) per pole.
 *   LRES_ROUTE_TRIDIAG  the standard-form window A = L^-1 H_W L^-T reduced once per
 *                       Hamiltonian to tridiagonal form T = Q^T A Q (Householder), the owned
 *                       rows carried through the reflectors (Y = F^ Q), then each pole is a
 *                       tridiagonal LDL^T of z I - T and one forward sweep per row (O(n)):
 *                       the mu trials of a density call cost O(P m n) each (tridiag.cu).
 * Both evaluate the same resolvent quadratic forms; the default is the tridiagonal route
 * unless the context has fewer than 4 windows or windows too large for its shared-memory
 * panels. */
enum { LRES_ROUTE_LDL = 0, LRES_ROUTE_TRIDIAG = 1 };

typedef struct lres_ctx lres_ctx;

/* System description, host pointers; copied to the device by lres_ctx_create. */
typedef struct {
    int64_t nb;            /* basis functions */
    int64_t shape[3];      /* grid shape; ng = shape[0]*shape[1]*shape[2] */
    double cell[3];        /* orthorhombic box lengths (bohr) */
    double dV;             /* grid volume element */
    /* basis values on the grid: CSR, ng rows x nb columns */
    const int64_t* Xp; const int64_t* Xi; const double* Xv;
    /* overlap S and kinetic T = X^T T_FD X dV: CSR, nb x nb.  T may be NULL, then the
       Hamiltonian can only be given with lres_set_hamiltonian_csr. */
    const int64_t* Sp; const int64_t* Si; const double* Sv;
    const int64_t* Tp; const int64_t* Ti; const double* Tv;
    /* functions grouped by atom: group g owns functions [gptr[g], gptr[g+1]), at most
       8 per group, all with the same support on the grid */
    int64_t ngroups; const int64_t* gptr;
    /* windows and owned grid points */
    int64_t nwin;
    const int64_t* Wflat; const int64_t* Woff;
    const int64_t* Oflat; const int64_t* Ooff;
} lres_system_desc;

const char* lres_version(void);
const char* lres_last_error(void);

/* Create a context: uploads the system, builds the dense window overlaps S_W and the
 * owned-point basis blocks F_W = X[own(w), W]^T, and for LRES_MIXED the FP64 Cholesky
 * inverses L_W^-1 and F^_W = L_W^-1 F_W.  M is the (even) number of poles. */
int lres_ctx_create(lres_ctx** out, const lres_system_desc* desc, int precision, int M, void* stream);
int lres_ctx_destroy(lres_ctx* ctx);

/* Set the Hamiltonian H = T + X^T diag(v) X dV from the local potential v[ng]
 * (host or device pointer as v_on_device says): assembled on the GPU by atom pairs,
 * then gathered into the dense window blocks H_W (and H^_W = L^-1 H_W L^-T in
 * LRES_MIXED).  Requires T in the system description. */
int lres_set_potential(lres_ctx* ctx, const double* v, int v_on_device, void* stream);

/* Set the Hamiltonian from a host CSR matrix (any sorted pattern inside the window
 * blocks), e.g. one built on the host with extra nonlocal terms. */
int lres_set_hamiltonian_csr(lres_ctx* ctx, const int64_t* Hp, const int64_t* Hi, const double* Hv, void* stream);

/* One pole pass at chemical potential mu and filter edge e_lo (e_lo < mu): all
 * windows x M/2 upper-half-plane poles z_j = c + R exp(i pi (2j+1)/M), c = (mu+e_lo)/2,
 * R = (mu-e_lo)/2, weights w_j = R exp(i pi (2j+1)/M) / M.  Writes
 *   dens[ng]  spin-summed density on the grid (host or device pointer per dens_on_device;
 *             NULL to skip the copy-out, the device copy stays in the context)
 *   out[0]    electron count N(mu) = dV sum dens
 *   out[1]    band energy E_band = 2 sum_w tr(P^lambda_W O_W)
 *   out[2]    status bits of the window kernels: 1 = some window met a zero or non-finite
 *             pivot, 2 = some window exceeded the launch limits; 0 when clean
 * and returns LRES_ENUMERIC (bit 1) or LRES_EINVAL (bit 2) when out[2] != 0. */
int lres_pass(lres_ctx* ctx, double mu, double e_lo, double* dens, int dens_on_device, double* out, void* stream);

/* The pass of lres_pass without any host synchronisation or host memory: pole nodes and
 * weights are computed on the device, d_out[0..1] (device) receives N(mu) and E_band, the
 * density stays in the context (lres_density_ptr).  Enqueues kernels and memsets only, so
 * lres_set_potential(v on device) + lres_pass_async can be captured in a CUDA graph and
 * replayed (after one ordinary call has set the kernel attributes).  Check the kernel
 * status afterwards with lres_status. */
int lres_pass_async(lres_ctx* ctx, double mu, double e_lo, double* d_out, void* stream);
/* Status bits of the most recent pass (see lres_pass out[2]); synchronises the stream. */
int lres_status(lres_ctx* ctx, int32_t* status, void* stream);
/* Device address of the context's density array (ng doubles, valid until destroy). */
int lres_density_ptr(lres_ctx* ctx, const double** d_dens);

/* Tile configuration of the pole solves, force_config in [0, 5]; -1 times every
 * configuration on the current Hamiltonian and keeps the fastest eligible one for this context.
 * On the LDL^T route it is the tile configuration of the fused pole kernel, timed with full
 * passes at (mu, e_lo) (LRES_MIXED configuration 4 runs the chunk products on the tensor cores,
 * tcgen05 with a 3xTF32 split; it is timed but kept only when forced, its error being ~5x that
 * of the FP32 configurations).  On the tridiagonal route it selects the reduction (working
 * copy in L2, or with LRES_MIXED the window's lower triangle in shared memory), the row
 * application (rows resident in shared memory with LRES_MIXED, or one row per thread), their
 * panel widths and rows per item (six measured variants, each capped by the shared memory),
 * timed as reduction + rows (mu, e_lo unused).
 * *chosen (may be NULL) receives the choice, ms_per_config[6] (may be NULL) the measured times. */
int lres_autotune(lres_ctx* ctx, double mu, double e_lo, int32_t force_config, int32_t* chosen,
                  double* ms_per_config, void* stream);

/* Route of the pole solves (LRES_ROUTE_LDL or LRES_ROUTE_TRIDIAG, see above).  Switching
 * to the tridiagonal route allocates its buffers and, when a Hamiltonian is set, reduces
 * it (LRES_EINVAL if the windows are too large for the reduction); the tile configuration
 * of lres_autotune applies to the LDL^T kernel.  On the tridiagonal route lres_inertia and
 * lres_min_eig count by Sturm sequences of T - sigma, T being congruent to the pencil
 * (H_W, S_W) (for LRES_MIXED: of the FP32 standard form). */
int lres_set_route(lres_ctx* ctx, int32_t route, void* stream);
int lres_get_route(lres_ctx* ctx, int32_t* route);

/* Kernel of the FP32 standard form A = L^-1 H_W L^-T of the LRES_MIXED tridiagonal route:
 * LRES_SF_SIMT, batched FP32 GEMMs on the SIMT pipes; LRES_SF_TENSOR, the same products on
 * the tensor cores (tcgen05.mma kind::tf32, operands split into TF32 pairs, hi.hi + hi.lo +
 * lo.hi, accumulated from zero per 32-term chunk in tensor memory and across chunks in FP32,
 * as the SIMT kernels block their sums).  Takes effect at the next Hamiltonian
 * (lres_set_potential / lres_set_hamiltonian_csr / lres_set_windows); no other route or
 * precision uses it.  A timed-out completion wait of the tensor cores is reported by the
 * next pass as status bit 4 (LRES_EINVAL). */
enum { LRES_SF_SIMT = 0, LRES_SF_TENSOR = 1 };
int lres_set_standard_form_kernel(lres_ctx* ctx, int32_t kind);
int lres_get_standard_form_kernel(lres_ctx* ctx, int32_t* kind);

/* Device time (ms, CUDA events on the launching stream) of the most recent launch of:
 * ms[0] the pole kernel (LDL^T kernel, or the shifted tridiagonal solves), ms[1] the pole
 * sums, ms[2] the H(v) assembly, ms[3] the window gather, ms[4] the standard-form transform,
 * ms[5] the inertia kernel, ms[6] the tridiagonal reduction, ms[7] the rows through its
 * reflectors; -1 for one not launched yet.  Fills min(n, 8) entries, waits for their end
 * events. */
int lres_timings(lres_ctx* ctx, double* ms, int n);

/* Per-window electron counts and band energies of the last pass (host arrays of nwin). */
int lres_window_sums(lres_ctx* ctx, double* n_w, double* e_w);

/* Sylvester inertia of every window at shift sigma: below[w] = number of generalised
 * eigenvalues of (H_W, S_W) below sigma (FP64 pivot-free LDL^T of sigma S_W - H_W).
 * below may be NULL; *total receives the sum over windows. */
int lres_inertia(lres_ctx* ctx, double sigma, int32_t* below, int64_t* total, void* stream);

/* Smallest generalised eigenvalue over all windows by bisection on the inertia count,
 * starting from the bracket [lo, hi] (widened if needed), to absolute width tol. */
int lres_min_eig(lres_ctx* ctx, double lo, double hi, double tol, double* lam_min, void* stream);

/* Voronoi ownership of the grid (lrft/lcao3d.py:139-151): owner[p] = index of the
 * nearest centre in minimum-image distance, the lowest index on exact ties, with the
 * reference's floating-point operation order.  Host arrays in and out. */
int lres_voronoi_owner(const int64_t shape[3], const double cell[3], int64_t ncent, const double* centres,
                       int32_t* owner);

/* Window inertia counts that allocate nothing — no counterpart in the reference.
 * For callers that cannot allocate device memory themselves: hosts that own all GPU
 * memory through their own arena or caching allocator, or loops that cannot afford the
 * device-wide synchronisation of cudaMalloc / cudaFree.  Counts by a pivot-free FP64
 * LDL^T of sigma S_W - H_W (Sylvester inertia), computed from caller-provided device
 * arrays: n_w[nwin] (int32 window dimensions), offC[nwin] (int64 offsets of each
 * window's column-major n_w x n_w block in H and S), dense window blocks H and S
 * (float64), output below[nwin] (int32, device) = number of generalised eigenvalues of
 * (H_W, S_W) below sigma.  nmax bounds every n_w.
 * Scratch comes from one fixed array inside the library (16.5 MiB, held by every GPU
 * that loads it until the process exits): at most 65536 windows and nmax <= 512 per
 * call, larger requests return LRES_EINVAL (so does a window larger than the nmax
 * given).  The array holds eight factorisation workspaces, so the windows are spread
 * over eight CTAs: on many windows this runs several times slower than lres_inertia.
 * Returns LRES_ENUMERIC when some window meets a zero or non-finite pivot (NaN or Inf in
 * H or S, or sigma exactly on an eigenvalue); its counts are then meaningless.  The
 * first call on each device looks up the array's device address (once per device).  All
 * calls on a device share the array and reset its work queue and status at the start:
 * calls that overlap on the GPU race and must be serialised by the caller (one stream, or
 * events).  Every call waits for the stream to read the kernel status back, so it cannot
 * be captured in a CUDA graph. */
int lres_inertia_noalloc(int32_t nwin, const int32_t* n_w, const int64_t* offC, const double* H, const double* S,
                         double sigma, int32_t* below, int32_t nmax, void* stream);

/* Replaces the dense window matrices directly (H and/or S may be NULL to keep the current
 * one): float64 arrays in the window layout of the context — window w's column-major
 * n_w x n_w block at offset offC[w] = sum_{u<w} n_u^2, windows in the order of Woff.  The
 * LRES_MIXED path refactors S_W (standard form) when S is given.  The blocks stay in place
 * until the next lres_set_potential / lres_set_hamiltonian_csr, which re-gather H_W only.
 * The reference builds H_W, S_W only by gather (src/lrft_cpp.cpp:116-127); this entry makes
 * the window matrices inputs of their own, as the adjoint below differentiates them. */
int lres_set_windows(lres_ctx* ctx, const double* HW, const double* SW, int on_device, void* stream);

/* Device addresses of the context's dense window matrices H_W and S_W (float64, window
 * layout as lres_set_windows; valid until destroy, contents change with every update). */
int lres_window_ptrs(lres_ctx* ctx, const double** d_HW, const double** d_SW);

/* Adjoint of the band energy at fixed electron number (e_lo fixed), at (mu, e_lo) on the
 * current window matrices.  The reference has no gradient code; its finite-M
 * Hellmann-Feynman check (tests/test_lrft.py:59-79) is the template.  Runs one pole pass
 * whose factors are kept (pole batches of whole windows, as many as free device memory
 * admits), back-substitutes Z_k = (z_k S_W - H_W)^-1 F_W^T, accumulates Re sum_k c_k Z_k Z_k^T
 * for c in {w, w z, w z^2} and returns, each optional:
 *   dv[ng]           dE_band/dv(r) at fixed N (the grid local potential through
 *                    H = T + X^T diag(v) X dV, lrft/lcao3d.py:98-100);
 *   dHW, dSW[sizeC]  dE_band/dH_W and dE_band/dS_W at fixed N, window layout as
 *                    lres_set_windows (each window's matrices taken as independent);
 *   out[6]           N(mu), E_band(mu), dN/dmu, dE/dmu, kappa = (dE/dmu)/(dN/dmu), status.
 * The pass also leaves the density in the context (lres_density_ptr).  Synchronises. */
int lres_adjoint(lres_ctx* ctx, double mu, double e_lo, double* dv, int dv_on_device, double* dHW, double* dSW,
                 int dW_on_device, double* out, void* stream);

/* Trace rows — no counterpart in the reference.  N(mu), E_band and the adjoint depend on
 * the owned-point rows F_W = X[own(B), W] only through F_W^T F_W, so on fine grids
 * (|own(B)| >> n_W) a factor R_W with R_W^T R_W = F_W^T F_W and at most n_W rows gives the
 * same sums with far fewer rows.  lres_owned_gram writes K_W = F_W^T F_W (window layout,
 * n_W x n_W column-major at offC[w]; host or device).  lres_set_trace_rows installs
 * r_w[w] rows per window, R = the r_w x n_W blocks (column-major, leading dimension r_w[w])
 * concatenated in window order (host); NULL r_w removes them.  While installed, lres_pass
 * with dens == NULL and lres_adjoint run over the trace rows (no density is produced and
 * the context's density array is left as it was); passes that return a density use the
 * owned points. */
int lres_owned_gram(lres_ctx* ctx, double* K, int on_device, void* stream);
int lres_set_trace_rows(lres_ctx* ctx, const int32_t* r_w, const double* R, void* stream);

/* Host assembly of an atom-grouped grid basis (no GPU involved) — replaces the sparse
 * assembly of LCAOBasis.__init__ and LCAOBasis._matrices (lrft/lcao3d.py:86-96; T_FD of
 * lrft/three_d.py:151-164).  Input: ngroups groups of functions, group g owning functions
 * [gptr[g], gptr[g+1]) (1..8) that share one support; cnt[g] tabulated points per group,
 * their grid indices idx[] concatenated in group order (duplicates allowed: periodic
 * images of one point, summed in the order given), values val[] concatenated in group
 * order, each group function-major (function f of group g at point e: val[voff_g + f *
 * cnt[g] + e]).  Builds X (ng x nb), S = dV X^T X and T = dV X^T T_FD X, where T_FD is
 * the periodic 7-point stencil with diagonal t_diag and off-diagonal t_off (3/dx^2 and
 * -0.5/dx^2 for -Lap/2).  Every entry is the sum of the reference's scipy products in
 * their order (ascending shared index, each product rounded, zero sums dropped), so S
 * and T equal the reference's bit for bit; threads (nthreads, 0 = all cores) only split
 * the rows.  nnz[3] receives the entries of X, S and T; lres_basis_fetch copies out X as
 * CSC (Xp[nb+1], columns = functions) and CSR (Xrp[ng+1]) and S, T as CSR (nb+1
 * pointers), all with sorted indices; any triple may be NULL to skip it. */
typedef struct lres_basis lres_basis;
int lres_basis_build(lres_basis** out, int64_t ngroups, const int64_t* gptr, const int64_t* cnt,
                     const int64_t* idx, const double* val, const int64_t shape[3], double dV, double t_diag,
                     double t_off, int nthreads, int64_t* nnz);
int lres_basis_fetch(const lres_basis* b, int64_t* Xp, int64_t* Xi, double* Xv, int64_t* Xrp, int64_t* Xri,
                     double* Xrv, int64_t* Sp, int64_t* Si, double* Sv, int64_t* Tp, int64_t* Ti, double* Tv);
int lres_basis_free(lres_basis* b);

/* Tabulation of the atom-centred grid basis on the GPU (lrft/lcao3d.py:61-84), the input of
 * lres_basis_build.  Atom a at pos[3a..3a+2] has ns[a] s exponents then np[a] p exponents in
 * exps (atoms concatenated), 1..8 functions (s: exp(-e r^2) cut(r); p: x, y, z times
 * exp(-e r^2) cut(r); cut(r) = (1 - (r / rcut)^2)^2).  Its points are those of the cube
 * round(R / dx) + [-ceil(rcut / dx), ceil(rcut / dx)]^3 (lexicographic) whose minimum-image
 * distance (cell[]) is below rcut, in cube order; each function is normalised on the grid
 * (f / sqrt(sum f^2 dV)).  The operations are the reference's, rounded in its order: the
 * points are the same, the values differ from numpy's by CUDA's exp (a few ulp) and by the
 * order of the normalisation sum.  Host arrays.  Two calls: idx = val = NULL fills cnt[natoms]
 * (points per atom); then idx[sum cnt] (grid indices) and val[sum cnt * functions] (atom by
 * atom, function by function) are filled.  Synchronous on the current device. */
int lres_basis_tabulate(int64_t natoms, const double* pos, const int32_t* ns, const int32_t* np,
                        const double* exps, const int64_t shape[3], const double cell[3], double dx, double rcut,
                        double dV, int64_t* cnt, int64_t* idx, double* val);

/* Dense Kohn-Sham LCAO of the whole cell (ks_lcao, lrft/lcao3d.py:110-117; ks_density,
 * src/lrft_cpp.cpp:235-284): the generalised eigenproblem H C = S C diag(w) (H, S: nb x nb
 * CSR), w[0..nocc] = the lowest nocc + 1 eigenvalues, dens[ng] = 2 sum_{i < nocc}
 * (X[r,:] C_i)^2 with X the ng x nb CSR basis, *e_band = 2 sum_{i < nocc} w_i.  Host arrays;
 * synchronous on the current device.  The dense eigensolver is cuSOLVER's dsygvd, opened at
 * run time (LRES_ESTATE if libcusolver is absent); LRES_ENUMERIC if S is not positive
 * definite.  The oracle side of LRes(R_w >= cell) = KS, not the window solve. */
int lres_ks_density(int64_t nb, const int64_t* Hp, const int64_t* Hi, const double* Hv, const int64_t* Sp,
                    const int64_t* Si, const double* Sv, int64_t ng, const int64_t* Xp, const int64_t* Xi,
                    const double* Xv, int32_t nocc, double* dens, double* w, double* e_band);

/* Grid kernels on device arrays of ng doubles (context supplies shape and cell). */
int lres_lda_xc(lres_ctx* ctx, const double* dens, double* exc, double* vxc, void* stream);
int lres_hartree(lres_ctx* ctx, const double* dens, double* vh, void* stream);
int lres_ion_potential(lres_ctx* ctx, int64_t natoms, const double* pos, const double* Z, const double* rc,
                       double* vion, void* stream);

#ifdef __cplusplus
}
#endif
#endif

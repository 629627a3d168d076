// Tabulation of the atom-centred grid basis on the GPU (lrft/lcao3d.py:61-84): for every
// atom the grid points of the cube c + [-rad, rad]^3 (c = round(R / dx)) whose minimum-image
// distance r from the atom is below rcut, in cube order, with the s functions
// exp(-a r^2) cut(r) and the p functions d_x g, d_y g, d_z g (g = exp(-a r^2) cut(r)),
// cut(r) = (1 - (r / rcut)^2)^2, each normalised on the grid, f / sqrt(sum f^2 dV).
//
// Every operation is the reference's, in its order, rounded as numpy rounds it (explicit
// _rn intrinsics: no contraction into FMAs), so the points are the same and the values
// differ only where CUDA's exp and numpy's exp differ (a few ulp) and in the order of the
// sum of squares of the normalisation (numpy sums pairwise; here each thread sums its
// points in order and the threads' sums are added in a fixed tree).
//
// One CTA per atom.  Points are kept in cube order by an ordered compaction per chunk of
// the cube (warp ballots + a scan over the warps).  Output: the (cnt, idx, val) arrays of
// lres_basis_build (values atom by atom, function by function, point by point).
#include "common.cuh"
#include "lres_internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace lres {
namespace {

constexpr int kTabNT = 256;
constexpr int kMaxFn = 8;                       // functions per atom (s + 3 p) at most

struct TabParams {
    int natoms;
    const double* pos;        // [natoms][3]
    const int* ns;            // s exponents per atom
    const int* np;            // p exponents per atom
    const int* eoff;          // first exponent of each atom in exps (s then p)
    const double* exps;
    int rad;
    int n1, n2, n3;
    double L1, L2, L3, dx, rcut, dV;
    const long long* base;    // first point of each atom (count pass: unused)
    long long* cnt;           // points per atom (count pass)
    long long* idx;           // grid index of every point (fill pass)
    double* val;              // values (fill pass), unnormalised then normalised
    const long long* vbase;   // first value of each atom
};

// Minimum image of one displacement component, d - L round(d / L) (np.round: half to even).
__device__ __forceinline__ double min_image(double d, double L) {
    return __dsub_rn(d, __dmul_rn(L, rint(__ddiv_rn(d, L))));
}

// The point of cube offset o (lexicographic over [-rad, rad]^3) of the atom at R with cube
// centre c: displacement d, distance r; returns whether r < rcut.
__device__ __forceinline__ bool cube_point(const TabParams& p, const double R[3], const long long c[3], long long o,
                                           long long P[3], double d[3], double& r) {
    const long long side = 2 * p.rad + 1;
    const long long oi = o / (side * side), oj = (o / side) % side, ok = o % side;
    P[0] = c[0] + oi - p.rad;
    P[1] = c[1] + oj - p.rad;
    P[2] = c[2] + ok - p.rad;
    const double L[3] = {p.L1, p.L2, p.L3};
#pragma unroll
    for (int a = 0; a < 3; ++a) d[a] = min_image(__dsub_rn(__dmul_rn((double)P[a], p.dx), R[a]), L[a]);
    r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2])));
    return r < p.rcut;
}

__device__ __forceinline__ long long floor_mod(long long a, long long n) {
    const long long m = a % n;
    return m < 0 ? m + n : m;
}

// Sum over the CTA in a fixed order (every thread gets the same value).
__device__ __forceinline__ double cta_sum(double x, double* red) {
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    double s = red[0];
    for (int w = 1; w < kTabNT / 32; ++w) s += red[w];
    return s;
}

template <bool FILL>
__global__ void __launch_bounds__(kTabNT) basis_tab_kernel(TabParams p) {
    __shared__ int wcount[kTabNT / 32];
    __shared__ double red[kTabNT / 32];
    const int a = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double R[3] = {p.pos[3 * a], p.pos[3 * a + 1], p.pos[3 * a + 2]};
    long long c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = (long long)rint(__ddiv_rn(R[k], p.dx));
    const long long side = 2 * p.rad + 1, ncube = side * side * side;
    const int ns = p.ns[a], np = p.np[a], nf = ns + 3 * np;
    const double* ex = p.exps + p.eoff[a];
    const long long n_a = FILL ? p.cnt[a] : 0;
    long long* idx = FILL ? p.idx + p.base[a] : nullptr;
    double* val = FILL ? p.val + p.vbase[a] : nullptr;
    double ss[kMaxFn];
#pragma unroll
    for (int f = 0; f < kMaxFn; ++f) ss[f] = 0.0;
    long long kept = 0;                                   // points kept before this chunk
    for (long long o0 = 0; o0 < ncube; o0 += kTabNT) {
        const long long o = o0 + tid;
        long long P[3] = {0, 0, 0};
        double d[3] = {0.0, 0.0, 0.0}, r = 0.0;
        const bool in = o < ncube && cube_point(p, R, c, o, P, d, r);
        const unsigned m = __ballot_sync(0xffffffffu, in);
        if (lane == 0) wcount[warp] = __popc(m);
        __syncthreads();
        long long before = kept;
        for (int w = 0; w < warp; ++w) before += wcount[w];
        long long total = 0;
        for (int w = 0; w < kTabNT / 32; ++w) total += wcount[w];
        const long long slot = before + __popc(m & ((1u << lane) - 1u));
        if (FILL && in) {
            idx[slot] = (floor_mod(P[0], p.n1) * p.n2 + floor_mod(P[1], p.n2)) * p.n3 + floor_mod(P[2], p.n3);
            const double q = __ddiv_rn(r, p.rcut);
            const double u = __dsub_rn(1.0, __dmul_rn(q, q));
            const double cut = __dmul_rn(u, u);
            const double r2 = __dmul_rn(r, r);
            int f = 0;
            for (int k = 0; k < ns; ++k, ++f) {
                const double v = __dmul_rn(exp(__dmul_rn(-ex[k], r2)), cut);
                val[(long long)f * n_a + slot] = v;
                ss[f] = __dadd_rn(ss[f], __dmul_rn(v, v));
            }
            for (int k = 0; k < np; ++k) {
                const double g = __dmul_rn(exp(__dmul_rn(-ex[ns + k], r2)), cut);
#pragma unroll
                for (int ax = 0; ax < 3; ++ax, ++f) {
                    const double v = __dmul_rn(d[ax], g);
                    val[(long long)f * n_a + slot] = v;
                    ss[f] = __dadd_rn(ss[f], __dmul_rn(v, v));
                }
            }
        }
        kept += total;
        __syncthreads();                                  // wcount is rewritten by the next chunk
    }
    if (!FILL) {
        if (tid == 0) p.cnt[a] = kept;
        return;
    }
    // normalisation: f / sqrt(sum f^2 dV)
    for (int f = 0; f < nf; ++f) {
        const double s = cta_sum(ss[f < kMaxFn ? f : 0], red);
        const double nrm = __dsqrt_rn(__dmul_rn(s, p.dV));
        for (long long k = tid; k < n_a; k += kTabNT) val[(long long)f * n_a + k] = __ddiv_rn(val[(long long)f * n_a + k], nrm);
    }
}

template <class T>
int dcopy(T** d, const std::vector<T>& h) {
    LRES_CUDA_TRY(cudaMalloc(d, sizeof(T) * std::max<size_t>(h.size(), 1)));
    if (!h.empty()) LRES_CUDA_TRY(cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
    return LRES_OK;
}

}  // namespace
}  // namespace lres

using namespace lres;

extern "C" int lres_basis_tabulate(int64_t natoms, const double* pos, const int32_t* ns, const int32_t* np,
                                   const double* exps, const int64_t shape[3], const double cell[3], double dx,
                                   double rcut, double dV, int64_t* cnt, int64_t* idx, double* val) {
    if (natoms <= 0 || !pos || !ns || !np || !exps || !shape || !cell || !cnt || !(dx > 0.0) || !(rcut > 0.0)) {
        lres_set_error("lres_basis_tabulate: bad arguments");
        return LRES_EINVAL;
    }
    if ((idx == nullptr) != (val == nullptr)) {
        lres_set_error("lres_basis_tabulate: idx and val are given together (fill) or not at all (count)");
        return LRES_EINVAL;
    }
    for (int k = 0; k < 3; ++k)
        if (shape[k] < 1 || shape[k] > (1 << 20) || !(cell[k] > 0.0)) {
            lres_set_error("lres_basis_tabulate: bad grid");
            return LRES_EINVAL;
        }
    const double radd = std::ceil(rcut / dx);
    if (!(radd < 512.0)) {
        lres_set_error("lres_basis_tabulate: rcut / dx too large");
        return LRES_EINVAL;
    }
    std::vector<int> hns(natoms), hnp(natoms), eoff(natoms + 1, 0);
    for (int64_t a = 0; a < natoms; ++a) {
        hns[a] = ns[a];
        hnp[a] = np[a];
        if (ns[a] < 0 || np[a] < 0 || ns[a] + 3 * np[a] < 1 || ns[a] + 3 * np[a] > kMaxFn) {
            lres_set_error("lres_basis_tabulate: atom %lld has %d s and %d p exponents (1..%d functions)",
                           (long long)a, ns[a], np[a], kMaxFn);
            return LRES_EINVAL;
        }
        eoff[a + 1] = eoff[a] + ns[a] + np[a];
    }
    std::vector<double> hexps(exps, exps + eoff[natoms]), hpos(pos, pos + 3 * natoms);
    TabParams p{};
    p.natoms = (int)natoms;
    p.rad = (int)radd;
    p.n1 = (int)shape[0];
    p.n2 = (int)shape[1];
    p.n3 = (int)shape[2];
    p.L1 = cell[0];
    p.L2 = cell[1];
    p.L3 = cell[2];
    p.dx = dx;
    p.rcut = rcut;
    p.dV = dV;
    double *dpos = nullptr, *dexps = nullptr, *dval = nullptr;
    int *dns = nullptr, *dnp = nullptr, *deoff = nullptr;
    long long *dcnt = nullptr, *dbase = nullptr, *dvbase = nullptr, *didx = nullptr;
    int rc = LRES_OK;
    auto run = [&]() -> int {
        if (int e = dcopy(&dpos, hpos)) return e;
        if (int e = dcopy(&dexps, hexps)) return e;
        if (int e = dcopy(&dns, hns)) return e;
        if (int e = dcopy(&dnp, hnp)) return e;
        if (int e = dcopy(&deoff, eoff)) return e;
        LRES_CUDA_TRY(cudaMalloc(&dcnt, sizeof(long long) * natoms));
        p.pos = dpos;
        p.exps = dexps;
        p.ns = dns;
        p.np = dnp;
        p.eoff = deoff;
        p.cnt = dcnt;
        basis_tab_kernel<false><<<(unsigned)natoms, kTabNT>>>(p);
        LRES_CUDA_TRY(cudaGetLastError());
        std::vector<long long> hcnt(natoms);
        LRES_CUDA_TRY(cudaMemcpy(hcnt.data(), dcnt, sizeof(long long) * natoms, cudaMemcpyDeviceToHost));
        for (int64_t a = 0; a < natoms; ++a) cnt[a] = hcnt[a];
        if (!idx) return LRES_OK;
        std::vector<long long> base(natoms + 1, 0), vbase(natoms + 1, 0);
        for (int64_t a = 0; a < natoms; ++a) {
            base[a + 1] = base[a] + hcnt[a];
            vbase[a + 1] = vbase[a] + hcnt[a] * (hns[a] + 3 * hnp[a]);
        }
        if (int e = dcopy(&dbase, base)) return e;
        if (int e = dcopy(&dvbase, vbase)) return e;
        LRES_CUDA_TRY(cudaMalloc(&didx, sizeof(long long) * std::max<long long>(base[natoms], 1)));
        LRES_CUDA_TRY(cudaMalloc(&dval, sizeof(double) * std::max<long long>(vbase[natoms], 1)));
        p.base = dbase;
        p.vbase = dvbase;
        p.idx = didx;
        p.val = dval;
        basis_tab_kernel<true><<<(unsigned)natoms, kTabNT>>>(p);
        LRES_CUDA_TRY(cudaGetLastError());
        LRES_CUDA_TRY(cudaMemcpy(idx, didx, sizeof(long long) * base[natoms], cudaMemcpyDeviceToHost));
        LRES_CUDA_TRY(cudaMemcpy(val, dval, sizeof(double) * vbase[natoms], cudaMemcpyDeviceToHost));
        return LRES_OK;
    };
    rc = run();
    for (void* q : {(void*)dpos, (void*)dexps, (void*)dval, (void*)dns, (void*)dnp, (void*)deoff, (void*)dcnt,
                    (void*)dbase, (void*)dvbase, (void*)didx})
        if (q) cudaFree(q);
    return rc;
}

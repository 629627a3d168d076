// Host assembly of the atom-grouped grid basis: X (CSC and CSR), S = dV X^T X and
// T = dV X^T T_FD X, with T_FD the periodic 7-point -Lap/2 (lrft/lcao3d.py:86-96,
// lrft/three_d.py:151-164).  See lres_basis_build in include/lres_gb300.h.
//
// The reference forms these with scipy.sparse: X from COO triplets (duplicates summed),
// S = (X.T @ X) * dV, T = (X.T @ (T_FD @ X)) * dV.  scipy's sparse product sums every
// output entry (i, j) sequentially over the shared index in ascending order, starting
// from 0, rounds each product before adding it, and keeps an entry only if its sum is
// non-zero.  Here every sum runs over the same terms in the same order, so S and T are
// the reference's bit for bit (the file is compiled without FMA contraction).  What
// differs is the organisation: the functions of one atom share one support, so the sums
// are formed per atom pair as 8-lane blocks (no sparse merge per function), atoms are
// spread over threads, and every output row is written by one thread (deterministic).
#include "lres_gb300.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <new>
#include <numeric>
#include <thread>
#include <vector>

extern "C" void lres_set_error(const char* fmt, ...);

namespace {

constexpr int kMaxLanes = 8;   // functions per group

struct Rows {                // one group's output rows (S or T)
    std::vector<int64_t> cnt;     // entries per function row
    std::vector<int64_t> col;
    std::vector<double> val;
};

template <class F>
void parallel_for(int nthreads, int64_t n, F&& body) {
    // dynamic distribution of [0, n); body(i, thread) must not depend on the schedule
    // (an allocation failure in a worker is carried to the caller as std::bad_alloc)
    std::atomic<int64_t> next{0};
    std::atomic<bool> failed{false};
    auto run = [&](int t) {
        try {
            for (int64_t i; !failed.load() && (i = next.fetch_add(1)) < n;) body(i, t);
        } catch (const std::bad_alloc&) {
            failed = true;
        }
    };
    if (nthreads <= 1 || n <= 1) {
        run(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 1; t < nthreads; ++t) th.emplace_back(run, t);
        run(0);
        for (auto& x : th) x.join();
    }
    if (failed) throw std::bad_alloc();
}

}  // namespace

struct lres_basis {
    int64_t nb = 0, ng = 0, ngroups = 0;
    int nthreads = 1, lanes = 1;
    std::vector<int64_t> gptr;
    // group supports: grid indices ascending, values in `lanes` lanes per point
    std::vector<int64_t> sptr, sidx;
    std::vector<double> sval;            // [slot][lanes]
    // point -> (group, slot), groups ascending within a point
    std::vector<int64_t> pptr;
    std::vector<int32_t> pgrp;
    std::vector<int64_t> pslot;
    std::vector<Rows> S, T;               // rows of each group
};

// The assembly with L value lanes per grid point (L = the largest group; lanes past a
// group's own functions hold zeros).
template <int L>
int build(lres_basis** out, int64_t ngroups, const int64_t* gptr, const int64_t* cnt, const int64_t* idx,
          const double* val, const int64_t shape[3], double dV, double t_diag, double t_off, int nthreads,
          int64_t* nnz) {
    const int64_t n1 = shape[0], n2 = shape[1], n3 = shape[2], ng = n1 * n2 * n3;
    lres_basis* b = nullptr;
    try {
        b = new lres_basis;
        b->nb = gptr[ngroups];
        b->ng = ng;
        b->ngroups = ngroups;
        b->nthreads = nthreads;
        b->lanes = L;
        b->gptr.assign(gptr, gptr + ngroups + 1);
        std::vector<int64_t> eoff(ngroups + 1, 0), voff(ngroups + 1, 0);
        for (int64_t g = 0; g < ngroups; ++g) {
            eoff[g + 1] = eoff[g] + cnt[g];
            voff[g + 1] = voff[g] + (gptr[g + 1] - gptr[g]) * cnt[g];
        }

        // ---- supports: sort each group's points by grid index (stable: duplicates in
        // the order given), sum duplicates sequentially as scipy's sum_duplicates does
        std::vector<std::vector<int64_t>> gidx(ngroups);
        std::vector<std::vector<double>> gval(ngroups);
        parallel_for(nthreads, ngroups, [&](int64_t g, int) {
            const int64_t c = cnt[g], nf = gptr[g + 1] - gptr[g];
            const int64_t* ix = idx + eoff[g];
            const double* v = val + voff[g];
            std::vector<int64_t> perm(c);
            std::iota(perm.begin(), perm.end(), 0);
            std::stable_sort(perm.begin(), perm.end(), [&](int64_t a, int64_t q) { return ix[a] < ix[q]; });
            auto& oi = gidx[g];
            auto& ov = gval[g];
            for (int64_t k = 0; k < c;) {
                const int64_t r = ix[perm[k]];
                double acc[L] = {0};
                for (int f = 0; f < nf; ++f) acc[f] = v[f * c + perm[k]];
                int64_t j = k + 1;
                for (; j < c && ix[perm[j]] == r; ++j)
                    for (int f = 0; f < nf; ++f) acc[f] += v[f * c + perm[j]];
                oi.push_back(r);
                ov.insert(ov.end(), acc, acc + L);
                k = j;
            }
        });
        b->sptr.assign(ngroups + 1, 0);
        for (int64_t g = 0; g < ngroups; ++g) b->sptr[g + 1] = b->sptr[g] + (int64_t)gidx[g].size();
        const int64_t nslot = b->sptr[ngroups];
        b->sidx.resize(nslot);
        b->sval.resize((size_t)nslot * L);
        parallel_for(nthreads, ngroups, [&](int64_t g, int) {
            std::copy(gidx[g].begin(), gidx[g].end(), b->sidx.begin() + b->sptr[g]);
            std::copy(gval[g].begin(), gval[g].end(), b->sval.begin() + b->sptr[g] * L);
            std::vector<int64_t>().swap(gidx[g]);
            std::vector<double>().swap(gval[g]);
        });

        // ---- point -> (group, slot), groups ascending
        b->pptr.assign(ng + 1, 0);
        for (int64_t s = 0; s < nslot; ++s) ++b->pptr[b->sidx[s] + 1];
        for (int64_t r = 0; r < ng; ++r) b->pptr[r + 1] += b->pptr[r];
        b->pgrp.resize(nslot);
        b->pslot.resize(nslot);
        {
            std::vector<int64_t> cur(b->pptr.begin(), b->pptr.end() - 1);
            for (int64_t g = 0; g < ngroups; ++g)
                for (int64_t s = b->sptr[g]; s < b->sptr[g + 1]; ++s) {
                    const int64_t at = cur[b->sidx[s]]++;
                    b->pgrp[at] = (int32_t)g;
                    b->pslot[at] = s;
                }
        }

        // ---- Y = T_FD X per point, grouped: row r sums coef(r, c) * X[c, :] over the
        // sorted stencil columns c of row r (the 6 neighbours, duplicates merged when an
        // axis has fewer than 3 points, plus the diagonal)
        const int64_t nchunk = std::min<int64_t>(ng, (int64_t)nthreads * 16);
        std::vector<std::vector<int64_t>> ycnt(nchunk);
        std::vector<std::vector<int32_t>> ygrp(nchunk);
        std::vector<std::vector<double>> yval(nchunk);
        struct Scratch {
            std::vector<int32_t> loc;
            std::vector<int32_t> touched, order;
            std::vector<double> acc;
        };
        std::vector<Scratch> scr(nthreads);
        for (auto& s : scr) s.loc.assign(ngroups, -1);
        parallel_for(nthreads, nchunk, [&](int64_t ch, int t) {
            Scratch& sc = scr[t];
            const int64_t r0 = ng * ch / nchunk, r1 = ng * (ch + 1) / nchunk;
            auto& yc = ycnt[ch];
            auto& yg = ygrp[ch];
            auto& yv = yval[ch];
            yc.reserve(r1 - r0);
            for (int64_t r = r0; r < r1; ++r) {
                const int64_t i = r / (n2 * n3), j = (r / n3) % n2, k = r % n3;
                int64_t col[7];
                double coef[7];
                int nc = 0;
                const int64_t nbr[6] = {((i + 1) % n1) * n2 * n3 + j * n3 + k, ((i + n1 - 1) % n1) * n2 * n3 + j * n3 + k,
                                        i * n2 * n3 + ((j + 1) % n2) * n3 + k, i * n2 * n3 + ((j + n2 - 1) % n2) * n3 + k,
                                        i * n2 * n3 + j * n3 + (k + 1) % n3, i * n2 * n3 + j * n3 + (k + n3 - 1) % n3};
                int64_t sorted[6];
                std::copy(nbr, nbr + 6, sorted);
                std::sort(sorted, sorted + 6);
                for (int q = 0; q < 6; ++q) {
                    if (nc && col[nc - 1] == sorted[q]) {
                        coef[nc - 1] += t_off;
                    } else {
                        col[nc] = sorted[q];
                        coef[nc++] = t_off;
                    }
                }
                // diagonal: off-diagonal sum (if the stencil wraps onto r) + t_diag
                int self = -1;
                for (int q = 0; q < nc; ++q)
                    if (col[q] == r) self = q;
                if (self >= 0) {
                    coef[self] += t_diag;
                } else {
                    int q = nc++;
                    while (q > 0 && col[q - 1] > r) {
                        col[q] = col[q - 1];
                        coef[q] = coef[q - 1];
                        --q;
                    }
                    col[q] = r;
                    coef[q] = t_diag;
                }
                sc.touched.clear();
                for (int q = 0; q < nc; ++q) {
                    const int64_t c = col[q];
                    if (coef[q] == 0.0) continue;
                    for (int64_t p = b->pptr[c]; p < b->pptr[c + 1]; ++p) {
                        const int32_t g = b->pgrp[p];
                        int32_t l = sc.loc[g];
                        if (l < 0) {
                            l = (int32_t)sc.touched.size();
                            sc.loc[g] = l;
                            sc.touched.push_back(g);
                            if ((size_t)(l + 1) * L > sc.acc.size()) sc.acc.resize((size_t)(l + 1) * L * 2);
                            std::fill(sc.acc.begin() + (size_t)l * L, sc.acc.begin() + (size_t)(l + 1) * L, 0.0);
                        }
                        const double* x = &b->sval[(size_t)b->pslot[p] * L];
                        double* a = &sc.acc[(size_t)l * L];
                        const double cf = coef[q];
                        for (int h = 0; h < L; ++h) a[h] += cf * x[h];
                    }
                }
                sc.order.assign(sc.touched.begin(), sc.touched.end());
                std::sort(sc.order.begin(), sc.order.end());
                yc.push_back((int64_t)sc.order.size());
                for (int32_t g : sc.order) {
                    yg.push_back(g);
                    const double* a = &sc.acc[(size_t)sc.loc[g] * L];
                    yv.insert(yv.end(), a, a + L);
                }
                for (int32_t g : sc.touched) sc.loc[g] = -1;
            }
        });
        std::vector<int64_t> yptr(ng + 1, 0);
        {
            int64_t r = 0;
            for (int64_t ch = 0; ch < nchunk; ++ch)
                for (int64_t c : ycnt[ch]) {
                    yptr[r + 1] = yptr[r] + c;
                    ++r;
                }
        }
        std::vector<int32_t> Yg(yptr[ng]);
        std::vector<double> Yv((size_t)yptr[ng] * L);
        {
            std::vector<int64_t> chstart(nchunk + 1, 0);
            for (int64_t ch = 0; ch < nchunk; ++ch) chstart[ch + 1] = chstart[ch] + (int64_t)ygrp[ch].size();
            parallel_for(nthreads, nchunk, [&](int64_t ch, int) {
                std::copy(ygrp[ch].begin(), ygrp[ch].end(), Yg.begin() + chstart[ch]);
                std::copy(yval[ch].begin(), yval[ch].end(), Yv.begin() + chstart[ch] * L);
                std::vector<int32_t>().swap(ygrp[ch]);
                std::vector<double>().swap(yval[ch]);
            });
        }

        // ---- S and T rows of each group A: sums over r in supp(A), ascending
        b->S.resize(ngroups);
        b->T.resize(ngroups);
        struct Acc {
            std::vector<int32_t> loc, touched;
            std::vector<double> a;   // [local group][8 f][8 h]
        };
        std::vector<Acc> accS(nthreads), accT(nthreads);
        for (int t = 0; t < nthreads; ++t) {
            accS[t].loc.assign(ngroups, -1);
            accT[t].loc.assign(ngroups, -1);
        }
        auto slot_of = [](Acc& A, int32_t g) -> double* {
            int32_t l = A.loc[g];
            if (l < 0) {
                l = (int32_t)A.touched.size();
                A.loc[g] = l;
                A.touched.push_back(g);
                const size_t need = (size_t)(l + 1) * L * L;
                if (need > A.a.size()) A.a.resize(need * 2);
                std::fill(A.a.begin() + (size_t)l * L * L, A.a.begin() + need, 0.0);
            }
            return &A.a[(size_t)l * L * L];
        };
        auto emit = [&](Acc& A, int64_t ga, Rows& rows) {
            const int nfa = (int)(gptr[ga + 1] - gptr[ga]);
            std::vector<int32_t> order(A.touched);
            std::sort(order.begin(), order.end());
            rows.cnt.assign(nfa, 0);
            for (int f = 0; f < nfa; ++f)
                for (int32_t g : order) {
                    const int nfb = (int)(gptr[g + 1] - gptr[g]);
                    const double* a = &A.a[((size_t)A.loc[g] * L + f) * L];
                    for (int h = 0; h < nfb; ++h)
                        if (a[h] != 0.0) {
                            rows.col.push_back(gptr[g] + h);
                            rows.val.push_back(a[h] * dV);
                            ++rows.cnt[f];
                        }
                }
            for (int32_t g : A.touched) A.loc[g] = -1;
            A.touched.clear();
        };
        parallel_for(nthreads, ngroups, [&](int64_t ga, int t) {
            const int nfa = (int)(gptr[ga + 1] - gptr[ga]);
            for (int64_t s = b->sptr[ga]; s < b->sptr[ga + 1]; ++s) {
                const int64_t r = b->sidx[s];
                const double* xa = &b->sval[(size_t)s * L];
                for (int64_t p = b->pptr[r]; p < b->pptr[r + 1]; ++p) {
                    double* a = slot_of(accS[t], b->pgrp[p]);
                    const double* xb = &b->sval[(size_t)b->pslot[p] * L];
                    for (int f = 0; f < nfa; ++f) {
                        const double xf = xa[f];
                        for (int h = 0; h < L; ++h) a[f * L + h] += xf * xb[h];
                    }
                }
                for (int64_t p = yptr[r]; p < yptr[r + 1]; ++p) {
                    double* a = slot_of(accT[t], Yg[p]);
                    const double* yb = &Yv[(size_t)p * L];
                    for (int f = 0; f < nfa; ++f) {
                        const double xf = xa[f];
                        for (int h = 0; h < L; ++h) a[f * L + h] += xf * yb[h];
                    }
                }
            }
            emit(accS[t], ga, b->S[ga]);
            emit(accT[t], ga, b->T[ga]);
        });
        int64_t ns = 0, nt = 0;
        for (int64_t g = 0; g < ngroups; ++g) {
            ns += (int64_t)b->S[g].col.size();
            nt += (int64_t)b->T[g].col.size();
        }
        nnz[0] = 0;
        for (int64_t g = 0; g < ngroups; ++g) nnz[0] += (gptr[g + 1] - gptr[g]) * (b->sptr[g + 1] - b->sptr[g]);
        nnz[1] = ns;
        nnz[2] = nt;
    } catch (const std::bad_alloc&) {
        delete b;
        lres_set_error("lres_basis_build: host allocation failed");
        return LRES_ENOMEM;
    }
    *out = b;
    return LRES_OK;
}

extern "C" int lres_basis_build(lres_basis** out, int64_t ngroups, const int64_t* gptr, const int64_t* cnt,
                                const int64_t* idx, const double* val, const int64_t shape[3], double dV,
                                double t_diag, double t_off, int nthreads, int64_t* nnz) {
    if (!out || !gptr || !cnt || !shape || !nnz || ngroups <= 0) {
        lres_set_error("lres_basis_build: null argument or no groups");
        return LRES_EINVAL;
    }
    *out = nullptr;
    for (int i = 0; i < 3; ++i)
        if (shape[i] < 1) {
            lres_set_error("lres_basis_build: grid shape must be positive");
            return LRES_EINVAL;
        }
    if (gptr[0] != 0) {
        lres_set_error("lres_basis_build: gptr must start at 0");
        return LRES_EINVAL;
    }
    int64_t nent = 0;
    for (int64_t g = 0; g < ngroups; ++g) {
        const int64_t nf = gptr[g + 1] - gptr[g];
        if (nf < 1 || nf > kMaxLanes || cnt[g] < 0) {
            lres_set_error("lres_basis_build: group %lld has %lld functions (1..8) and %lld points", (long long)g,
                           (long long)nf, (long long)cnt[g]);
            return LRES_EINVAL;
        }
        nent += cnt[g];
    }
    if (nent && (!idx || !val)) {
        lres_set_error("lres_basis_build: null idx / val");
        return LRES_EINVAL;
    }
    const int64_t n1 = shape[0], n2 = shape[1], n3 = shape[2], ng = n1 * n2 * n3;
    for (int64_t e = 0; e < nent; ++e)
        if (idx[e] < 0 || idx[e] >= ng) {
            lres_set_error("lres_basis_build: grid index %lld out of range", (long long)idx[e]);
            return LRES_EINVAL;
        }
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());

    int nfmax = 1;
    for (int64_t g = 0; g < ngroups; ++g) nfmax = std::max<int>(nfmax, (int)(gptr[g + 1] - gptr[g]));
    switch (nfmax) {
        case 1: return build<1>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
        case 2: return build<2>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
        case 3: return build<3>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
        case 4: return build<4>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
        case 5: return build<5>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
        case 6: return build<6>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
        case 7: return build<7>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
        default: return build<8>(out, ngroups, gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads, nnz);
    }
}

extern "C" int lres_basis_fetch(const lres_basis* b, int64_t* Xp, int64_t* Xi, double* Xv, int64_t* Xrp, int64_t* Xri,
                                double* Xrv, int64_t* Sp, int64_t* Si, double* Sv, int64_t* Tp, int64_t* Ti,
                                double* Tv) {
    if (!b) {
        lres_set_error("lres_basis_fetch: null basis");
        return LRES_EINVAL;
    }
    const int64_t ngroups = b->ngroups, ng = b->ng;
    const int nth = b->nthreads;
    const std::vector<int64_t>& gp = b->gptr;
    try {
        if (Xp && Xi && Xv) {   // CSC, columns = functions: group g's columns are contiguous
            std::vector<int64_t> base(ngroups + 1, 0);
            for (int64_t g = 0; g < ngroups; ++g)
                base[g + 1] = base[g] + (gp[g + 1] - gp[g]) * (b->sptr[g + 1] - b->sptr[g]);
            Xp[0] = 0;
            parallel_for(nth, ngroups, [&](int64_t g, int) {
                const int64_t len = b->sptr[g + 1] - b->sptr[g];
                for (int64_t f = 0; f < gp[g + 1] - gp[g]; ++f) {
                    const int64_t at = base[g] + f * len;
                    for (int64_t s = 0; s < len; ++s) {
                        Xi[at + s] = b->sidx[b->sptr[g] + s];
                        Xv[at + s] = b->sval[(size_t)(b->sptr[g] + s) * b->lanes + f];
                    }
                    Xp[gp[g] + f + 1] = at + len;
                }
            });
        }
        if (Xrp && Xri && Xrv) {   // CSR, rows = grid points
            Xrp[0] = 0;
            for (int64_t r = 0; r < ng; ++r) {
                int64_t n = 0;
                for (int64_t p = b->pptr[r]; p < b->pptr[r + 1]; ++p) n += gp[b->pgrp[p] + 1] - gp[b->pgrp[p]];
                Xrp[r + 1] = Xrp[r] + n;
            }
            const int64_t nchunk = std::min<int64_t>(ng, (int64_t)nth * 16);
            parallel_for(nth, nchunk, [&](int64_t ch, int) {
                for (int64_t r = ng * ch / nchunk; r < ng * (ch + 1) / nchunk; ++r) {
                    int64_t at = Xrp[r];
                    for (int64_t p = b->pptr[r]; p < b->pptr[r + 1]; ++p) {
                        const int32_t g = b->pgrp[p];
                        for (int64_t f = 0; f < gp[g + 1] - gp[g]; ++f) {
                            Xri[at] = gp[g] + f;
                            Xrv[at] = b->sval[(size_t)b->pslot[p] * b->lanes + f];
                            ++at;
                        }
                    }
                }
            });
        }
        for (int pass = 0; pass < 2; ++pass) {
            int64_t* Ap = pass ? Tp : Sp;
            int64_t* Ai = pass ? Ti : Si;
            double* Av = pass ? Tv : Sv;
            if (!Ap || !Ai || !Av) continue;
            const std::vector<Rows>& R = pass ? b->T : b->S;
            Ap[0] = 0;
            for (int64_t g = 0; g < ngroups; ++g) {
                int64_t row = gp[g];
                for (int64_t c : R[g].cnt) {
                    Ap[row + 1] = Ap[row] + c;
                    ++row;
                }
            }
            parallel_for(nth, ngroups, [&](int64_t g, int) {
                const Rows& rw = R[g];
                const int64_t at = Ap[gp[g]];
                std::memcpy(Ai + at, rw.col.data(), rw.col.size() * sizeof(int64_t));
                std::memcpy(Av + at, rw.val.data(), rw.val.size() * sizeof(double));
            });
        }
    } catch (const std::bad_alloc&) {
        lres_set_error("lres_basis_fetch: host allocation failed");
        return LRES_ENOMEM;
    }
    return LRES_OK;
}

extern "C" int lres_basis_free(lres_basis* b) {
    delete b;
    return LRES_OK;
}

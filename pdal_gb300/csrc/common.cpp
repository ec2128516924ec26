/*
 * common.cpp -- host CSR helpers and the row-block planner.
 */
#include "common.h"
#include "rowblock_config.h"

#include <algorithm>
#include <functional>
#include <thread>

namespace pdal {

/* Host threads for setup work over `work` items (1 below ~1M items). */
int host_threads(long long work) {
    if (work < (1ll << 20)) return 1;
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    return std::max(1, std::min(hw, 32));
}

void parallel_for(int nt, const std::function<void(int)> &f) {
    if (nt <= 1) {
        f(0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(nt - 1);
    for (int t = 1; t < nt; ++t) th.emplace_back(f, t);
    f(0);
    for (auto &x : th) x.join();
}

/*
 * Counting-sort transpose.  The rows of A are cut into nt chunks of about
 * equal nonzero count; chunk t counts its entries per column, the counts are
 * turned into each chunk's first slot in every column (columns in order,
 * chunks in order within a column), and each chunk then scatters its rows in
 * order.  Every column of the result therefore lists its entries in
 * increasing row order -- the output of the one-thread scatter, bit for bit,
 * for any thread count.
 */
HostCsr csr_transpose(int nr, int nc, const int *rp, const int *ci, const double *v) {
    HostCsr T;
    T.nr = nc;
    T.nc = nr;
    const int nnz = rp[nr];
    T.rp.assign((size_t)nc + 1, 0);
    T.ci.resize(nnz);
    T.v.resize(nnz);
    int nt = host_threads(nnz);
    /* per-chunk column counts: nt x nc ints, kept under 512 MB */
    while (nt > 1 && (size_t)nt * (size_t)nc * sizeof(int) > ((size_t)512 << 20)) --nt;
    if (nt <= 1) {
        for (int k = 0; k < nnz; ++k) T.rp[ci[k] + 1]++;
        for (int j = 0; j < nc; ++j) T.rp[j + 1] += T.rp[j];
        std::vector<int> next(T.rp.begin(), T.rp.end() - 1);
        for (int i = 0; i < nr; ++i)
            for (int k = rp[i]; k < rp[i + 1]; ++k) {
                const int p = next[ci[k]]++;
                T.ci[p] = i;
                T.v[p] = v[k];
            }
        return T;
    }
    std::vector<int> rb(nt + 1, nr);
    rb[0] = 0;
    for (int t = 1; t < nt; ++t)
        rb[t] = (int)(std::lower_bound(rp, rp + nr + 1, (int)((long long)nnz * t / nt)) - rp);
    for (int t = 1; t <= nt; ++t) rb[t] = std::max(rb[t], rb[t - 1]);
    std::vector<int> cnt((size_t)nt * nc);
    parallel_for(nt, [&](int t) {
        int *c = cnt.data() + (size_t)t * nc;
        std::fill(c, c + nc, 0);
        for (int k = rp[rb[t]]; k < rp[rb[t + 1]]; ++k) c[ci[k]]++;
    });
    /* column totals, then each chunk's first slot per column */
    const int ntc = nt;
    parallel_for(ntc, [&](int t) {
        const int j0 = (int)((long long)nc * t / ntc), j1 = (int)((long long)nc * (t + 1) / ntc);
        for (int j = j0; j < j1; ++j) {
            int s = 0;
            for (int q = 0; q < nt; ++q) s += cnt[(size_t)q * nc + j];
            T.rp[j + 1] = s;
        }
    });
    for (int j = 0; j < nc; ++j) T.rp[j + 1] += T.rp[j];
    parallel_for(ntc, [&](int t) {
        const int j0 = (int)((long long)nc * t / ntc), j1 = (int)((long long)nc * (t + 1) / ntc);
        for (int j = j0; j < j1; ++j) {
            int at = T.rp[j];
            for (int q = 0; q < nt; ++q) {
                int &c = cnt[(size_t)q * nc + j];
                const int n = c;
                c = at;
                at += n;
            }
        }
    });
    parallel_for(nt, [&](int t) {
        int *next = cnt.data() + (size_t)t * nc;
        for (int i = rb[t]; i < rb[t + 1]; ++i)
            for (int k = rp[i]; k < rp[i + 1]; ++k) {
                const int p = next[ci[k]]++;
                T.ci[p] = i;
                T.v[p] = v[k];
            }
    });
    return T;
}

std::vector<int> csr_transpose_rp(int nr, int nc, const int *rp, const int *ci) {
    const int nnz = rp[nr];
    std::vector<int> trp((size_t)nc + 1, 0);
    const int nt = host_threads(nnz);
    int *cnt = trp.data() + 1;
    if (nt <= 1) {
        for (int k = 0; k < nnz; ++k) cnt[ci[k]]++;
    } else {
        /* one shared count per column, relaxed atomic increments (measured
         * 25% faster than per-thread count arrays and their reduction on a
         * 20M-nonzero matrix) */
        parallel_for(nt, [&](int t) {
            const long long k0 = (long long)nnz * t / nt, k1 = (long long)nnz * (t + 1) / nt;
            for (long long k = k0; k < k1; ++k) __atomic_fetch_add(&cnt[ci[k]], 1, __ATOMIC_RELAXED);
        });
    }
    for (int j = 0; j < nc; ++j) trp[j + 1] += trp[j];
    return trp;
}

void csr_validate(int nr, int nc, const int *rp, const int *ci, int nnz, const char *what) {
    if (nr < 0 || nc < 0 || nnz < 0) throw Error(std::string(what) + ": negative dimension");
    if (nr > 0 && !rp) throw Error(std::string(what) + ": missing row pointers");
    if (nnz > 0 && !ci) throw Error(std::string(what) + ": missing column indices");
    if (rp && rp[0] != 0) throw Error(std::string(what) + ": row_ptr[0] != 0");
    for (int i = 0; i < nr; ++i)
        if (rp[i + 1] < rp[i]) throw Error(std::string(what) + ": row pointers decrease");
    if (rp && rp[nr] != nnz) throw Error(std::string(what) + ": row_ptr[m] != nnz");
    const int nt = host_threads(nnz);
    std::vector<char> bad(nt, 0);
    parallel_for(nt, [&](int t) {
        const long long k0 = (long long)nnz * t / nt, k1 = (long long)nnz * (t + 1) / nt;
        for (long long k = k0; k < k1; ++k)
            if (ci[k] < 0 || ci[k] >= nc) {
                bad[t] = 1;
                break;
            }
    });
    for (char b : bad)
        if (b) throw Error(std::string(what) + ": column index out of range");
}

HostPlan plan_rows(int nr, const int *rp, int S) {
    HostPlan P;
    P.S = S;
    int r = 0;
    while (r < nr) {
        const int len = rp[r + 1] - rp[r];
        if (len > S) {
            const int np = (len + S - 1) / S;
            const int lid = P.nlong++;
            P.linfo.insert(P.linfo.end(), {r, np, P.npieces, rp[r]});
            for (int p = 0; p < np; ++p) {
                const int k0 = rp[r] + p * S;
                const int k1 = std::min(k0 + S, rp[r + 1]);
                P.desc.insert(P.desc.end(), {r, ~lid, k0, k1});
            }
            P.npieces += np;
            ++r;
            continue;
        }
        const int r0 = r;
        int k = 0;
        while (r < nr && (r - r0) < kMaxRowsPerBlock) {
            const int l = rp[r + 1] - rp[r];
            if (l > S || k + l > S) break;
            k += l;
            ++r;
        }
        P.desc.insert(P.desc.end(), {r0, r, rp[r0], rp[r]});
    }
    P.nblocks = (int)(P.desc.size() / 4);
    return P;
}

HostPanels plan_panels(int nr, int nc, const int *rp, const int *ci, int S, int W, int target_blocks) {
    HostPanels Q;
    Q.W = W;
    Q.P = nc > 0 ? (nc + W - 1) / W : 0;
    for (int r = 0; r < nr; ++r)
        if (rp[r + 1] - rp[r] > S) {
            Q.rows.push_back(r);
            Q.long_nnz += rp[r + 1] - rp[r];
        }
    Q.H = (int)Q.rows.size();
    const int H = Q.H, P = Q.P;
    if (H == 0 || P == 0) return Q;
    /* entries of long row h in panel p, then padded segment starts: panel
     * major, rows in order within a panel */
    std::vector<int> cnt((size_t)H * P, 0);
    const int nt = host_threads(Q.long_nnz);
    parallel_for(nt, [&](int t) {
        for (int h = t; h < H; h += nt) {
            const int r = Q.rows[h];
            int *c = cnt.data() + (size_t)h * P;
            for (int k = rp[r]; k < rp[r + 1]; ++k) c[ci[k] / W]++;
        }
    });
    std::vector<long long> start((size_t)H * P, 0);
    size_t used = 0; /* (row, panel) pairs with entries: the segments */
    for (int c : cnt) used += c > 0 ? 1 : 0;
    Q.seg.reserve(4 * used);
    long long pos = 0;
    for (int p = 0; p < P; ++p)
        for (int h = 0; h < H; ++h) {
            const int c = cnt[(size_t)h * P + p];
            start[(size_t)h * P + p] = pos;
            if (c > 0) {
                Q.seg.insert(Q.seg.end(), {h, (int)pos, (int)(pos + ((c + 3) & ~3)), p});
                pos += (c + 3) & ~3;
            }
        }
    if (pos > (long long)INT32_MAX - 16) throw Error("long rows too large for the panel plan");
    Q.len = pos;
    /* every position is written once below, by the thread that owns its
     * row: the entries, then the segment's padding (-1, offset 0) */
    Q.pmap.resize((size_t)pos);
    Q.off.resize((size_t)pos);
    parallel_for(nt, [&](int t) {
        std::vector<long long> at((size_t)P);
        for (int h = t; h < H; h += nt) {
            const int r = Q.rows[h];
            for (int p = 0; p < P; ++p) at[p] = start[(size_t)h * P + p];
            for (int k = rp[r]; k < rp[r + 1]; ++k) {
                const int p = ci[k] / W;
                const long long q = at[p]++;
                Q.pmap[(size_t)q] = k;
                Q.off[(size_t)q] = (uint16_t)(ci[k] - p * W);
            }
            for (int p = 0; p < P; ++p) {
                const int c = cnt[(size_t)h * P + p];
                const long long end = start[(size_t)h * P + p] + ((c + 3) & ~3);
                for (long long q = at[p]; q < end; ++q) {
                    Q.pmap[(size_t)q] = -1;
                    Q.off[(size_t)q] = 0;
                }
            }
        }
    });
    /* blocks: target_blocks ranges of consecutive segments of about equal
     * nonzero counts (one wave of equal work); a range may cross panel
     * borders -- the block then stages each panel in turn */
    const int nseg = (int)(Q.seg.size() / 4);
    std::vector<long long> cum((size_t)nseg + 1, 0);
    for (int s = 0; s < nseg; ++s) cum[s + 1] = cum[s] + (Q.seg[4 * s + 2] - Q.seg[4 * s + 1]);
    const int nb = std::max(1, std::min(target_blocks, nseg));
    int s0 = 0;
    for (int b = 0; b < nb && s0 < nseg; ++b) {
        const long long goal = cum[nseg] * (b + 1) / nb;
        int s1 = (int)(std::lower_bound(cum.begin() + s0 + 1, cum.end(), goal) - cum.begin());
        s1 = std::max(s0 + 1, std::min(s1, nseg));
        if (b == nb - 1) s1 = nseg;
        /* the block's range cut at panel borders into pieces of one panel */
        const int first_piece = (int)(Q.piece.size() / 4);
        for (int a = s0; a < s1;) {
            const int p = Q.seg[4 * a + 3];
            int e = a + 1;
            while (e < s1 && Q.seg[4 * e + 3] == p) ++e;
            Q.piece.insert(Q.piece.end(), {p, a, e, 0});
            a = e;
        }
        Q.cta.insert(Q.cta.end(), {first_piece, (int)(Q.piece.size() / 4), 0, 0});
        s0 = s1;
    }
    return Q;
}

int auto_block_nnz(long long nnz, int nr) {
    (void)nr;
    const long long target_blocks = 2 * 152;
    const int choices[] = {256, 512, 1024, 2048};
    for (int c : {2048, 1024, 512}) {
        if (nnz / c >= target_blocks) return c;
    }
    (void)choices;
    return 256;
}

} // namespace pdal

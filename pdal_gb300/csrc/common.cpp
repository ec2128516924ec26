/*
 * common.cpp -- host CSR helpers and the row-block planner.
 */
#include "common.h"
#include "rowblock_config.h"

#include <algorithm>

namespace pdal {

HostCsr csr_transpose(int nr, int nc, const int *rp, const int *ci, const double *v) {
    HostCsr T;
    T.nr = nc;
    T.nc = nr;
    const int nnz = rp[nr];
    T.rp.assign((size_t)nc + 1, 0);
    T.ci.resize(nnz);
    T.v.resize(nnz);
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

void csr_validate(int nr, int nc, const int *rp, const int *ci, int nnz, const char *what) {
    if (nr < 0 || nc < 0 || nnz < 0) throw Error(std::string(what) + ": negative dimension");
    if (nr > 0 && !rp) throw Error(std::string(what) + ": missing row pointers");
    if (nnz > 0 && !ci) throw Error(std::string(what) + ": missing column indices");
    if (rp && rp[0] != 0) throw Error(std::string(what) + ": row_ptr[0] != 0");
    for (int i = 0; i < nr; ++i)
        if (rp[i + 1] < rp[i]) throw Error(std::string(what) + ": row pointers decrease");
    if (rp && rp[nr] != nnz) throw Error(std::string(what) + ": row_ptr[m] != nnz");
    for (int k = 0; k < nnz; ++k)
        if (ci[k] < 0 || ci[k] >= nc) throw Error(std::string(what) + ": column index out of range");
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

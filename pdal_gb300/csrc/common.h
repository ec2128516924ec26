/*
 * common.h -- host-side helpers shared by the solver translation units:
 * CUDA error handling that never exits the process, a device arena, CSR
 * utilities and row-block planning.
 */
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace pdal {

/* Every CUDA failure becomes an exception that the C entry points turn into a
 * NULL result plus a message (the reference calls exit(): internal/utils.h:32-63). */
struct Error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define PDAL_CUDA(call)                                                                                 \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            throw ::pdal::Error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " + __FILE__ + \
                                ":" + std::to_string(__LINE__));                                        \
        }                                                                                               \
    } while (0)

/* One cudaMalloc for all buffers of a solve; sub-allocations are 256-byte
 * aligned so every vector can be read with 128-bit loads.  The same
 * allocation code runs twice: once in measuring mode (take() only counts),
 * then for real after reserve(). */
class Arena {
  public:
    Arena() = default;
    Arena(const Arena &) = delete;
    Arena &operator=(const Arena &) = delete;
    ~Arena() { release(); }
    void begin_measure() {
        release();
        measuring_ = true;
        off_ = 0;
    }
    void reserve_measured() {
        const size_t bytes = off_;
        measuring_ = false;
        cap_ = bytes + 256;
        PDAL_CUDA(cudaMalloc(&base_, cap_));
        off_ = 0;
    }
    template <typename T>
    T *take(size_t count) {
        /* 256-byte aligned, with at least 64 bytes of slack after the last
         * element: kernels that copy 16-byte-aligned windows (bulk copies,
         * 128-bit loads) may read up to 15 bytes past an array's end */
        size_t bytes = ((count * sizeof(T)) + 64 + 255) & ~size_t(255);
        if (bytes == 0) bytes = 256;
        if (measuring_) {
            off_ += bytes;
            return reinterpret_cast<T *>(alignof(T) > 256 ? alignof(T) : 256);
        }
        if (off_ + bytes > cap_) throw Error("device arena exhausted");
        T *p = reinterpret_cast<T *>(static_cast<char *>(base_) + off_);
        off_ += bytes;
        return p;
    }
    void release() {
        if (base_) cudaFree(base_);
        base_ = nullptr;
        cap_ = off_ = 0;
    }
    size_t used() const { return off_; }
    size_t capacity() const { return cap_; }

  private:
    void *base_ = nullptr;
    size_t cap_ = 0, off_ = 0;
    bool measuring_ = false;
};

/* Host CSR. */
struct HostCsr {
    int nr = 0, nc = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
    int nnz() const { return (int)ci.size(); }
};

/* Host threads worth using for setup work over `work` items, and a fork-join
 * over thread ids 0..nt-1 (id 0 runs on the calling thread). */
int host_threads(long long work);
void parallel_for(int nt, const std::function<void(int)> &f);

/* Transpose with rows of A^T in increasing row order of A (host threads;
 * the result does not depend on their number). */
HostCsr csr_transpose(int nr, int nc, const int *rp, const int *ci, const double *v);

/* Checks row pointers (monotone, rp[0]=0, rp[nr]=nnz) and column range; the
 * kernels index vectors with these values, so a malformed matrix is refused
 * on the host instead of reading outside a device buffer. */
void csr_validate(int nr, int nc, const int *rp, const int *ci, int nnz, const char *what);

/* Row-block plan (see rowblock.cuh). */
struct HostPlan {
    int S = 0;
    std::vector<int> desc;  /* 4 ints per block */
    std::vector<int> linfo; /* 4 ints per long row */
    int nblocks = 0, nlong = 0, npieces = 0;
};
HostPlan plan_rows(int nr, const int *rp, int S);

/*
 * Column-panel plan of the long rows (more than S nonzeros) of a CSR matrix,
 * for the dual product A x of a matrix whose long rows hold much of its
 * nonzeros (the power-law rows of the large LP).  The columns are cut into
 * panels of W; a CUDA block takes a contiguous range of segments (one long
 * row restricted to one panel; panel-major order) of about equal nonzero
 * count and stages each panel its range touches in shared memory in turn, so
 * the long rows' random gathers become shared-memory reads.
 * The long rows' nonzeros are stored again in panel order, each segment
 * padded with zeros to a multiple of 4 entries (128-bit loads), with the
 * column as a 16-bit offset in its panel (W <= 65536).  Segment (h, p) --
 * long row h, panel p -- writes partial sum h * P + p; a row's total is the
 * sum of its P partials in panel order (zeros where the row has no entry in
 * a panel), so the result is deterministic.
 */
/* An allocator that leaves new elements uninitialised, so that a large host
 * array is first touched by the threads that fill it (in parallel) instead
 * of being zeroed on one thread. */
template <typename T>
struct UninitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind {
        using other = UninitAlloc<U>;
    };
    UninitAlloc() = default;
    template <typename U>
    UninitAlloc(const UninitAlloc<U> &) {}
    template <typename U>
    void construct(U *) noexcept {}
    template <typename U, typename... A>
    void construct(U *p, A &&...a) {
        ::new ((void *)p) U(std::forward<A>(a)...);
    }
};

struct HostPanels {
    int W = 0, P = 0, H = 0;
    std::vector<int> rows;      /* H long rows (ascending) */
    std::vector<int, UninitAlloc<int>> pmap;          /* panel-array position -> CSR position, -1 for padding */
    std::vector<uint16_t, UninitAlloc<uint16_t>> off; /* column - p * W (0 for padding) */
    std::vector<int> seg;       /* 4 ints per segment: {h, k0, k1, p} (k0, k1 multiples of 4) */
    std::vector<int> piece;     /* 4 ints per piece: {panel, first segment, end segment, 0} */
    std::vector<int> cta;       /* 4 ints per block: {first piece, end piece, 0, 0} */
    long long long_nnz = 0;
    long long len = 0;          /* panel-array length, padding included */
};
HostPanels plan_panels(int nr, int nc, const int *rp, const int *ci, int S, int W, int target_blocks);

/* Nonzero budget per block for a matrix of `nnz` nonzeros when none is
 * requested: enough blocks to cover the 152 SMs twice, at most 2048. */
int auto_block_nnz(long long nnz, int nr);

/* Row pointers of the transpose of an nr x nc CSR matrix (its column counts,
 * summed), on the host threads; the transpose itself can then be built on
 * the device. */
std::vector<int> csr_transpose_rp(int nr, int nc, const int *rp, const int *ci);

} // namespace pdal

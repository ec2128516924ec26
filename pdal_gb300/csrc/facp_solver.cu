/*
 * facp_solver.cu -- host side of the FA_CP (convex QP) solver: equilibration,
 * device layout, the evaluation / restart / sigma control of
 * QP/FA_CP/src/solver.cu:74-165, and the C entry points solve_qp_problem and
 * fa_cp_gb300_solve.
 *
 * The iterations themselves run in the persistent kernel of facp_kernels.cuh:
 * the host launches one segment per evaluation point (every print-frequency
 * iteration and every major iteration, the only places where the reference
 * makes a data-dependent decision), reads a few scalars back, and decides
 * termination and restarts exactly where the reference does.
 */
#include "../../include/fa_cp.h"
#include "../../include/fa_cp_gb300.h"
#include "common.h"
#include "facp_kernels.cuh"

#include <algorithm>
#include <memory>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace pdal {
namespace {

using namespace facp;

thread_local fa_cp_gb300_stats_t g_stats;
thread_local std::string g_error;

double now_sec() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

/* The C library's rand() as a fresh process sees it (seed 1): the additive
 * feedback generator r[i] = r[i-3] + r[i-31] (mod 2^32) over a table seeded
 * with the Park-Miller sequence 16807^i mod (2^31 - 1), the first 310 outputs
 * discarded, each output shifted right by one bit.  Kept per solve so the
 * process-wide rand() state is never touched. */
class CRandom {
  public:
    explicit CRandom(unsigned seed = 1) {
        std::vector<int32_t> r(34);
        r[0] = (int32_t)seed;
        for (int i = 1; i < 31; ++i) {
            const long long v = (16807LL * r[i - 1]) % 2147483647LL;
            r[i] = (int32_t)(v < 0 ? v + 2147483647LL : v);
        }
        for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
        for (int i = 0; i < 34; ++i) s_[i] = (uint32_t)r[i];
        k_ = 34;
        for (int i = 34; i < 344; ++i) next_raw();
    }
    int next() { return (int)(next_raw() >> 1); }
    static constexpr int kMax = 2147483647;

  private:
    uint32_t next_raw() {
        const uint32_t v = s_[(k_ - 31) % 34] + s_[(k_ - 3) % 34];
        s_[k_ % 34] = v;
        ++k_;
        return v;
    }
    uint32_t s_[34];
    long long k_;
};

struct HostQP {
    int n = 0, m = 0, nr = 0;
    HostCsr A, Q, R;
    std::vector<double> c, vlb, vub, clb, cub;
    std::vector<double> dcum, rcum;
    double cbr = 1.0, ovr = 1.0, c0 = 0.0;
    double obj_norm = 0.0, bnd_norm = 0.0;
};

HostCsr from_component(const CsrComponent *cc, int rows, int cols, int nnz, const char *what) {
    HostCsr M;
    M.nr = rows;
    M.nc = cols;
    M.rp.assign((size_t)rows + 1, 0);
    if (cc && cc->row_ptr && nnz > 0) {
        csr_validate(rows, cols, cc->row_ptr, cc->col_ind, nnz, what);
        M.rp.assign(cc->row_ptr, cc->row_ptr + rows + 1);
        M.ci.assign(cc->col_ind, cc->col_ind + nnz);
        M.v.assign(cc->val, cc->val + nnz);
    } else if (cc && cc->row_ptr && rows > 0) {
        csr_validate(rows, cols, cc->row_ptr, cc->col_ind, 0, what);
    }
    return M;
}

/* ---------------------------------------------------------------- equilibration
 * QP/FA_CP/src/preconditioner.c:92-331: Ruiz passes (columns see A and Q),
 * one Pock-Chambolle pass, then bound/objective scaling that also rescales Q
 * by ovr/cbr and R by sqrt(ovr/cbr).
 *
 * Run on the device.  Column statistics come from the rows of the transposes
 * A' and Q', which hold each column's entries in increasing row order -- the
 * order the reference's row-major scatter visits them -- and each row's
 * statistic is formed by one thread in storage order, so every sum has the
 * reference's order.  Every matrix and transpose value is divided by the
 * same product of scale factors as in the reference, with IEEE division and
 * multiplication, and the bound/objective norms are summed on the host in
 * the reference's loop order: the scaled problem is bit-identical to the
 * reference's (|a|^deg uses pow() except for deg 1 and 2, where it is exact
 * on both sides). */
__device__ __forceinline__ double pow_deg(double a, double deg) {
    if (deg == 1.0) return a;
    if (deg == 2.0) return __dmul_rn(a, a);
    return pow(a, deg);
}

/* abs max (mode 0) or sum of |a|^deg in storage order (mode 1) of each row */
__global__ void k_row_stat(int rows, const int *__restrict__ rp, const double *__restrict__ v, int mode, double deg,
                           double *out, int accumulate) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        double acc = accumulate ? out[r] : 0.0;
        for (int k = rp[r]; k < rp[r + 1]; ++k) {
            const double a = fabs(v[k]);
            if (mode == 0) {
                if (a > acc) acc = a;
            } else {
                acc = __dadd_rn(acc, pow_deg(a, deg));
            }
        }
        out[r] = acc;
    }
}

/* s = s < 1e-12 ? 1 : sqrt(s); cum *= s */
__global__ void k_finish_scale(int len, double *s, double *cum) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        const double v = s[i];
        const double f = (v < 1e-12) ? 1.0 : sqrt(v);
        s[i] = f;
        cum[i] = __dmul_rn(cum[i], f);
    }
}

/* a_rk /= rs[r] * cs[col] (a missing factor is left out) */
__global__ void k_scale_csr(int rows, const int *__restrict__ rp, const int *__restrict__ ci, double *v,
                            const double *__restrict__ rs, const double *__restrict__ cs) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        for (int k = rp[r]; k < rp[r + 1]; ++k) {
            const double den = rs ? (cs ? __dmul_rn(rs[r], cs[ci[k]]) : rs[r]) : cs[ci[k]];
            v[k] = __ddiv_rn(v[k], den);
        }
    }
}

__global__ void k_scale_vectors(int n, int m, double *c, double *vlb, double *vub, double *clb, double *cub,
                                const double *__restrict__ d, const double *__restrict__ r) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < max(n, m); i += gridDim.x * blockDim.x) {
        if (i < n) {
            c[i] = __ddiv_rn(c[i], d[i]);
            vub[i] = __dmul_rn(vub[i], d[i]);
            vlb[i] = __dmul_rn(vlb[i], d[i]);
        }
        if (i < m) {
            clb[i] = __ddiv_rn(clb[i], r[i]);
            cub[i] = __ddiv_rn(cub[i], r[i]);
        }
    }
}

__global__ void k_bound_objective(int n, int m, double cbr, double ovr, double *c, double *vlb, double *vub,
                                  double *clb, double *cub) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < max(n, m); i += gridDim.x * blockDim.x) {
        if (i < m) {
            clb[i] = __dmul_rn(clb[i], cbr);
            cub[i] = __dmul_rn(cub[i], cbr);
        }
        if (i < n) {
            vlb[i] = __dmul_rn(vlb[i], cbr);
            vub[i] = __dmul_rn(vub[i], cbr);
            c[i] = __dmul_rn(c[i], ovr);
        }
    }
}

__global__ void k_mul(long long len, double *v, double f) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
        v[i] = __dmul_rn(v[i], f);
}

__global__ void k_fill(int len, double *v, double val) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) v[i] = val;
}

/* finite part of a bound vector (infinite entries become 0) */
__global__ void k_finite(int len, const double *__restrict__ src, double *dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
        dst[i] = isfinite(src[i]) ? src[i] : 0.0;
}

__global__ void k_to_float(long long len, const double *__restrict__ src, float *dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

/* diagonal of a diagonal Q plus 1e-12 (solver_state.cu:252-270) */
__global__ void k_diag(int rows, int n, const int *__restrict__ rp, const int *__restrict__ ci,
                       const double *__restrict__ v, double *diag) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
        for (int k = rp[r]; k < rp[r + 1]; ++k)
            if (ci[k] < n) diag[ci[k]] = __dadd_rn(v[k], 1e-12);
}

int detect_q_type(const HostCsr &Q, const HostCsr &R) { /* QP/FA_CP/src/utils.cu:1576-1616 */
    if (Q.nnz() == 0 && R.nnz() == 0) return Q_NONE;
    if (R.nnz() > 0) return Q.nnz() > 0 ? Q_LOWRANK_SPARSE : Q_LOWRANK;
    for (int i = 0; i < Q.nr; ++i)
        for (int k = Q.rp[i]; k < Q.rp[i + 1]; ++k)
            if (Q.ci[k] != i) return Q_SPARSE;
    return Q_DIAG;
}

double sane_positive(double v, double fb) { return (std::isfinite(v) && v > 0.0) ? v : fb; }
double score_component(double v) { return std::isfinite(v) ? std::fmax(v, 1e-300) : INFINITY; }
double clamp_d(double v, double lo, double hi) { return std::fmin(std::fmax(v, lo), hi); }

int print_frequency_host(int iter) {
    int step = 10;
    long long threshold = 1000;
    while (iter >= threshold) {
        step *= 10;
        threshold *= 10;
    }
    return step;
}

struct DevMat {
    HostCsr h;
    HostPlan plan;
    DMat d{};
};

class FacpSolver {
  public:
    FacpSolver(const qp_problem_t *prob, const fa_cp_parameters_t &prm, const fa_cp_gb300_options_t &opt)
        : prob_(prob), p_(prm), o_(opt) {}
    ~FacpSolver() {
        if (stream_) cudaStreamDestroy(stream_);
        if (ev0_) cudaEventDestroy(ev0_);
        if (ev1_) cudaEventDestroy(ev1_);
    }
    fa_cp_result_t *run();
    /* prepare, upload and equilibrate only; the scale vectors and factors */
    void scaling(double *dcum, double *rcum, double *cbr_ovr) {
        prepare();
        upload();
        if (dcum) std::copy(H_.dcum.begin(), H_.dcum.end(), dcum);
        if (rcum) std::copy(H_.rcum.begin(), H_.rcum.end(), rcum);
        if (cbr_ovr) {
            cbr_ovr[0] = H_.cbr;
            cbr_ovr[1] = H_.ovr;
        }
    }

  private:
    void prepare();
    void upload();
    void launch(Args a);
    void launch(Args a, const Prob &P);
    void read_ctl();
    Args base_args(int mode) const;
    void power_iterations();
    void equilibrate_device();
    void evaluate(bool infeas);
    bool check_termination(double elapsed);
    bool should_restart();
    void choose_restart_candidate(double elapsed);
    void perform_restart();
    void update_sigma(double pd, double dd, double normal);
    void set_sigma_active(double s, double zt);
    double clipped(double cur, double ratio) const;
    void print_eval() const;
    void polish(double t_loop);
    int polish_phase(bool primal, double pw0, double &abs_r, double &rel_r, double &obj);
    void trajectory_header() const;
    void trajectory_row(double elapsed, bool restart) const;

    const qp_problem_t *prob_;
    fa_cp_parameters_t p_;
    fa_cp_gb300_options_t o_;
    HostQP H_;
    HostCsr Qt_; /* Q' for the column statistics of the equilibration */
    int *qt_rp_ = nullptr, *qt_ci_ = nullptr;
    double *qt_v_ = nullptr;
    double transpose_sec_ = 0.0;
    int qtype_ = Q_NONE;
    DevMat M_[NMAT];
    Arena arena_;
    Prob P_{};
    Ctl ctl_{};
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    int grid_ = 0;
    std::vector<double> diag_;
    double qnorm_ = 0.0, nonconvexity_ = 0.0;
    double sv_max_ = 0.0;
    double setup_sec_ = 0.0, rescale_sec_ = 0.0, upload_sec_ = 0.0, power_sec_ = 0.0;
    int power_iters_a_ = 0, power_iters_q_ = 0;
    long long launches_ = 0;
    float dev_ms_ = 0.f;

    /* solver state (solver_state.cu:494-877 of the reference) */
    int total_ = 0, inner_ = 0;
    double step_ = 0.0, pw_ = 1.0, best_pw_ = 1.0, pw_esum_ = 0.0, pw_last_ = 0.0, best_gap_ = INFINITY;
    double fp_ = INFINITY, fp0_ = INFINITY, fp_last_ = INFINITY;
    bool al_available_ = false, use_al_ = false, has_inner_ = false;
    double al_sigma_ = 0.0, best_al_sigma_ = 0.0, best_sigma_score_ = INFINITY, last_sigma_score_ = INFINITY;
    double last_rp_ = INFINITY, last_rd_ = INFINITY, last_rg_ = INFINITY;
    int sigma_updates_ = 0, sigma_dir_ = 1;
    int inner_limit_ = 1000;
    termination_reason_t reason_ = TERMINATION_REASON_UNSPECIFIED;
    int restart_target_ = 0;
    int restarts_ = 0, evals_ = 0;
    bool fp32_ = false; /* FP32 segments (first phase of precision 1) */
    /* feasibility polishing (problems without Q) */
    int polish_iters_ = 0, polish_status_[2] = {-1, -1};
    double polish_sec_ = 0.0;
    double fp32_best_ = INFINITY;
    int fp32_stall_ = 0, fp32_iters_ = 0;
};

void FacpSolver::prepare() {
    const qp_problem_t *q = prob_;
    if (!q) throw Error("solve_qp_problem: invalid arguments");
    if (o_.precision != 0 && o_.precision != 1) throw Error("precision must be 0 (FP64) or 1 (FP32 + FP64 refinement)");
    if (o_.precision == 1 && !(o_.fp32_switch_tol >= 0.0)) throw Error("fp32_switch_tol must be >= 0");
    if (p_.termination_evaluation_frequency < 1) throw Error("termination_evaluation_frequency must be >= 1");
    HostQP &P = H_;
    P.n = q->num_variables;
    P.m = q->num_constraints;
    P.nr = q->num_rank_lowrank_obj;
    if (P.n < 1 || P.m < 0 || P.nr < 0) throw Error("solve_qp_problem: the problem needs n >= 1 variables");
    if (!q->objective_vector || !q->variable_lower_bound || !q->variable_upper_bound ||
        (P.m > 0 && (!q->constraint_lower_bound || !q->constraint_upper_bound)))
        throw Error("solve_qp_problem: missing problem vectors");
    P.A = from_component(q->constraint_matrix, P.m, P.n, q->constraint_matrix_num_nonzeros, "A");
    P.Q = from_component(q->objective_sparse_matrix, P.n, P.n, q->objective_sparse_matrix_num_nonzeros, "Q");
    P.R = from_component(q->objective_lowrank_matrix, P.nr, P.n, q->objective_lowrank_matrix_num_nonzeros, "R");
    P.c.assign(q->objective_vector, q->objective_vector + P.n);
    P.vlb.assign(q->variable_lower_bound, q->variable_lower_bound + P.n);
    P.vub.assign(q->variable_upper_bound, q->variable_upper_bound + P.n);
    if (P.m > 0) {
        P.clb.assign(q->constraint_lower_bound, q->constraint_lower_bound + P.m);
        P.cub.assign(q->constraint_upper_bound, q->constraint_upper_bound + P.m);
    }
    P.c0 = q->objective_constant;
    /* norms of the unscaled problem (solver_state.cu:700-740) */
    const bool linf = p_.optimality_norm == NORM_TYPE_L_INF;
    {
        double s = 0.0, mx = 0.0;
        for (int i = 0; i < P.n; ++i) {
            const double v = q->objective_vector[i];
            if (linf)
                mx = std::max(mx, std::fabs(v));
            else
                s += v * v;
        }
        P.obj_norm = linf ? mx : std::sqrt(s);
        s = 0.0;
        mx = 0.0;
        for (int i = 0; i < P.m; ++i) {
            const double lo = q->constraint_lower_bound[i], up = q->constraint_upper_bound[i];
            if (linf) {
                if (std::isfinite(lo) && lo != up) mx = std::max(mx, std::fabs(lo));
                if (std::isfinite(up)) mx = std::max(mx, std::fabs(up));
            } else {
                if (std::isfinite(lo) && lo != up) s += lo * lo;
                if (std::isfinite(up)) s += up * up;
            }
        }
        P.bnd_norm = linf ? mx : std::sqrt(s);
    }
    const double t0 = now_sec();
    HostCsr At = csr_transpose(P.m, P.n, P.A.rp.data(), P.A.ci.data(), P.A.v.data());
    Qt_ = csr_transpose(P.n, P.n, P.Q.rp.data(), P.Q.ci.data(), P.Q.v.data());
    transpose_sec_ = now_sec() - t0;
    qtype_ = detect_q_type(P.Q, P.R);
    /* unscaled values: equilibration runs on the device after the upload */
    M_[MAT_A].h = std::move(P.A);
    M_[MAT_AT].h = std::move(At);
    M_[MAT_Q].h = std::move(P.Q);
    M_[MAT_R].h = P.R;
    M_[MAT_RT].h = csr_transpose(P.nr, P.n, P.R.rp.data(), P.R.ci.data(), P.R.v.data());
    M_[MAT_A].h.nr = P.m;
    M_[MAT_A].h.nc = P.n;
    int lbase = 0;
    for (int k = 0; k < NMAT; ++k) {
        DevMat &dm = M_[k];
        dm.plan = plan_rows(dm.h.nr, dm.h.rp.data(), kS);
        dm.d.rows = dm.h.nr;
        dm.d.lbase = lbase;
        lbase += dm.plan.nlong;
    }
    P_.nlong_total = lbase;
    P_.bar_extra = std::max(0, o_.barrier_extra_arrivals);
    P_.spin_limit = o_.barrier_spin_limit > 0 ? o_.barrier_spin_limit : kSpinLimit;
}

void FacpSolver::upload() {
    const double t_up = now_sec();
    const HostQP &H = H_;
    const size_t n = H.n, m = H.m, nr = H.nr;
    int dev = 0;
    if (o_.device >= 0) PDAL_CUDA(cudaSetDevice(o_.device));
    PDAL_CUDA(cudaGetDevice(&dev));
    PDAL_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    PDAL_CUDA(cudaEventCreate(&ev0_));
    PDAL_CUDA(cudaEventCreate(&ev1_));
    int coop = 0, sms = 0;
    PDAL_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    PDAL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (!coop) throw Error("the device does not support cooperative launches");
    int per_sm = 0;
    PDAL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_facp, kThreads, 0));
    if (per_sm < 1) throw Error("the persistent kernel does not fit on one SM");
    if (o_.blocks_per_sm > 0) per_sm = std::min(per_sm, o_.blocks_per_sm);
    long long work = 0;
    for (int k = 0; k < NMAT; ++k) work = std::max<long long>(work, M_[k].plan.nblocks);
    work = std::max<long long>(work, ((long long)std::max(n, m) + kThreads - 1) / kThreads);
    grid_ = (int)std::max<long long>(1, std::min<long long>((long long)per_sm * sms, work));

    const size_t vec = std::max<size_t>(std::max(n, m), 1);
    const int nl = std::max(P_.nlong_total, 1);
    auto alloc_all = [&]() {
        for (int k = 0; k < NMAT; ++k) {
            DevMat &dm = M_[k];
            const size_t nnz = dm.h.ci.size();
            dm.d.rp = arena_.take<int>((size_t)dm.h.nr + 1);
            dm.d.ci = arena_.take<int>(nnz + 8);
            dm.d.v = arena_.take<double>(nnz + 8);
            dm.d.plan.nblocks = dm.plan.nblocks;
            dm.d.plan.nlong = dm.plan.nlong;
            dm.d.plan.desc = arena_.take<int4>(std::max(dm.plan.nblocks, 1));
            dm.d.plan.linfo = arena_.take<int4>(std::max(dm.plan.nlong, 1));
            dm.d.plan.lpart = arena_.take<double>(kLongStride * (size_t)std::max(dm.plan.npieces, 1));
            dm.d.plan.lcount = arena_.take<unsigned>(std::max(dm.plan.nlong, 1));
        }
        double **consts[] = {(double **)&P_.c,       (double **)&P_.vlb,     (double **)&P_.vub,
                             (double **)&P_.vlb_fin, (double **)&P_.vub_fin, (double **)&P_.diag,
                             (double **)&P_.dcum};
        for (double **p : consts) *p = arena_.take<double>(n);
        double **cons[] = {(double **)&P_.clb, (double **)&P_.cub, (double **)&P_.clb_fin, (double **)&P_.cub_fin,
                           (double **)&P_.rcum};
        for (double **p : cons) *p = arena_.take<double>(std::max<size_t>(m, 1));
        for (double **p : {&P_.x0, &P_.x, &P_.xh, &P_.xbar, &P_.dprod, &P_.dslack, &P_.dx, &P_.qx, &P_.grad, &P_.dir,
                           &P_.out_x, &P_.out_rc})
            *p = arena_.take<double>(n);
        for (double **p : {&P_.y0, &P_.y, &P_.yh, &P_.ybar, &P_.dy, &P_.aldual, &P_.out_y})
            *p = arena_.take<double>(std::max<size_t>(m, 1));
        qt_rp_ = arena_.take<int>(Qt_.rp.size());
        qt_ci_ = arena_.take<int>(std::max<size_t>(Qt_.ci.size(), 1));
        qt_v_ = arena_.take<double>(std::max<size_t>(Qt_.v.size(), 1));
        P_.rx = arena_.take<double>(std::max<size_t>(nr, 1));
        P_.pv = arena_.take<double>(vec);
        P_.pv2 = arena_.take<double>(vec);
        P_.pv3 = arena_.take<double>(vec);
        P_.part = arena_.take<double>((size_t)3 * grid_ * kSlot);
        P_.lpart = arena_.take<double>((size_t)3 * nl * kSlot);
        P_.bar = arena_.take<GridBar>(1);
        P_.ctl = arena_.take<Ctl>(1);
        P_.f = SegV<float>{};
        if (o_.precision == 1) { /* FP32 mirror of the segment path */
            SegV<float> &f = P_.f;
            const size_t mm = std::max<size_t>(m, 1), rr = std::max<size_t>(nr, 1);
            for (const float **q : {&f.c, &f.vlb, &f.vub, &f.diag}) *q = arena_.take<float>(n);
            for (const float **q : {&f.clb, &f.cub}) *q = arena_.take<float>(mm);
            for (float **q : {&f.x, &f.xh, &f.xbar, &f.dprod, &f.dslack, &f.dx, &f.qx, &f.grad, &f.dir})
                *q = arena_.take<float>(n);
            for (float **q : {&f.y, &f.yh, &f.ybar, &f.dy, &f.aldual}) *q = arena_.take<float>(mm);
            f.rx = arena_.take<float>(rr);
            f.x0 = arena_.take<float2>(n);
            f.y0 = arena_.take<float2>(mm);
            for (int k = 0; k < NMAT; ++k) f.mv[k] = arena_.take<float>(M_[k].h.ci.size() + 8);
        }
    };
    arena_.begin_measure();
    alloc_all();
    arena_.reserve_measured();
    alloc_all();

    auto h2d = [&](const void *dst, const void *src, size_t bytes) {
        if (bytes) PDAL_CUDA(cudaMemcpyAsync((void *)dst, src, bytes, cudaMemcpyHostToDevice, stream_));
    };
    for (int k = 0; k < NMAT; ++k) {
        DevMat &dm = M_[k];
        h2d(dm.d.rp, dm.h.rp.data(), dm.h.rp.size() * sizeof(int));
        h2d(dm.d.ci, dm.h.ci.data(), dm.h.ci.size() * sizeof(int));
        h2d(dm.d.v, dm.h.v.data(), dm.h.v.size() * sizeof(double));
        h2d(dm.d.plan.desc, dm.plan.desc.data(), dm.plan.desc.size() * sizeof(int));
        h2d(dm.d.plan.linfo, dm.plan.linfo.data(), dm.plan.linfo.size() * sizeof(int));
        PDAL_CUDA(cudaMemsetAsync(dm.d.plan.lcount, 0, sizeof(unsigned) * std::max(dm.plan.nlong, 1), stream_));
        P_.M[k] = dm.d;
    }
    P_.n = H.n;
    P_.m = H.m;
    P_.nr = H.nr;
    P_.qtype = qtype_;
    h2d(qt_rp_, Qt_.rp.data(), Qt_.rp.size() * sizeof(int));
    h2d(qt_ci_, Qt_.ci.data(), Qt_.ci.size() * sizeof(int));
    h2d(qt_v_, Qt_.v.data(), Qt_.v.size() * sizeof(double));
    h2d(P_.c, H.c.data(), n * 8);
    h2d(P_.vlb, H.vlb.data(), n * 8);
    h2d(P_.vub, H.vub.data(), n * 8);
    if (m > 0) {
        h2d(P_.clb, H.clb.data(), m * 8);
        h2d(P_.cub, H.cub.data(), m * 8);
    }
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    upload_sec_ = now_sec() - t_up;
    equilibrate_device();
    /* iterates: zero, or the scaled warm start (solver_state.cu:621-656) */
    for (double *p : {P_.x0, P_.x, P_.xh, P_.xbar, P_.dprod, P_.dslack, P_.dx, P_.qx, P_.grad, P_.dir})
        PDAL_CUDA(cudaMemsetAsync(p, 0, n * 8, stream_));
    for (double *p : {P_.y0, P_.y, P_.yh, P_.ybar, P_.dy, P_.aldual})
        PDAL_CUDA(cudaMemsetAsync(p, 0, std::max<size_t>(m, 1) * 8, stream_));
    PDAL_CUDA(cudaMemsetAsync(P_.rx, 0, std::max<size_t>(nr, 1) * 8, stream_));
    std::vector<double> ws;
    if (prob_->primal_start) {
        ws.resize(n);
        for (size_t i = 0; i < n; ++i) ws[i] = prob_->primal_start[i] * H.dcum[i] * H.cbr;
        for (double *p : {P_.x0, P_.x, P_.xh}) h2d(p, ws.data(), n * 8);
        PDAL_CUDA(cudaStreamSynchronize(stream_));
    }
    if (prob_->dual_start && m > 0) {
        ws.resize(m);
        for (size_t i = 0; i < m; ++i) ws[i] = prob_->dual_start[i] * H.rcum[i] * H.ovr;
        for (double *p : {P_.y0, P_.y, P_.yh}) h2d(p, ws.data(), m * 8);
        PDAL_CUDA(cudaStreamSynchronize(stream_));
    }
    PDAL_CUDA(cudaMemsetAsync(P_.lpart, 0, (size_t)3 * nl * kSlot * 8, stream_));
    PDAL_CUDA(cudaMemsetAsync(P_.ctl, 0, sizeof(Ctl), stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
}

Args FacpSolver::base_args(int mode) const {
    Args a{};
    a.mode = mode;
    a.F = p_.termination_evaluation_frequency;
    a.linf = p_.optimality_norm == NORM_TYPE_L_INF;
    a.cbr = H_.cbr;
    a.ovr = H_.ovr;
    a.c0 = H_.c0;
    a.obj_norm = H_.obj_norm;
    a.bnd_norm = H_.bnd_norm;
    a.step = step_;
    a.pw = pw_;
    a.tau_eval = step_ > 0 ? step_ / pw_ : 1.0;
    a.refl = p_.reflection_coefficient;
    a.max_iter = p_.sv_max_iter;
    a.tol = p_.sv_tol;
    return a;
}

void FacpSolver::launch(Args a) { launch(a, P_); }

void FacpSolver::launch(Args a, const Prob &P) {
    PDAL_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), stream_));
    if (P.nlong_total > 0)
        PDAL_CUDA(cudaMemsetAsync(P.lpart, 0, (size_t)3 * P.nlong_total * kSlot * 8, stream_));
    Prob Pc = P;
    void *args[] = {(void *)&Pc, (void *)&a};
    PDAL_CUDA(cudaLaunchCooperativeKernel((const void *)k_facp, dim3(grid_), dim3(kThreads), args, 0, stream_));
    ++launches_;
}

void FacpSolver::read_ctl() {
    PDAL_CUDA(cudaMemcpyAsync(&ctl_, P_.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    if (ctl_.status != 0) throw Error("the persistent kernel gave up waiting at a grid barrier");
}

void FacpSolver::power_iterations() {
    const HostQP &H = H_;
    if (qtype_ == Q_SPARSE) { /* solver_state.cu:462-476 */
        CRandom rnd(1);
        std::vector<double> v(H.n);
        for (double &x : v) x = (double)rnd.next() / CRandom::kMax;
        PDAL_CUDA(cudaMemcpyAsync(P_.pv, v.data(), H.n * 8, cudaMemcpyHostToDevice, stream_));
        launch(base_args(MODE_POWER_QMAX));
        read_ctl();
        qnorm_ = ctl_.power_value;
        power_iters_q_ += ctl_.power_iters;
        for (double &x : v) x = (double)rnd.next() / CRandom::kMax;
        PDAL_CUDA(cudaMemcpyAsync(P_.pv, v.data(), H.n * 8, cudaMemcpyHostToDevice, stream_));
        Args a = base_args(MODE_POWER_QMIN);
        a.lam_max = qnorm_;
        launch(a);
        read_ctl();
        nonconvexity_ = ctl_.power_value;
        power_iters_q_ += ctl_.power_iters;
    }
    if (M_[MAT_A].h.nnz() == 0) { /* fa_cp_core_op.cu:1022-1040 */
        step_ = 1.0;
    } else {
        std::mt19937 gen(1);
        std::normal_distribution<double> dist(0.0, 1.0);
        std::vector<double> v(H.m);
        for (double &x : v) x = dist(gen);
        PDAL_CUDA(cudaMemcpyAsync(P_.pv, v.data(), H.m * 8, cudaMemcpyHostToDevice, stream_));
        launch(base_args(MODE_POWER_A));
        read_ctl();
        sv_max_ = ctl_.power_value;
        power_iters_a_ = ctl_.power_iters;
        step_ = 0.998 / sv_max_;
    }
    pw_ = p_.bound_objective_rescaling ? 1.0 : (H.obj_norm + 1.0) / (H.bnd_norm + 1.0);
    best_pw_ = pw_;
}

void FacpSolver::equilibrate_device() {
    const double t0 = now_sec();
    HostQP &H = H_;
    const int n = H.n, m = H.m, nr = H.nr;
    auto grid = [&](long long len) {
        return (int)std::max<long long>(1, std::min<long long>(152 * 16, (len + 255) / 256));
    };
    const int gv = grid(std::max(n, m));
    double *cr = P_.pv, *vr = P_.pv2;
    k_fill<<<grid(n), 256, 0, stream_>>>(n, (double *)P_.dcum, 1.0);
    if (m) k_fill<<<grid(m), 256, 0, stream_>>>(m, (double *)P_.rcum, 1.0);
    const DMat &A = P_.M[MAT_A], &At = P_.M[MAT_AT], &Q = P_.M[MAT_Q], &R = P_.M[MAT_R], &Rt = P_.M[MAT_RT];
    const bool has_q = !Qt_.ci.empty(), has_r = !M_[MAT_R].h.ci.empty();
    auto pass = [&](int mode, double deg_rows, double deg_cols) {
        if (m) k_row_stat<<<grid(m), 256, 0, stream_>>>(m, A.rp, A.v, mode, deg_rows, cr, 0);
        k_row_stat<<<grid(n), 256, 0, stream_>>>(n, At.rp, At.v, mode, deg_cols, vr, 0);
        if (has_q) k_row_stat<<<grid(n), 256, 0, stream_>>>(n, qt_rp_, qt_v_, mode, deg_cols, vr, 1);
        k_finish_scale<<<grid(n), 256, 0, stream_>>>(n, vr, (double *)P_.dcum);
        if (m) k_finish_scale<<<grid(m), 256, 0, stream_>>>(m, cr, (double *)P_.rcum);
        k_scale_vectors<<<gv, 256, 0, stream_>>>(n, m, (double *)P_.c, (double *)P_.vlb, (double *)P_.vub,
                                                 (double *)P_.clb, (double *)P_.cub, vr, cr);
        if (m) k_scale_csr<<<grid(m), 256, 0, stream_>>>(m, A.rp, A.ci, (double *)A.v, cr, vr);
        k_scale_csr<<<grid(n), 256, 0, stream_>>>(n, At.rp, At.ci, (double *)At.v, vr, cr);
        if (has_q) {
            k_scale_csr<<<grid(n), 256, 0, stream_>>>(n, Q.rp, Q.ci, (double *)Q.v, vr, vr);
            k_scale_csr<<<grid(n), 256, 0, stream_>>>(n, qt_rp_, qt_ci_, qt_v_, vr, vr);
        }
        if (has_r) {
            k_scale_csr<<<grid(nr), 256, 0, stream_>>>(nr, R.rp, R.ci, (double *)R.v, nullptr, vr);
            k_scale_csr<<<grid(n), 256, 0, stream_>>>(n, Rt.rp, Rt.ci, (double *)Rt.v, vr, nullptr);
        }
        PDAL_CUDA(cudaGetLastError());
        launches_ += 8;
    };
    for (int it = 0; it < p_.l_inf_ruiz_iterations; ++it) pass(0, 0.0, 0.0);
    if (p_.has_pock_chambolle_alpha) pass(1, p_.pock_chambolle_alpha, 2.0 - p_.pock_chambolle_alpha);
    /* bound/objective scaling: the two norms are summed on the host in the
     * reference's loop order (preconditioner.c:245-289) */
    H.dcum.resize(n);
    H.rcum.resize(m);
    std::vector<double> c(n), lo(m), up(m);
    PDAL_CUDA(cudaMemcpyAsync(c.data(), P_.c, (size_t)n * 8, cudaMemcpyDeviceToHost, stream_));
    PDAL_CUDA(cudaMemcpyAsync(H.dcum.data(), P_.dcum, (size_t)n * 8, cudaMemcpyDeviceToHost, stream_));
    if (m) {
        PDAL_CUDA(cudaMemcpyAsync(lo.data(), P_.clb, (size_t)m * 8, cudaMemcpyDeviceToHost, stream_));
        PDAL_CUDA(cudaMemcpyAsync(up.data(), P_.cub, (size_t)m * 8, cudaMemcpyDeviceToHost, stream_));
        PDAL_CUDA(cudaMemcpyAsync(H.rcum.data(), P_.rcum, (size_t)m * 8, cudaMemcpyDeviceToHost, stream_));
    }
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    if (p_.bound_objective_rescaling) {
        double bsq = 0.0, csq = 0.0;
        for (int i = 0; i < m; ++i) {
            if (std::isfinite(lo[i]) && lo[i] != up[i]) bsq += lo[i] * lo[i];
            if (std::isfinite(up[i])) bsq += up[i] * up[i];
        }
        for (int i = 0; i < n; ++i) csq += c[i] * c[i];
        H.cbr = 1.0 / (std::sqrt(bsq) + 1.0);
        H.ovr = 1.0 / (std::sqrt(csq) + 1.0);
        k_bound_objective<<<gv, 256, 0, stream_>>>(n, m, H.cbr, H.ovr, (double *)P_.c, (double *)P_.vlb,
                                                   (double *)P_.vub, (double *)P_.clb, (double *)P_.cub);
        if (has_q) k_mul<<<grid((long long)M_[MAT_Q].h.ci.size()), 256, 0, stream_>>>(
            (long long)M_[MAT_Q].h.ci.size(), (double *)Q.v, H.ovr / H.cbr);
        if (has_r) {
            const double f = std::sqrt(H.ovr / H.cbr);
            k_mul<<<grid((long long)M_[MAT_R].h.ci.size()), 256, 0, stream_>>>((long long)M_[MAT_R].h.ci.size(),
                                                                               (double *)R.v, f);
            k_mul<<<grid((long long)M_[MAT_RT].h.ci.size()), 256, 0, stream_>>>((long long)M_[MAT_RT].h.ci.size(),
                                                                                (double *)Rt.v, f);
        }
        launches_ += 4;
    } else {
        H.cbr = H.ovr = 1.0;
    }
    /* finite parts of the bounds, and the diagonal of a diagonal Q */
    k_finite<<<grid(n), 256, 0, stream_>>>(n, P_.vlb, (double *)P_.vlb_fin);
    k_finite<<<grid(n), 256, 0, stream_>>>(n, P_.vub, (double *)P_.vub_fin);
    if (m) {
        k_finite<<<grid(m), 256, 0, stream_>>>(m, P_.clb, (double *)P_.clb_fin);
        k_finite<<<grid(m), 256, 0, stream_>>>(m, P_.cub, (double *)P_.cub_fin);
    }
    launches_ += 4;
    if (qtype_ == Q_DIAG) { /* solver_state.cu:252-270, 478-492 */
        k_fill<<<grid(n), 256, 0, stream_>>>(n, (double *)P_.diag, 0.0);
        k_diag<<<grid(n), 256, 0, stream_>>>(n, n, Q.rp, Q.ci, Q.v, (double *)P_.diag);
        diag_.resize(n);
        PDAL_CUDA(cudaMemcpyAsync(diag_.data(), P_.diag, (size_t)n * 8, cudaMemcpyDeviceToHost, stream_));
        launches_ += 2;
    }
    PDAL_CUDA(cudaGetLastError());
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    if (qtype_ == Q_DIAG) {
        double mx = 0.0, mn = 0.0;
        for (double d : diag_) {
            mx = std::fmax(mx, std::fabs(d));
            mn = std::fmin(mn, d);
        }
        qnorm_ = mx;
        nonconvexity_ = mn;
    }
    if (o_.precision == 1) { /* FP32 copies of the scaled data; zero product buffers */
        SegV<float> &f = P_.f;
        auto cv = [&](const double *src, const float *dst, long long len) {
            if (len > 0) k_to_float<<<grid(len), 256, 0, stream_>>>(len, src, (float *)dst);
        };
        cv(P_.c, f.c, n);
        cv(P_.vlb, f.vlb, n);
        cv(P_.vub, f.vub, n);
        cv(P_.clb, f.clb, m);
        cv(P_.cub, f.cub, m);
        if (qtype_ == Q_DIAG) cv(P_.diag, f.diag, n);
        for (int k = 0; k < NMAT; ++k) cv(P_.M[k].v, f.mv[k], (long long)M_[k].h.ci.size());
        PDAL_CUDA(cudaMemsetAsync(f.qx, 0, (size_t)n * sizeof(float), stream_));
        PDAL_CUDA(cudaMemsetAsync(f.rx, 0, (size_t)std::max(nr, 1) * sizeof(float), stream_));
        PDAL_CUDA(cudaGetLastError());
        launches_ += 6 + NMAT;
        PDAL_CUDA(cudaStreamSynchronize(stream_));
    }
    rescale_sec_ = transpose_sec_ + (now_sec() - t0);
}

void FacpSolver::evaluate(bool infeas) {
    Args a = base_args(MODE_EVAL);
    a.infeas = infeas ? 1 : 0;
    launch(a);
    read_ctl();
    ++evals_;
}

bool FacpSolver::check_termination(double elapsed) { /* QP/FA_CP/src/utils.cu:413-462 */
    const auto &T = p_.termination_criteria;
    if (ctl_.rel_d < T.eps_feasible_relative && ctl_.rel_p < T.eps_feasible_relative &&
        ctl_.rel_gap < T.eps_optimal_relative)
        reason_ = TERMINATION_REASON_OPTIMAL;
    else if (ctl_.dray_obj > 0.0 && ctl_.max_dray / ctl_.dray_obj <= T.eps_infeasible)
        reason_ = TERMINATION_REASON_PRIMAL_INFEASIBLE;
    else if (ctl_.pray_lin < 0.0 && ctl_.max_pray / (-ctl_.pray_lin) <= T.eps_infeasible)
        reason_ = TERMINATION_REASON_DUAL_INFEASIBLE;
    else if (total_ >= T.iteration_limit)
        reason_ = TERMINATION_REASON_ITERATION_LIMIT;
    else if (elapsed >= T.time_sec_limit)
        reason_ = TERMINATION_REASON_TIME_LIMIT;
    return reason_ != TERMINATION_REASON_UNSPECIFIED;
}

bool FacpSolver::should_restart() { /* QP/FA_CP/src/utils.cu:464-492 */
    const auto &R = p_.restart_params;
    const int F = p_.termination_evaluation_frequency;
    bool rs = false;
    if (total_ == F) {
        rs = true;
    } else if (total_ > F) {
        if (fp_ <= R.sufficient_reduction_for_restart * fp0_) rs = true;
        if (fp_ <= R.necessary_reduction_for_restart * fp0_ && fp_ > fp_last_) rs = true;
        if (inner_ >= R.artificial_restart_threshold * total_) rs = true;
    }
    fp_last_ = fp_;
    return rs;
}

void FacpSolver::choose_restart_candidate(double elapsed) { /* fa_cp_core_op.cu:1130-1169 */
    restart_target_ = 0;
    const double cur = std::isfinite(fp_) ? fp_ : INFINITY;
    if (o_.restart_select == 0 || total_ == 0 || !std::isfinite(cur)) return;
    if (total_ < o_.restart_select_min_iters || elapsed < o_.restart_select_min_time) return;
    launch(base_args(MODE_DELTA_SCORE));
    read_ctl();
    const double halpern = ctl_.score;
    if (!(cur > 0.0)) return;
    if (o_.restart_select == 2 || (std::isfinite(halpern) && halpern < o_.restart_select_margin * cur)) {
        restart_target_ = 1;
        fp_ = halpern;
    }
}

void FacpSolver::set_sigma_active(double s, double zt) {
    if (!std::isfinite(s) || s <= zt) {
        al_sigma_ = 0.0;
        use_al_ = false;
    } else {
        al_sigma_ = s;
        use_al_ = al_available_;
    }
}

double FacpSolver::clipped(double cur, double ratio) const {
    const double gain = sane_positive(p_.sigma_update_gain, 0.5);
    double lo = sane_positive(p_.sigma_clip_low, 0.6), hi = sane_positive(p_.sigma_clip_high, 1.7);
    if (lo > hi) std::swap(lo, hi);
    ratio = sane_positive(ratio, 1.0);
    return cur * clamp_d(std::pow(ratio, gain), lo, hi);
}

/* The sigma rules of update_al_sigma_at_restart (fa_cp_core_op.cu:722-906). */
void FacpSolver::update_sigma(double pd, double dd, double normal) {
    const int rule = p_.sigma_update_rule;
    const bool bal = rule == FA_CP_SIGMA_UPDATE_BALANCED_GUARDED;
    const bool guarded = rule == FA_CP_SIGMA_UPDATE_GUARDED || bal;
    if (!al_available_ || rule == FA_CP_SIGMA_UPDATE_FIXED) return;
    if (!guarded && !use_al_) return;
    const double ref = bal ? sane_positive(step_ * pw_, 1.0) : 1.0;
    double smin = sane_positive(p_.sigma_min, 1e-8) * ref;
    double smax = sane_positive(p_.sigma_max, 10.0) * ref;
    const double zt = sane_positive(p_.sigma_zero_threshold, sane_positive(p_.sigma_min, 1e-8)) * ref;
    if (smin > smax) std::swap(smin, smax);
    if (zt > smin) smin = zt;
    const double cur = use_al_ ? clamp_d(sane_positive(al_sigma_, smin), smin, smax) : 0.0;
    set_sigma_active(cur, zt);
    const double rp = sane_positive(ctl_.rel_p, 1e-300), rd = sane_positive(ctl_.rel_d, 1e-300),
                 rg = sane_positive(ctl_.rel_gap, 1e-300);
    const double score = std::fmax(score_component(ctl_.rel_p),
                                   std::fmax(score_component(ctl_.rel_d), score_component(ctl_.rel_gap)));
    if (!std::isfinite(score)) return;
    if (!std::isfinite(best_sigma_score_) || score < best_sigma_score_) {
        best_sigma_score_ = score;
        best_al_sigma_ = cur;
    }
    auto record = [&]() {
        last_sigma_score_ = score;
        last_rp_ = rp;
        last_rd_ = rd;
        last_rg_ = rg;
        sigma_updates_++;
    };
    if (p_.sigma_rollback_tol > 0.0 && (!guarded || cur > zt) && std::isfinite(best_sigma_score_) &&
        best_sigma_score_ > 0.0 && score > p_.sigma_rollback_tol * best_sigma_score_ &&
        std::isfinite(best_al_sigma_) && (guarded ? best_al_sigma_ >= 0.0 : best_al_sigma_ > 0.0)) {
        set_sigma_active((guarded && best_al_sigma_ <= zt) ? 0.0 : clamp_d(best_al_sigma_, smin, smax), zt);
        record();
        return;
    }
    double prop = cur;
    switch (rule) {
    case FA_CP_SIGMA_UPDATE_RESIDUAL_BALANCE:
        prop = clipped(cur, rp / rd);
        break;
    case FA_CP_SIGMA_UPDATE_KKT_BALANCE:
        prop = clipped(cur, rp / std::fmax(rd, rg));
        break;
    case FA_CP_SIGMA_UPDATE_DISPLACEMENT:
        if (std::isfinite(pd) && std::isfinite(dd) && pd > 1e-16 && dd > 1e-16)
            prop = clipped(cur, clamp_d(dd / pd, smin, smax) / cur);
        break;
    case FA_CP_SIGMA_UPDATE_PROGRESS: {
        const double last_other = std::fmax(last_rd_, last_rg_), other = std::fmax(rd, rg);
        if (std::isfinite(last_rp_) && std::isfinite(last_other) && last_rp_ > 0.0 && last_other > 0.0)
            prop = clipped(cur, (last_other / other) / (last_rp_ / rp));
        else
            prop = clipped(cur, rp / std::fmax(rd, rg));
        break;
    }
    case FA_CP_SIGMA_UPDATE_GREEDY_SCORE:
        if (sigma_updates_ == 0)
            sigma_dir_ = (rp >= std::fmax(rd, rg)) ? 1 : -1;
        else if (std::isfinite(last_sigma_score_) && score > last_sigma_score_)
            sigma_dir_ = -sigma_dir_;
        prop = clipped(cur, sigma_dir_ > 0 ? p_.sigma_clip_high : p_.sigma_clip_low);
        break;
    case FA_CP_SIGMA_UPDATE_GUARDED:
    case FA_CP_SIGMA_UPDATE_BALANCED_GUARDED: {
        const double nmt = sane_positive(p_.sigma_normal_motion_threshold, 1e-10);
        const bool normal_ok = !std::isfinite(normal) || normal > nmt;
        const bool zero_ok = !std::isfinite(normal) || normal > std::fmax(nmt, 2e-1);
        const bool bottleneck =
            rp >= sane_positive(p_.sigma_activation_threshold, 2.0) * sane_positive(std::fmax(rd, rg), 1e-300);
        const bool zero_stalled = cur <= zt && std::isfinite(last_sigma_score_) && score > 0.9 * last_sigma_score_;
        const bool primal_signal = rp >= 0.5 * sane_positive(rd, 1e-300);
        const double act = sane_positive(p_.sigma_activation_value, 0.1) * ref;
        const bool scale_ok = !bal || act >= 1e-6;
        const bool activate = cur <= zt ? (zero_ok && zero_stalled && primal_signal && scale_ok) : (normal_ok && bottleneck);
        if (cur <= zt)
            prop = activate ? act : 0.0;
        else if (!normal_ok || !activate)
            prop = clipped(cur, p_.sigma_clip_low);
        else
            prop = clipped(cur, rp / std::fmax(rd, rg));
        break;
    }
    default:
        break;
    }
    prop = prop > zt ? clamp_d(prop, smin, smax) : 0.0;
    set_sigma_active(prop, zt);
    record();
}

void FacpSolver::perform_restart() { /* fa_cp_core_op.cu:908-1020 */
    Args a = base_args(MODE_RESTART);
    const bool to_halpern = o_.restart_select != 0 && restart_target_ == 1;
    if (to_halpern) {
        /* measure against the current (Halpern) iterate: swap the roles of
         * xh/x and yh/y for the measurement launch */
        std::swap(P_.xh, P_.x);
        std::swap(P_.yh, P_.y);
    }
    launch(a);
    read_ctl();
    if (to_halpern) {
        std::swap(P_.xh, P_.x);
        std::swap(P_.yh, P_.y);
    }
    const double pd = ctl_.pd, dd = ctl_.dd;
    double normal = INFINITY;
    if (pd > 1e-16 && std::isfinite(pd)) normal = ctl_.normal_dist / pd;
    const double ratio = ctl_.rel_d / ctl_.rel_p;
    const auto &R = p_.restart_params;
    if (pd > 1e-16 && dd > 1e-16 && pd < 1e12 && dd < 1e12 && ratio > 1e-8 && ratio < 1e8) {
        const double err = std::log(dd) - std::log(pd) - std::log(pw_);
        pw_esum_ *= R.i_smooth;
        pw_esum_ += err;
        const double de = err - pw_last_;
        pw_ *= std::exp(R.k_p * err + R.k_i * pw_esum_ + R.k_d * de);
        pw_last_ = err;
    } else {
        pw_ = best_pw_;
        pw_esum_ = 0.0;
        pw_last_ = 0.0;
    }
    const double g = std::fabs(std::log10(ctl_.rel_d / ctl_.rel_p));
    if (g < best_gap_) {
        best_gap_ = g;
        best_pw_ = pw_;
    }
    update_sigma(pd, dd, normal);
    const size_t nb = (size_t)H_.n * 8, mb = (size_t)H_.m * 8;
    double *src_x = to_halpern ? P_.x : P_.xh, *src_y = to_halpern ? P_.y : P_.yh;
    double *dst_x = to_halpern ? P_.xh : P_.x, *dst_y = to_halpern ? P_.yh : P_.y;
    PDAL_CUDA(cudaMemcpyAsync(P_.x0, src_x, nb, cudaMemcpyDeviceToDevice, stream_));
    PDAL_CUDA(cudaMemcpyAsync(dst_x, src_x, nb, cudaMemcpyDeviceToDevice, stream_));
    if (mb) {
        PDAL_CUDA(cudaMemcpyAsync(P_.y0, src_y, mb, cudaMemcpyDeviceToDevice, stream_));
        PDAL_CUDA(cudaMemcpyAsync(dst_y, src_y, mb, cudaMemcpyDeviceToDevice, stream_));
    }
    inner_ = 0;
    fp_last_ = INFINITY;
    ++restarts_;
}

/* QP/FA_CP/src/solver.cu:35-70: one CSV row per evaluation point (the file
 * is created with its header before the loop and reopened for each row). */
/* ---------------- feasibility polishing (fa_cp_core_op.cu:1241-1735) ----------------
 * Built for problems without Q (for a QP the reference's dual phase measures
 * a dual slack that nothing refreshes, and it runs to its limits).  Each phase
 * runs the solve's iteration (the same persistent kernel and evaluation
 * cadence) on a copy of the state whose problem is the feasibility problem:
 * primal phase, c = 0 and objective constant 0, from the solve's primal
 * iterates with the dual ones at zero; dual phase, every finite bound zero,
 * from the solve's dual iterates and dual slack with the primal ones at zero.
 * Both use the primal weight of the start of the solve, restart by the
 * solve's rule on a one-sided fixed-point error by moving the anchor to the
 * current point, and stop when their relative residual is at most
 * eps_feas_polish_relative (utils.cu:1360-1384).  As in the reference's loop,
 * a phase runs one more iteration after its stopping test and counts
 * total - 1 iterations. */
namespace {
struct DevBuf {
    void *p = nullptr;
    explicit DevBuf(size_t bytes) { PDAL_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16))); }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
};

__global__ void k_zero_finite_copy(const double *__restrict__ src, double *dst, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[i] = isfinite(src[i]) ? 0.0 : src[i];
}
} // namespace

int FacpSolver::polish_phase(bool primal, double pw0, double &abs_r, double &rel_r, double &obj) {
    const size_t n = H_.n, m = H_.m, mm = std::max<size_t>(m, 1), nr = std::max<size_t>(H_.nr, 1);
    std::vector<std::unique_ptr<DevBuf>> keep;
    auto buf = [&](size_t len) {
        keep.emplace_back(new DevBuf(len * sizeof(double)));
        return (double *)keep.back()->p;
    };
    auto zeros = [&](size_t len) {
        double *p = buf(len);
        PDAL_CUDA(cudaMemsetAsync(p, 0, std::max<size_t>(len, 1) * sizeof(double), stream_));
        return p;
    };
    auto copy = [&](const double *src, size_t len) {
        double *p = buf(len);
        if (len) PDAL_CUDA(cudaMemcpyAsync(p, src, len * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
        return p;
    };
    auto zero_finite = [&](const double *src, size_t len) {
        double *p = buf(len);
        if (len) k_zero_finite_copy<<<(int)std::min<size_t>((len + kThreads - 1) / kThreads, 1024), kThreads, 0,
                                      stream_>>>(src, p, (int)len);
        return p;
    };
    Prob Q = P_;
    Q.ref_c = P_.c;
    Q.ref_clb_fin = P_.clb_fin;
    Q.ref_cub_fin = P_.cub_fin;
    Q.ref_xh = P_.xh;
    if (primal) { /* fa_cp_core_op.cu:1410-1478 */
        Q.c = zeros(n);
        Q.x0 = copy(P_.x0, n);
        Q.x = copy(P_.x, n);
        Q.xh = copy(P_.xh, n);
        Q.xbar = copy(P_.xbar, n);
        Q.y0 = zeros(mm);
        Q.y = zeros(mm);
        Q.yh = zeros(mm);
        Q.ybar = zeros(mm);
        Q.dprod = zeros(n);
        Q.dslack = zeros(n);
    } else { /* fa_cp_core_op.cu:1525-1607 */
        Q.clb = zero_finite(P_.clb, m);
        Q.cub = zero_finite(P_.cub, m);
        Q.vlb = zero_finite(P_.vlb, n);
        Q.vub = zero_finite(P_.vub, n);
        Q.clb_fin = zeros(mm);
        Q.cub_fin = zeros(mm);
        Q.vlb_fin = zeros(n);
        Q.vub_fin = zeros(n);
        Q.y0 = copy(P_.y0, m);
        Q.y = copy(P_.y, m);
        Q.yh = copy(P_.yh, m);
        Q.ybar = copy(P_.ybar, m);
        Q.dprod = copy(P_.dprod, n);
        Q.dslack = copy(P_.dslack, n);
        Q.x0 = zeros(n);
        Q.x = zeros(n);
        Q.xh = zeros(n);
        Q.xbar = zeros(n);
    }
    Q.aldual = zeros(mm);
    Q.dx = zeros(n);
    Q.dy = zeros(mm);
    Q.qx = zeros(n);
    Q.grad = zeros(n);
    Q.dir = zeros(n);
    Q.rx = zeros(nr);
    keep.emplace_back(new DevBuf(sizeof(Ctl)));
    Q.ctl = (Ctl *)keep.back()->p;
    Ctl cl = ctl_; /* the state copy keeps the inner solver's tolerance */
    cl.fp = INFINITY;
    cl.fp_first = INFINITY;
    cl.status = 0;
    PDAL_CUDA(cudaMemcpyAsync(Q.ctl, &cl, sizeof(Ctl), cudaMemcpyHostToDevice, stream_));
    auto read = [&]() {
        PDAL_CUDA(cudaMemcpyAsync(&cl, Q.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream_));
        PDAL_CUDA(cudaStreamSynchronize(stream_));
        if (cl.status != 0) throw Error("the persistent kernel gave up waiting at a grid barrier");
    };
    const auto &T = p_.termination_criteria;
    const auto &R = p_.restart_params;
    const int F = p_.termination_evaluation_frequency;
    int total = 0, inner = 0, status = TERMINATION_REASON_UNSPECIFIED;
    double fp = INFINITY, fp0 = INFINITY, fp_last = INFINITY;
    bool major = false, do_restart = false;
    const double t0 = now_sec();
    while (status == TERMINATION_REASON_UNSPECIFIED) { /* fa_cp_core_op.cu:1313-1355, 1362-1404 */
        if (major || total == 0 || total % print_frequency_host(total) == 0) {
            Args a = base_args(primal ? MODE_POLISH_EVAL_P : MODE_POLISH_EVAL_D);
            a.pw = pw0;
            a.c0 = primal ? 0.0 : H_.c0;
            launch(a, Q);
            read();
            abs_r = primal ? cl.abs_p : cl.abs_d;
            rel_r = primal ? cl.rel_p : cl.rel_d;
            obj = primal ? cl.pobj : cl.dobj;
            if (rel_r <= T.eps_feas_polish_relative)
                status = TERMINATION_REASON_FEAS_POLISH_SUCCESS;
            else if (total >= T.iteration_limit)
                status = TERMINATION_REASON_ITERATION_LIMIT;
            else if (now_sec() - t0 >= T.time_sec_limit)
                status = TERMINATION_REASON_TIME_LIMIT;
        }
        if (major || total == 0) { /* utils.cu:464-492, then fa_cp_core_op.cu:1649-1668 */
            bool rs = false;
            if (total == F) {
                rs = true;
            } else if (total > F) {
                if (fp <= R.sufficient_reduction_for_restart * fp0) rs = true;
                if (fp <= R.necessary_reduction_for_restart * fp0 && fp > fp_last) rs = true;
                if (inner >= R.artificial_restart_threshold * total) rs = true;
            }
            fp_last = fp;
            do_restart = rs;
            if (rs) {
                const size_t len = primal ? n : m;
                double *anchor = primal ? Q.x0 : Q.y0, *cur = primal ? Q.x : Q.y;
                const double *sol = primal ? Q.xh : Q.yh;
                if (len) {
                    PDAL_CUDA(cudaMemcpyAsync(anchor, sol, len * 8, cudaMemcpyDeviceToDevice, stream_));
                    PDAL_CUDA(cudaMemcpyAsync(cur, sol, len * 8, cudaMemcpyDeviceToDevice, stream_));
                }
                inner = 0;
                fp_last = INFINITY;
            }
        }
        /* up to the next evaluation point, or the one iteration the
         * reference's loop runs after its stopping test */
        int t_end = total + 1;
        if (status == TERMINATION_REASON_UNSPECIFIED)
            while ((t_end % F) != 0 && (t_end % print_frequency_host(t_end)) != 0) ++t_end;
        Args a = base_args(MODE_SEGMENT);
        a.pw = pw0;
        a.t0 = total;
        a.t1 = t_end;
        a.inner0 = inner;
        a.fp_first = do_restart ? 1 : 0;
        a.has_inner = has_inner_ ? 1 : 0;
        a.inner_limit = inner_limit_;
        a.use_al = use_al_ ? 1 : 0;
        a.tau = step_ / pw0;
        a.rho = step_ * pw0;
        a.sigma = use_al_ ? al_sigma_ : 0.0;
        a.fp32 = 0;
        a.polish = primal ? 1 : 2;
        launch(a, Q);
        read();
        major = (t_end % F) == 0;
        if (major || do_restart) fp = cl.fp;
        if (do_restart) {
            fp0 = cl.fp_first;
            do_restart = false;
        }
        inner += t_end - total;
        total = t_end;
    }
    if (status == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
        const size_t len = primal ? n : m;
        if (len)
            PDAL_CUDA(cudaMemcpyAsync(primal ? P_.xh : P_.yh, primal ? Q.xh : Q.yh, len * 8, cudaMemcpyDeviceToDevice,
                                      stream_));
    }
    PDAL_CUDA(cudaStreamSynchronize(stream_)); /* the phase's buffers are released next */
    polish_iters_ += total - 1;
    return status;
}

void FacpSolver::polish(double) { /* QP/FA_CP/src/solver.cu:156-160, fa_cp_core_op.cu:1242-1309 */
    polish_status_[0] = polish_status_[1] = -1;
    polish_iters_ = 0;
    polish_sec_ = 0.0;
    if (!p_.feasibility_polishing || reason_ == TERMINATION_REASON_PRIMAL_INFEASIBLE ||
        reason_ == TERMINATION_REASON_DUAL_INFEASIBLE)
        return;
    if (qtype_ != Q_NONE) {
        fprintf(stderr, "[fa_cp_gb300] feasibility polishing is built for problems without Q; solved without it\n");
        return;
    }
    const double t0 = now_sec();
    const auto &T = p_.termination_criteria;
    if (ctl_.rel_p < T.eps_feas_polish_relative && ctl_.rel_d < T.eps_feas_polish_relative) return;
    const double pw0 = p_.bound_objective_rescaling ? 1.0 : (H_.obj_norm + 1.0) / (H_.bnd_norm + 1.0);
    double a = 0, r = 0, o = 0;
    polish_status_[0] = polish_phase(true, pw0, a, r, o);
    if (polish_status_[0] == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
        ctl_.abs_p = a;
        ctl_.rel_p = r;
        ctl_.pobj = o;
    }
    polish_status_[1] = polish_phase(false, pw0, a, r, o);
    if (polish_status_[1] == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
        ctl_.abs_d = a;
        ctl_.rel_d = r;
        ctl_.dobj = o;
    }
    ctl_.gap = std::fabs(ctl_.pobj - ctl_.dobj);
    ctl_.rel_gap = ctl_.gap / (1.0 + std::fabs(ctl_.pobj) + std::fabs(ctl_.dobj));
    /* the result launch reads the controller block back */
    PDAL_CUDA(cudaMemcpyAsync(P_.ctl, &ctl_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    polish_sec_ = now_sec() - t0;
}

void FacpSolver::trajectory_header() const {
    const char *path = p_.trajectory_csv;
    if (!path || !path[0]) return;
    FILE *f = fopen(path, "w");
    if (!f) throw Error(std::string("cannot open trajectory CSV ") + path);
    fprintf(f, "iteration,time_sec,rel_primal,rel_dual,rel_gap,kkt_residual,fixed_point_residual,restart,al_sigma,"
               "sigma_update_count\n");
    fclose(f);
}

void FacpSolver::trajectory_row(double elapsed, bool restart) const {
    const char *path = p_.trajectory_csv;
    if (!path || !path[0]) return;
    FILE *f = fopen(path, "a");
    if (!f) throw Error(std::string("cannot append to trajectory CSV ") + path);
    const double kkt = std::fmax(ctl_.rel_p, std::fmax(ctl_.rel_d, ctl_.rel_gap));
    const double fp = total_ == 0 ? NAN : fp_;
    fprintf(f, "%d,%.17e,%.17e,%.17e,%.17e,%.17e,%.17e,%d,%.17e,%d\n", total_, elapsed, ctl_.rel_p, ctl_.rel_d,
            ctl_.rel_gap, kkt, fp, restart ? 1 : 0, al_sigma_, sigma_updates_);
    fclose(f);
}

void FacpSolver::print_eval() const {
    printf("%6d %.1e | %8.1e  %8.1e | %.1e %.1e %.1e | %.1e %.1e %.1e \n", total_, 0.0, ctl_.pobj, ctl_.dobj,
           ctl_.abs_p, ctl_.abs_d, ctl_.gap, ctl_.rel_p, ctl_.rel_d, ctl_.rel_gap);
}

fa_cp_result_t *FacpSolver::run() {
    const double t_begin = now_sec();
    prepare();
    upload();
    /* solver state */
    al_available_ = p_.use_al_qp;
    use_al_ = p_.use_al_qp;
    al_sigma_ = p_.al_sigma;
    best_al_sigma_ = p_.al_sigma;
    const double t_pow = now_sec();
    power_iterations();
    power_sec_ = now_sec() - t_pow;
    if (al_available_ && p_.al_sigma <= p_.sigma_zero_threshold) {
        use_al_ = false;
        al_sigma_ = 0.0;
    }
    has_inner_ = use_al_ || al_available_ || !(qtype_ == Q_NONE || qtype_ == Q_DIAG);
    inner_limit_ = nonconvexity_ < 0 ? 1 : 1000;
    ctl_ = Ctl{};
    ctl_.inner_tol = 1e-3;
    ctl_.fp = INFINITY;
    ctl_.fp_first = INFINITY;
    PDAL_CUDA(cudaMemcpyAsync(P_.ctl, &ctl_, sizeof(Ctl), cudaMemcpyHostToDevice, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    const double t_loop = now_sec();
    setup_sec_ = t_loop - t_begin;

    const int F = p_.termination_evaluation_frequency;
    const int limit = p_.termination_criteria.iteration_limit;
    fp32_ = o_.precision == 1;
    fp32_best_ = INFINITY;
    fp32_stall_ = 0;
    fp32_iters_ = 0;
    trajectory_header();
    bool major = false, do_restart = false;
    double elapsed = 0.0;
    while (total_ < limit) { /* QP/FA_CP/src/solver.cu:94-144 */
        const bool consider = major || total_ == 0;
        bool planned = false;
        if (consider || (total_ % print_frequency_host(total_) == 0)) {
            evaluate(major && total_ < 3 * F);
            elapsed = now_sec() - t_loop;
            check_termination(elapsed);
            if (consider && reason_ == TERMINATION_REASON_UNSPECIFIED) {
                choose_restart_candidate(elapsed);
                planned = should_restart();
            }
            trajectory_row(elapsed, planned);
            if (p_.verbose >= 2) print_eval();
            if (reason_ != TERMINATION_REASON_UNSPECIFIED) break;
            if (fp32_) { /* end of the FP32 phase: tolerance reached, or no halving for a while */
                const double kkt = std::fmax(ctl_.rel_p, std::fmax(ctl_.rel_d, ctl_.rel_gap));
                if (kkt < 0.5 * fp32_best_) {
                    fp32_best_ = kkt;
                    fp32_stall_ = 0;
                } else {
                    ++fp32_stall_;
                }
                if (kkt < o_.fp32_switch_tol || (o_.fp32_stall_evals > 0 && fp32_stall_ >= o_.fp32_stall_evals))
                    fp32_ = false;
            }
        }
        if (consider) {
            do_restart = planned;
            if (do_restart) perform_restart();
        }
        /* iterations up to the next evaluation point */
        int t_end = total_ + 1;
        while (t_end < limit && (t_end % F) != 0 && (t_end % print_frequency_host(t_end)) != 0) ++t_end;
        double tau = step_ / pw_;
        if (nonconvexity_ < 0) {
            tau = std::fmax(tau, -1.01 * std::fmin(0.0, nonconvexity_));
            tau /= 2;
        }
        Args a = base_args(MODE_SEGMENT);
        a.t0 = total_;
        a.t1 = t_end;
        a.inner0 = inner_;
        a.fp_first = do_restart ? 1 : 0;
        a.has_inner = has_inner_ ? 1 : 0;
        a.inner_limit = inner_limit_;
        a.use_al = use_al_ ? 1 : 0;
        a.tau = tau;
        a.rho = step_ * pw_;
        a.sigma = use_al_ ? al_sigma_ : 0.0;
        a.fp32 = fp32_ ? 1 : 0;
        if (fp32_) fp32_iters_ += t_end - total_;
        PDAL_CUDA(cudaEventRecord(ev0_, stream_));
        launch(a);
        PDAL_CUDA(cudaEventRecord(ev1_, stream_));
        read_ctl();
        float ms = 0.f;
        PDAL_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
        dev_ms_ += ms;
        major = (t_end % F) == 0;
        if (major || do_restart) fp_ = ctl_.fp;
        if (do_restart) {
            fp0_ = ctl_.fp_first;
            do_restart = false;
        }
        inner_ += t_end - total_;
        total_ = t_end;
    }
    if (reason_ == TERMINATION_REASON_UNSPECIFIED) {
        reason_ = TERMINATION_REASON_ITERATION_LIMIT;
        evaluate(false);
        trajectory_row(now_sec() - t_loop, false);
        if (p_.verbose >= 2) print_eval();
    }
    elapsed = now_sec() - t_loop;
    polish(t_loop);

    launch(base_args(MODE_RESULT));
    fa_cp_result_t *r = (fa_cp_result_t *)calloc(1, sizeof(fa_cp_result_t));
    if (!r) throw Error("out of host memory");
    const int n = H_.n, m = H_.m;
    r->primal_solution = (double *)malloc(sizeof(double) * (size_t)std::max(n, 1));
    r->dual_solution = (double *)malloc(sizeof(double) * (size_t)std::max(m, 1));
    r->reduced_cost = (double *)malloc(sizeof(double) * (size_t)std::max(n, 1));
    if (!r->primal_solution || !r->dual_solution || !r->reduced_cost) {
        fa_cp_result_free(r);
        throw Error("out of host memory");
    }
    PDAL_CUDA(cudaMemcpyAsync(r->primal_solution, P_.out_x, (size_t)n * 8, cudaMemcpyDeviceToHost, stream_));
    PDAL_CUDA(cudaMemcpyAsync(r->reduced_cost, P_.out_rc, (size_t)n * 8, cudaMemcpyDeviceToHost, stream_));
    if (m > 0) PDAL_CUDA(cudaMemcpyAsync(r->dual_solution, P_.out_y, (size_t)m * 8, cudaMemcpyDeviceToHost, stream_));
    read_ctl();
    r->num_variables = n;
    r->num_constraints = m;
    r->num_nonzeros = prob_->constraint_matrix_num_nonzeros;
    r->total_count = total_;
    r->total_inner_count = (int)ctl_.inner_total;
    r->rescaling_time_sec = rescale_sec_;
    r->cumulative_time_sec = elapsed;
    r->absolute_primal_residual = ctl_.abs_p;
    r->relative_primal_residual = ctl_.rel_p;
    r->absolute_dual_residual = ctl_.abs_d;
    r->relative_dual_residual = ctl_.rel_d;
    r->primal_objective_value = ctl_.pobj;
    r->dual_objective_value = ctl_.dobj;
    r->objective_gap = ctl_.gap;
    r->relative_objective_gap = ctl_.rel_gap;
    r->max_primal_ray_infeasibility = ctl_.max_pray;
    r->max_dual_ray_infeasibility = ctl_.max_dray;
    r->primal_ray_linear_objective = ctl_.pray_lin;
    r->dual_ray_objective = ctl_.dray_obj;
    r->final_al_sigma = al_sigma_;
    r->sigma_update_count = sigma_updates_;
    r->sigma_update_rule = al_available_ ? p_.sigma_update_rule : FA_CP_SIGMA_UPDATE_FIXED;
    r->termination_reason = reason_;
    r->feasibility_iteration = polish_iters_;
    r->feasibility_polishing_time = polish_sec_;

    fa_cp_gb300_stats_t &st = g_stats;
    memset(&st, 0, sizeof(st));
    st.setup_sec = setup_sec_;
    st.loop_sec = elapsed;
    st.total_sec = now_sec() - t_begin;
    st.max_singular_value = sv_max_;
    st.q_norm = qnorm_;
    st.q_nonconvexity = nonconvexity_;
    st.q_type = qtype_;
    st.grid_blocks = grid_;
    st.restarts = restarts_;
    st.evaluations = evals_;
    st.kernel_launches = launches_;
    st.inner_iterations = ctl_.inner_total;
    st.primal_weight = pw_;
    st.step_size = step_;
    st.device_loop_ms = dev_ms_;
    st.equilibration_sec = rescale_sec_;
    st.upload_sec = upload_sec_;
    st.power_sec = power_sec_;
    st.power_iterations_a = power_iters_a_;
    st.power_iterations_q = power_iters_q_;
    st.fp32_iterations = fp32_iters_;
    st.polish_primal_status = polish_status_[0];
    st.polish_dual_status = polish_status_[1];
    if (p_.verbose >= 1)
        printf("[fa_cp_gb300] %s after %d iterations (%lld inner), objective %.10e, rel. KKT %.2e, %.3f s\n",
               reason_ == TERMINATION_REASON_OPTIMAL ? "optimal" : "stopped", total_, (long long)ctl_.inner_total,
               ctl_.pobj, std::max(ctl_.rel_p, std::max(ctl_.rel_d, ctl_.rel_gap)), st.total_sec);
    return r;
}

fa_cp_result_t *solve_guarded(const qp_problem_t *prob, const fa_cp_parameters_t *params,
                              const fa_cp_gb300_options_t *opts) {
    g_error.clear();
    fa_cp_parameters_t p;
    if (params)
        p = *params;
    else
        set_default_parameters(&p);
    fa_cp_gb300_options_t o;
    if (opts)
        o = *opts;
    else
        fa_cp_gb300_default_options(&o);
    try {
        FacpSolver s(prob, p, o);
        return s.run();
    } catch (const std::exception &e) {
        g_error = e.what();
        fprintf(stderr, "[fa_cp_gb300] %s\n", e.what());
        return nullptr;
    }
}

} // namespace

void facp_set_last_error(const std::string &msg) { g_error = msg; }

} // namespace pdal

extern "C" {

fa_cp_result_t *solve_qp_problem(const qp_problem_t *prob, const fa_cp_parameters_t *params) {
    fa_cp_gb300_options_t o;
    fa_cp_gb300_options_from_env(&o);
    return pdal::solve_guarded(prob, params, &o);
}

fa_cp_result_t *fa_cp_gb300_solve(const qp_problem_t *prob, const fa_cp_parameters_t *params,
                                  const fa_cp_gb300_options_t *opts) {
    return pdal::solve_guarded(prob, params, opts);
}

int fa_cp_gb300_scaling(const qp_problem_t *prob, const fa_cp_parameters_t *params,
                        const fa_cp_gb300_options_t *opts, double *dcum, double *rcum, double *cbr_ovr) {
    pdal::g_error.clear();
    fa_cp_parameters_t p;
    if (params)
        p = *params;
    else
        set_default_parameters(&p);
    fa_cp_gb300_options_t o;
    if (opts)
        o = *opts;
    else
        fa_cp_gb300_default_options(&o);
    try {
        pdal::FacpSolver s(prob, p, o);
        s.scaling(dcum, rcum, cbr_ovr);
        return 0;
    } catch (const std::exception &e) {
        pdal::g_error = e.what();
        fprintf(stderr, "[fa_cp_gb300] %s\n", e.what());
        return -1;
    }
}

void fa_cp_gb300_last_stats(fa_cp_gb300_stats_t *stats) {
    if (stats) *stats = pdal::g_stats;
}

const char *fa_cp_gb300_last_error(void) { return pdal::g_error.c_str(); }

void fa_cp_gb300_rand_sequence(unsigned seed, int count, int *out) {
    pdal::CRandom r(seed);
    for (int i = 0; i < count; ++i) out[i] = r.next();
}

} // extern "C"

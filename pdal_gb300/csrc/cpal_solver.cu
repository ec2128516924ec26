/*
 * cpal_solver.cu -- host driver of the CP_AL (LP) solver on one GPU.
 *
 * Control flow follows optimize() of the reference (LP/CP_AL/src/solver.cu:
 * 1175-1736): equilibrate, estimate sigma_max(A)^2, then repeat evaluation
 * blocks of F iterations until the KKT test passes.  Differences in form:
 *   - a block (F iterations + evaluation + controller + restart) is one CUDA
 *     graph; the host reads back one small struct per block and never
 *     synchronises inside it (the reference synchronises ~10 times per block);
 *   - every product is a fused row-block kernel (rowblock.cuh), no cuSPARSE,
 *     cuBLAS or CUB;
 *   - FP32_REFINE runs the iteration in FP32 (FP64 anchors and reductions)
 *     until the KKT error falls below fp32_switch_tol, then continues in FP64
 *     from the FP32 iterate.
 */
#include "../../include/cp_al.h"
#include "../../include/cp_al_gb300.h"
#include "common.h"
#include "cpal_kernels.cuh"
#include "cpal_setup.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <type_traits>

namespace pdal {

namespace {

thread_local cp_al_gb300_stats_t g_stats;

double now_sec() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int grid_for(long long len, int per_block = kThreads) {
    long long g = (len + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > 152 * 8) g = 152 * 8;
    return (int)g;
}

#define PDAL_LAUNCH_CHECK() PDAL_CUDA(cudaGetLastError())

/* Lanczos steps at most, and the steps between two convergence checks */
/* On the large LP the largest Ritz value after 128 steps (0.99989) is already
 * above the reference's power-iteration estimate after 5,000 steps (0.99987);
 * it is a lower bound, and the step's 0.998 margin covers the rest. */
constexpr int kLanczosMax = 128;
constexpr int kLanczosChunk = 16;

/* Largest eigenvalue of the symmetric tridiagonal matrix with diagonal a[0..k)
 * and off-diagonal b[0..k-1), by bisection on the Sturm count (the number of
 * negative pivots of T - x I). */
double tridiag_max_eig(const std::vector<double> &a, const std::vector<double> &b, int k) {
    double lo = 0.0, hi = 0.0;
    for (int i = 0; i < k; ++i) {
        const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < k ? std::fabs(b[i]) : 0.0);
        hi = std::max(hi, a[i] + r);
        lo = std::min(lo, a[i] - r);
    }
    auto below = [&](double x) { /* eigenvalues < x */
        int cnt = 0;
        double d = 1.0;
        for (int i = 0; i < k; ++i) {
            d = a[i] - x - (i > 0 ? b[i - 1] * b[i - 1] / d : 0.0);
            if (d == 0.0) d = -1e-300;
            if (d < 0.0) ++cnt;
        }
        return cnt;
    };
    for (int it = 0; it < 200 && hi - lo > 1e-15 * std::max(1.0, std::fabs(hi)); ++it) {
        const double mid = 0.5 * (lo + hi);
        if (below(mid) >= k) /* every eigenvalue is below mid */
            hi = mid;
        else
            lo = mid;
    }
    return hi;
}

/* Dispatch on the row-block nonzero budget. */
#define PDAL_WITH_S(Sval, ...)                     \
    switch (Sval) {                                 \
    case 256: {                                     \
        constexpr int SB = 256;                     \
        __VA_ARGS__;                                \
    } break;                                        \
    case 512: {                                     \
        constexpr int SB = 512;                     \
        __VA_ARGS__;                                \
    } break;                                        \
    case 1024: {                                    \
        constexpr int SB = 1024;                    \
        __VA_ARGS__;                                \
    } break;                                        \
    case 2048: {                                    \
        constexpr int SB = 2048;                    \
        __VA_ARGS__;                                \
    } break;                                        \
    default:                                        \
        throw Error("unsupported row-block budget"); \
    }

#define PDAL_WITH_SE(Sval, ...)                    \
    switch (Sval) {                                 \
    case 256: {                                     \
        constexpr int SE = 256;                     \
        __VA_ARGS__;                                \
    } break;                                        \
    case 512: {                                     \
        constexpr int SE = 512;                     \
        __VA_ARGS__;                                \
    } break;                                        \
    case 1024: {                                    \
        constexpr int SE = 1024;                    \
        __VA_ARGS__;                                \
    } break;                                        \
    default:                                        \
        throw Error("unsupported row-block budget"); \
    }

struct PlanDev {
    HostPlan hp;
    RowPlanDev d{};
};

struct DevMatrix {
    int nr = 0, nc = 0, nnz = 0;
    int *rp = nullptr, *ci = nullptr;
    double *v = nullptr;
    float *vf = nullptr;
    PlanDev it, ev;
};

template <typename T>
struct IterVecs {
    /* n */
    T *x = nullptr, *xbar = nullptr, *xh = nullptr, *lam = nullptr, *c = nullptr, *vlb = nullptr, *vub = nullptr;
    /* m */
    T *y = nullptr, *yh = nullptr, *ybar = nullptr, *ax = nullptr, *u = nullptr, *clb = nullptr, *cub = nullptr;
};

} // namespace

class CpalSolver {
  public:
    CpalSolver(const lp_problem_t *prob, const cp_al_parameters_t *params, const cp_al_gb300_options_t *opts)
        : prob_(prob), P_(*params), O_(*opts) {}
    ~CpalSolver() { release(); }

    /* host-side preparation that needs no device work */
    void prepare();
    /* allocate + upload the pristine problem */
    void upload();
    /* reset working buffers from the pristine copy, then equilibrate, power
     * iteration and initial schedule */
    void setup_device();
    void run_loop();
    /* feasibility polishing after the loop (LP/CP_AL/src/solver.cu:3912-4456) */
    void polish();
    double polish_sec = 0.0;
    double loop_t0_ = 0.0; /* wall clock at the start of the loop (time limit) */
    int polish_iters = 0;
    int polish_status[2] = {-1, -1};
    /* extends the iteration limit by n and continues (session iterate) */
    bool extend(int n);
    void download(cp_al_result_t *res, bool vectors);
    void result_on_device();
    void fetch_vectors(double *x, double *y, double *rc);
    void fetch_scaling(double *vals, double *rsc, double *csc, double *bo);

    CpalState host_state{};
    double setup_sec = 0, loop_sec = 0;
    double prepare_sec = 0, upload_sec = 0, equil_sec = 0, power_sec = 0;
    double upload_plan_sec = 0, upload_alloc_sec = 0; /* parts of upload_sec */
    int64_t launches = 0;
    int64_t h2d = 0, d2h = 0;
    int power_iters = 0;
    int cr_passes = 0; /* Curtis-Reid passes run (early stop may end them at 5) */
    int fp32_iters = 0;
    bool started = false;
    double sum_ms[2][3] = {{0, 0, 0}, {0, 0, 0}}; /* [fp64, fp32][primal, dual, block] */
    double sub_ms[2][2] = {{0, 0}, {0, 0}};       /* [fp64, fp32][dual short rows, dual panels] */
    int timed[2] = {0, 0};

  private:
    void release();
    template <typename T>
    void capture_block(cudaGraphExec_t &exec, int F);
    template <typename T>
    void launch_iteration(int koff, bool major);
    template <typename T>
    void launch_primal(int koff, bool major);
    template <typename T>
    void launch_dual(int koff, bool major, bool timed = false);
    template <typename T>
    void launch_eval();
    template <typename T>
    void launch_eval_terms();
    template <typename T>
    void launch_init_ax();
    template <typename T>
    IterVecs<T> &vecs();
    void power_iteration();
    void lanczos();
    /* the chosen form estimates sigma_max^2 by Lanczos unless told otherwise */
    bool use_lanczos() const { return m_ > 0 && fp32_phase_ && O_.power_method != 0; }
    void switch_to_fp64();
    void alloc_plan(PlanDev &pd);
    void upload_plan(PlanDev &pd);
    void alloc_all();

    const lp_problem_t *prob_;
    cp_al_parameters_t P_;
    cp_al_gb300_options_t O_;
    CpalParams cp_{};
    int n_ = 0, m_ = 0, nnz_ = 0;
    HostCsr At_host_;
    /* A^T built on the device from its host row pointers (k_transpose_*),
     * or on the host threads when a column is too long for the device sort */
    bool device_transpose_ = false;
    int *at_cursor_ = nullptr, *hot_id_d_ = nullptr;
    int S_it_ = 2048, S_ev_ = 1024;
    bool beta_on_ = false;
    bool fp32_phase_ = false;

    Arena arena_;
    cudaStream_t stream_ = nullptr;
    DevMatrix A_, At_;
    /* the long rows of the iteration's A x by column panels (HostPanels in
     * common.h); the iteration's row blocks then cover the other rows */
    bool use_panels_ = false;
    HostPanels pan_host_;
    /* the other rows of A: at most one entry (one thread each, compact copy)
     * and 2..S entries (one warp each) -- k_dual_short */
    std::vector<int> sh_r1_h, sh_p1_h, sh_c1_h, sh_r2_h, sh_r3_h;
    int *sh_r1_ = nullptr, *sh_p1_ = nullptr, *sh_c1_ = nullptr, *sh_r2_ = nullptr, *sh_r3_ = nullptr;
    double *sh_v64_ = nullptr;
    float *sh_v32_ = nullptr;
    int sh_b1_ = 0, sh_b2_ = 0, sh_b3_ = 0;
    template <typename T>
    ShortDev<T> short_dev() const;
    template <typename T>
    T *hot_ptr() const;
    /* shared-memory hot values in the primal product of the phase in T:
     * measured faster for FP64 and slower for FP32 on the large LP, so by
     * default only the FP64 phase uses them */
    template <typename T>
    bool hot_in() const {
        return use_hot_ && (std::is_same<T, double>::value || O_.primal_hot_rows == 1);
    }
    int *pan_rows_ = nullptr, *pan_pmap_ = nullptr;
    int4 *pan_seg_ = nullptr, *pan_piece_ = nullptr, *pan_cta_ = nullptr;
    uint16_t *pan_off_ = nullptr;
    double *pan_v64_ = nullptr, *pan_part64_ = nullptr;
    /* the fused finish of the long rows: arrivals and segments per long row */
    bool fuse_finish_ = false;
    /* the dual step's short-row and panel launches on two streams (forked and
     * joined with events, also inside the captured graphs) */
    bool dual_fork_ = false;   /* in the FP64 phase */
    bool dual_fork32_ = false; /* also in the FP32 phase */
    template <typename T>
    bool forked() const { return dual_fork_ && (dual_fork32_ || std::is_same<T, double>::value); }
    cudaStream_t side_ = nullptr;
    cudaEvent_t fork_ev_ = nullptr, join_ev_ = nullptr;
    unsigned *pan_cnt_ = nullptr;
    int *pan_nseg_ = nullptr;
    float *pan_v32_ = nullptr, *pan_part32_ = nullptr;
    /* the same long rows' gathered values in shared memory in the primal
     * product (k_primal_hot): A^T's column indices with entry -1 - h for long
     * row h, and the compact copy of those values */
    bool use_hot_ = false;
    int hot_grid_[2][2] = {{0, 0}, {0, 0}}; /* [FP64?][major?]: one wave of k_primal_hot */
    /* the staged primal product (k_primal_tma): one wave per variant, and
     * the flag a staging wait that ran out sets */
    bool use_staged_ = false;
    int staged_grid_[2][2] = {{0, 0}, {0, 0}};
    int *dev_err_ = nullptr;
    /* rows longer than kEqShort nonzeros (equilibration: a warp each) */
    std::vector<int> eq_long_h_[2];
    int *eq_long_[2] = {nullptr, nullptr}; /* [A, A^T] */
    void setup_staged();
    /* the persistent cooperative loop (k_cpal_loop) for small LPs */
    bool use_loop_ = false;
    int loop_grid_[2] = {0, 0}; /* [FP64?] */
    LoopBar *loop_bar_ = nullptr;
    void setup_loop();
    template <typename T>
    void launch_loop(int max_blocks);
    bool staged_rows() const { return O_.primal_staged == 2; }
    void check_device_error();
    int *At_ci_hot_ = nullptr;
    double *hot64_ = nullptr;
    float *hot32_ = nullptr;
    template <typename T>
    PanelDev<T> panel_dev() const;
    /* kernels one iteration launches */
    int iter_launches() const {
        return 1 + (m_ == 0 ? 0 : use_panels_ ? (sh_b1_ + sh_b2_ + sh_b3_ > 0 ? 2 : 1) + (fuse_finish_ ? 0 : 1) : 1);
    }

  public:
    int panel_rows() const { return use_panels_ ? pan_host_.H : 0; }
    int panels() const { return use_panels_ ? pan_host_.P : 0; }

  private:
    /* pristine copies (session solves start from these) */
    double *Av0_ = nullptr, *Atv0_ = nullptr, *c0_ = nullptr, *vlb0_ = nullptr, *vub0_ = nullptr, *clb0_ = nullptr,
           *cub0_ = nullptr, *x00_ = nullptr, *y00_ = nullptr;
    /* FP64 working data */
    double *c_ = nullptr, *vlb_ = nullptr, *vub_ = nullptr, *clb_ = nullptr, *cub_ = nullptr, *clbf_ = nullptr,
           *cubf_ = nullptr;
    double *x0_ = nullptr, *y0_ = nullptr, *ax0_ = nullptr, *phat_ = nullptr, *dsc_ = nullptr, *rsc_ = nullptr;
    double *tmp_n_ = nullptr, *tmp_m_ = nullptr, *tmp_m2_ = nullptr;
    double *part_row_ = nullptr, *part_col_ = nullptr, *part_misc_ = nullptr;
    double *part_ray_row_ = nullptr, *part_ray_col_ = nullptr; /* infeasibility detection */
    double *xout_ = nullptr, *yout_ = nullptr, *rcout_ = nullptr;
    float2 *x0f_ = nullptr, *y0f_ = nullptr, *ax0f_ = nullptr; /* FP32-phase anchors (hi, lo) */
    HalpernW *wt_ = nullptr;
    HalpernWf *wtf_ = nullptr;
    IterVecs<double> v64_;
    IterVecs<float> v32_;
    CpalState *st_ = nullptr;
    PowerState *ps_ = nullptr;
    /* Lanczos coefficients and step counter (chosen form's sigma_max^2) */
    double *lz_alpha_ = nullptr, *lz_beta_ = nullptr;
    int *lz_j_ = nullptr;
    CpalState *h_st_ = nullptr; /* pinned */
    PowerState *h_ps_ = nullptr;
    /* one graph per precision, predictor form and block length (the alpha
     * pulse and the sigma trigger switch the AL predictor on and off between
     * blocks, the dynamic evaluation frequency shortens the blocks):
     * [predictor][short blocks] */
    cudaGraphExec_t exec64_[2][2] = {}, exec32_[2][2] = {};
    /* the alpha pulse as the host last saw it, for its stderr lines */
    int pulse_seen_gate_ = 0, pulse_seen_phase_ = 0, pulse_gate_iter_ = 0, pulse_gate_k_[2] = {0, 0};
    bool dyn_reported_ = false;
    double pulse_gate_rate_[2] = {0.0, 0.0};
    void pulse_report();
    /* evaluation blocks per graph launch: 1 while a controller may change the
     * step form between blocks */
    int graph_blocks() const { return (cp_.pulse || cp_.trigger || cp_.dyn) ? 1 : std::max(1, O_.graph_blocks); }
    int nmisc_ = 0;
    cudaEvent_t ev_[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
};

template <>
IterVecs<double> &CpalSolver::vecs<double>() {
    return v64_;
}
template <>
IterVecs<float> &CpalSolver::vecs<float>() {
    return v32_;
}

template <>
double *CpalSolver::hot_ptr<double>() const {
    return hot64_;
}
template <>
float *CpalSolver::hot_ptr<float>() const {
    return hot32_;
}

template <>
ShortDev<double> CpalSolver::short_dev<double>() const {
    return ShortDev<double>{sh_r1_, sh_c1_, sh_v64_, sh_r2_, sh_r3_, (int)sh_r1_h.size(), (int)sh_r2_h.size(),
                            (int)sh_r3_h.size(), sh_b1_, sh_b2_, sh_b3_};
}
template <>
ShortDev<float> CpalSolver::short_dev<float>() const {
    return ShortDev<float>{sh_r1_, sh_c1_, sh_v32_, sh_r2_, sh_r3_, (int)sh_r1_h.size(), (int)sh_r2_h.size(),
                           (int)sh_r3_h.size(), sh_b1_, sh_b2_, sh_b3_};
}

template <>
PanelDev<double> CpalSolver::panel_dev<double>() const {
    return PanelDev<double>{pan_rows_, pan_seg_, pan_piece_, pan_cta_, pan_v64_, pan_off_, pan_part64_,
                            hot_in<double>() ? hot64_ : nullptr,
                            pan_host_.H, pan_host_.P, pan_host_.W, (int)(pan_host_.cta.size() / 4), pan_cnt_,
                            pan_nseg_};
}
template <>
PanelDev<float> CpalSolver::panel_dev<float>() const {
    return PanelDev<float>{pan_rows_, pan_seg_, pan_piece_, pan_cta_, pan_v32_, pan_off_, pan_part32_,
                           hot_in<float>() ? hot32_ : nullptr,
                           pan_host_.H, pan_host_.P, pan_host_.W, (int)(pan_host_.cta.size() / 4), pan_cnt_,
                           pan_nseg_};
}

void CpalSolver::release() {
    for (auto &e : ev_)
        if (e) cudaEventDestroy(e);
    for (auto *e : {&fork_ev_, &join_ev_}) {
        if (*e) cudaEventDestroy(*e);
        *e = nullptr;
    }
    if (side_) cudaStreamDestroy(side_);
    side_ = nullptr;
    for (auto *tab : {&exec64_, &exec32_})
        for (auto &row : *tab)
            for (auto &e : row) {
                if (e) cudaGraphExecDestroy(e);
                e = nullptr;
            }
    if (h_st_) cudaFreeHost(h_st_);
    if (h_ps_) cudaFreeHost(h_ps_);
    h_st_ = nullptr;
    h_ps_ = nullptr;
    arena_.release();
    if (stream_) cudaStreamDestroy(stream_);
    stream_ = nullptr;
}

/* Controller parameters of one solve: options resolved against the
 * parameters (NaN options fall back to them), and the norms of the unscaled
 * problem (LP/CP_AL/src/solver.cu:1999-2067). */
CpalParams resolve_cpal_params(const cp_al_parameters_t &P, const cp_al_gb300_options_t &O, const lp_problem_t *prob) {
    CpalParams cp{};
    const auto &R = P.restart_params;
    cp.F = P.termination_evaluation_frequency;
    cp.iteration_limit = P.termination_criteria.iteration_limit;
    cp.time_limit = P.termination_criteria.time_sec_limit;
    cp.eps_opt = P.termination_criteria.eps_optimal_relative;
    cp.eps_feas = P.termination_criteria.eps_feasible_relative;
    cp.norm_linf = P.optimality_norm == NORM_TYPE_L_INF;
    cp.refl = P.reflection_coefficient;
    cp.suff = std::isnan(O.restart_sufficient) ? R.sufficient_reduction_for_restart : O.restart_sufficient;
    cp.nec = std::isnan(O.restart_necessary) ? R.necessary_reduction_for_restart : O.restart_necessary;
    cp.art = std::isnan(O.restart_artificial) ? R.artificial_restart_threshold : O.restart_artificial;
    cp.kp = R.k_p;
    cp.ki = R.k_i;
    cp.kd = R.k_d;
    cp.ismooth = R.i_smooth;
    cp.sigma_mode = O.sigma_mode != 0;
    cp.sigma_adaptive = O.sigma_adaptive != 0;
    cp.s_kp = std::isnan(O.sigma_kp) ? R.k_p : O.sigma_kp;
    cp.s_ki = std::isnan(O.sigma_ki) ? R.k_i : O.sigma_ki;
    cp.s_kd = std::isnan(O.sigma_kd) ? R.k_d : O.sigma_kd;
    cp.s_ismooth = std::isnan(O.sigma_i_smooth) ? R.i_smooth : O.sigma_i_smooth;
    cp.s_gain = O.sigma_balance_gain;
    cp.s_umin = O.sigma_update_min;
    cp.s_umax = O.sigma_update_max;
    cp.step_margin = O.step_margin;
    cp.lambda_factor = O.lambda_factor;
    cp.lambda_param_set = O.lambda_param_set;
    cp.lambda_param_opt = O.lambda_param;
    cp.restart_select = O.restart_select;
    cp.restart_select_min_iters = O.restart_select_min_iters;
    cp.restart_select_margin = O.restart_select_margin;
    cp.restart_select_min_time = O.restart_select_min_time;
    /* LP/CP_AL/src/solver.cu:2774-2775: mode 3, or the three-point switch
     * with any other nonzero mode */
    cp.restart_threepoint = O.restart_select != 0 && (O.restart_select == 3 || O.restart_select_threepoint != 0);
    cp.infeas = O.infeasibility_detection != 0;
    cp.eps_infeas = O.eps_infeasible;
    cp.pulse = O.alpha_direct_pulse != 0;
    cp.pulse_force = O.pulse_force != 0;
    cp.pulse_test_limit = O.pulse_test_limit;
    cp.trigger = O.sigma_trigger != 0;
    cp.trigger_min_iters = O.sigma_trigger_min_iters;
    cp.trigger_p = O.sigma_trigger_primal;
    cp.trigger_d = O.sigma_trigger_dual;
    cp.trigger_ratio = O.sigma_trigger_ratio;
    cp.sigma_set = O.sigma_set;
    cp.sigma_value = O.sigma;
    cp.sigma_init_f = O.sigma_init_factor;
    cp.sigma_min_f = O.sigma_min_factor;
    cp.sigma_max_f = O.sigma_max_factor;
    /* LP/CP_AL/src/solver.cu:1229-1255 */
    const int F = cp.F;
    cp.dyn_fast = std::min(std::max(O.dynamic_eval_fast, 3), F);
    cp.dyn_resid = O.dynamic_eval != 0;
    cp.dyn_sec = O.dynamic_eval_after_sec;
    cp.dyn_iters = O.dynamic_eval_after_iters;
    cp.dyn = (cp.dyn_resid || cp.dyn_sec > 0.0 || cp.dyn_iters > 0) && cp.dyn_fast < F;
    cp.dyn_min_iters = std::max(O.dynamic_eval_min_iters > 0 ? O.dynamic_eval_min_iters : F, F);
    cp.dyn_small = O.dynamic_eval_small_res;
    cp.dyn_large = O.dynamic_eval_large_res;
    cp.dyn_ratio = O.dynamic_eval_ratio;
    cp.dyn_boot = std::max(O.dynamic_eval_bootstrap_iters, 0);
    cp.cr_early_stopped = 0; /* set after the equilibration */
    cp.obj_const = prob->objective_constant;
    const int n = prob->num_variables, m = prob->num_constraints;
    const bool linf = cp.norm_linf;
    double s = 0, mx = 0;
    for (int j = 0; j < n; ++j) {
        const double v = prob->objective_vector[j];
        if (linf)
            mx = std::fmax(mx, std::fabs(v));
        else
            s += v * v;
    }
    cp.obj_norm = linf ? mx : std::sqrt(s);
    s = 0;
    mx = 0;
    for (int i = 0; i < m; ++i) {
        const double lo = prob->constraint_lower_bound[i], up = prob->constraint_upper_bound[i];
        if (linf) {
            if (std::isfinite(lo) && lo != up) mx = std::fmax(mx, std::fabs(lo));
            if (std::isfinite(up)) mx = std::fmax(mx, std::fabs(up));
        } else {
            if (std::isfinite(lo) && lo != up) s += lo * lo;
            if (std::isfinite(up)) s += up * up;
        }
    }
    cp.bnd_norm = linf ? mx : std::sqrt(s);
    return cp;
}

void CpalSolver::prepare() {
    const double t_prep = now_sec();
    n_ = prob_->num_variables;
    m_ = prob_->num_constraints;
    nnz_ = prob_->constraint_matrix_num_nonzeros;
    if (n_ <= 0) throw Error("problem has no variables");
    if (m_ < 0) throw Error("negative number of constraints");
    if (P_.termination_evaluation_frequency < 3)
        throw Error("termination_evaluation_frequency must be >= 3 (got " +
                    std::to_string(P_.termination_evaluation_frequency) + ")");
    if (!prob_->objective_vector || !prob_->variable_lower_bound || !prob_->variable_upper_bound)
        throw Error("problem vectors missing");
    if (m_ > 0 && (!prob_->constraint_lower_bound || !prob_->constraint_upper_bound))
        throw Error("constraint bounds missing");
    csr_validate(m_, n_, prob_->constraint_matrix_row_pointers, prob_->constraint_matrix_col_indices, nnz_,
                 "constraint matrix");
    At_host_.rp = csr_transpose_rp(m_, n_, prob_->constraint_matrix_row_pointers, prob_->constraint_matrix_col_indices);
    int longest = 0;
    for (int j = 0; j < n_; ++j) longest = std::max(longest, At_host_.rp[j + 1] - At_host_.rp[j]);
    device_transpose_ = O_.device_transpose != 0 && longest <= kTransposeSort;
    At_host_.nr = n_;
    At_host_.nc = m_;
    if (!device_transpose_)
        At_host_ = csr_transpose(m_, n_, prob_->constraint_matrix_row_pointers, prob_->constraint_matrix_col_indices,
                                 prob_->constraint_matrix_values);
    S_it_ = O_.spmv_nnz_per_block > 0 ? O_.spmv_nnz_per_block : auto_block_nnz(nnz_, std::max(m_, n_));
    if (S_it_ != 256 && S_it_ != 512 && S_it_ != 1024 && S_it_ != 2048)
        throw Error("spmv_nnz_per_block must be 256, 512, 1024 or 2048");
    S_ev_ = std::min(S_it_, 1024);

    cp_ = resolve_cpal_params(P_, O_, prob_);
    fp32_phase_ = O_.precision == CP_AL_GB300_FP32_REFINE;
    prepare_sec = now_sec() - t_prep;
}

void CpalSolver::alloc_plan(PlanDev &pd) {
    pd.d.nblocks = pd.hp.nblocks;
    pd.d.nlong = pd.hp.nlong;
    pd.d.desc = arena_.take<int4>(std::max(pd.hp.nblocks, 1));
    pd.d.linfo = arena_.take<int4>(std::max(pd.hp.nlong, 1));
    pd.d.lpart = arena_.take<double>(kLongStride * (size_t)std::max(pd.hp.npieces, 1));
    pd.d.lcount = arena_.take<unsigned>(std::max(pd.hp.nlong, 1));
}

void CpalSolver::upload_plan(PlanDev &pd) {
    if (pd.hp.nblocks)
        PDAL_CUDA(cudaMemcpyAsync((void *)pd.d.desc, pd.hp.desc.data(), pd.hp.desc.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, stream_));
    if (pd.hp.nlong)
        PDAL_CUDA(cudaMemcpyAsync((void *)pd.d.linfo, pd.hp.linfo.data(), pd.hp.linfo.size() * sizeof(int),
                                  cudaMemcpyHostToDevice, stream_));
    PDAL_CUDA(cudaMemsetAsync(pd.d.lcount, 0, sizeof(unsigned) * std::max(pd.hp.nlong, 1), stream_));
    h2d += (pd.hp.desc.size() + pd.hp.linfo.size()) * sizeof(int);
}

void CpalSolver::alloc_all() {
    const size_t n = n_, m = m_, nnz = nnz_;
    /* +kPad: the row-block loads read 4-element windows that may extend
     * three elements past the last nonzero */
    constexpr size_t kPad = 8;
    A_.rp = arena_.take<int>(m + 1);
    A_.ci = arena_.take<int>(nnz + kPad);
    A_.v = arena_.take<double>(nnz + kPad);
    Av0_ = arena_.take<double>(nnz + kPad);
    At_.rp = arena_.take<int>(n + 1);
    At_.ci = arena_.take<int>(nnz + kPad);
    At_.v = arena_.take<double>(nnz + kPad);
    Atv0_ = arena_.take<double>(nnz + kPad);
    if (fp32_phase_) {
        A_.vf = arena_.take<float>(nnz + kPad);
        At_.vf = arena_.take<float>(nnz + kPad);
    }
    alloc_plan(A_.it);
    alloc_plan(At_.it);
    alloc_plan(A_.ev);
    alloc_plan(At_.ev);
    dev_err_ = arena_.take<int>(1);
    for (int q = 0; q < 2; ++q) eq_long_[q] = arena_.take<int>(std::max<size_t>(eq_long_h_[q].size(), 1));
    if (device_transpose_) at_cursor_ = arena_.take<int>(n + 1);
    if (device_transpose_ && use_hot_) hot_id_d_ = arena_.take<int>(std::max<size_t>(m, 1));
    loop_bar_ = arena_.take<LoopBar>(1);
    if (use_panels_) {
        const size_t len = (size_t)pan_host_.len, hp = (size_t)pan_host_.H * pan_host_.P;
        const size_t n1 = std::max<size_t>(sh_r1_h.size(), 1), n2 = std::max<size_t>(sh_r2_h.size(), 1),
                     n3 = std::max<size_t>(sh_r3_h.size(), 1);
        sh_r1_ = arena_.take<int>(n1);
        sh_p1_ = arena_.take<int>(n1);
        sh_c1_ = arena_.take<int>(n1);
        sh_r2_ = arena_.take<int>(n2);
        sh_r3_ = arena_.take<int>(n3);
        sh_v64_ = arena_.take<double>(n1);
        if (fp32_phase_) sh_v32_ = arena_.take<float>(n1);
        pan_rows_ = arena_.take<int>(pan_host_.rows.size());
        pan_pmap_ = arena_.take<int>(len);
        pan_seg_ = arena_.take<int4>(pan_host_.seg.size() / 4);
        pan_piece_ = arena_.take<int4>(pan_host_.piece.size() / 4);
        pan_cta_ = arena_.take<int4>(pan_host_.cta.size() / 4);
        pan_off_ = arena_.take<uint16_t>(len);
        if (use_hot_) {
            At_ci_hot_ = arena_.take<int>(nnz + kPad);
            hot64_ = arena_.take<double>(pan_host_.H);
            if (fp32_phase_ && O_.primal_hot_rows == 1) hot32_ = arena_.take<float>(pan_host_.H);
        }
        pan_v64_ = arena_.take<double>(len);
        pan_part64_ = arena_.take<double>(hp);
        pan_cnt_ = arena_.take<unsigned>(std::max(pan_host_.H, 1));
        pan_nseg_ = arena_.take<int>(std::max(pan_host_.H, 1));
        if (fp32_phase_) {
            pan_v32_ = arena_.take<float>(len);
            pan_part32_ = arena_.take<float>(hp);
        }
    }
    c0_ = arena_.take<double>(n);
    vlb0_ = arena_.take<double>(n);
    vub0_ = arena_.take<double>(n);
    x00_ = arena_.take<double>(n);
    clb0_ = arena_.take<double>(m);
    cub0_ = arena_.take<double>(m);
    y00_ = arena_.take<double>(m);
    c_ = arena_.take<double>(n);
    vlb_ = arena_.take<double>(n);
    vub_ = arena_.take<double>(n);
    x0_ = arena_.take<double>(n);
    dsc_ = arena_.take<double>(n);
    tmp_n_ = arena_.take<double>(n);
    xout_ = arena_.take<double>(n);
    rcout_ = arena_.take<double>(n);
    clb_ = arena_.take<double>(m);
    cub_ = arena_.take<double>(m);
    clbf_ = arena_.take<double>(m);
    cubf_ = arena_.take<double>(m);
    y0_ = arena_.take<double>(m);
    ax0_ = arena_.take<double>(m);
    phat_ = arena_.take<double>(m);
    rsc_ = arena_.take<double>(m);
    tmp_m_ = arena_.take<double>(m);
    tmp_m2_ = arena_.take<double>(m);
    yout_ = arena_.take<double>(m);
    {
        auto &v = v64_;
        v.x = arena_.take<double>(n);
        v.xbar = arena_.take<double>(n);
        v.xh = arena_.take<double>(n);
        v.lam = arena_.take<double>(n);
        v.c = c_;
        v.vlb = vlb_;
        v.vub = vub_;
        v.y = arena_.take<double>(m);
        v.yh = arena_.take<double>(m);
        v.ybar = arena_.take<double>(m);
        v.ax = arena_.take<double>(m);
        v.u = arena_.take<double>(m);
        v.clb = clb_;
        v.cub = cub_;
    }
    if (fp32_phase_) {
        auto &v = v32_;
        v.x = arena_.take<float>(n);
        v.xbar = arena_.take<float>(n);
        v.xh = arena_.take<float>(n);
        v.lam = arena_.take<float>(n);
        v.c = arena_.take<float>(n);
        v.vlb = arena_.take<float>(n);
        v.vub = arena_.take<float>(n);
        v.y = arena_.take<float>(m);
        v.yh = arena_.take<float>(m);
        v.ybar = arena_.take<float>(m);
        v.ax = arena_.take<float>(m);
        v.u = arena_.take<float>(m);
        v.clb = arena_.take<float>(m);
        v.cub = arena_.take<float>(m);
    }
    if (fp32_phase_) {
        x0f_ = arena_.take<float2>(n);
        y0f_ = arena_.take<float2>(m);
        ax0f_ = arena_.take<float2>(m);
    }
    wt_ = arena_.take<HalpernW>((size_t)cp_.F + 1);
    wtf_ = arena_.take<HalpernWf>((size_t)cp_.F + 1);
    part_row_ = arena_.take<double>((size_t)(A_.ev.hp.nblocks + A_.ev.hp.nlong + 1) * kEvalStride);
    part_col_ = arena_.take<double>((size_t)(At_.ev.hp.nblocks + At_.ev.hp.nlong + 1) * kEvalStride);
    if (cp_.infeas) {
        part_ray_row_ = arena_.take<double>((size_t)(A_.ev.hp.nblocks + A_.ev.hp.nlong + 1) * kEvalStride);
        part_ray_col_ = arena_.take<double>((size_t)(At_.ev.hp.nblocks + At_.ev.hp.nlong + 1) * kEvalStride);
    }
    nmisc_ = std::max({A_.ev.hp.nblocks + A_.ev.hp.nlong, A_.it.hp.nblocks + A_.it.hp.nlong,
                       grid_for(std::max(n_, m_)), 1});
    part_misc_ = arena_.take<double>(2 * (size_t)nmisc_ + 2);
    st_ = arena_.take<CpalState>(1);
    ps_ = arena_.take<PowerState>(1);
    lz_alpha_ = arena_.take<double>(kLanczosMax);
    lz_beta_ = arena_.take<double>(kLanczosMax);
    lz_j_ = arena_.take<int>(1);
}

/* The staged primal product needs more than 48 KB of dynamic shared memory
 * per block; its grid is one wave at the occupancy that leaves. */
void CpalSolver::setup_staged() {
    use_staged_ = O_.primal_staged > 0 && n_ > 0;
    if (!use_staged_) return;
    int dev = 0, sms = 0;
    PDAL_CUDA(cudaGetDevice(&dev));
    PDAL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    auto wave = [&](auto kernel, size_t smem) {
        PDAL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0;
        PDAL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kThreads, smem));
        if (occ < 1) throw Error("staged primal product does not fit on this device");
        return std::max(1, std::min(At_.it.hp.nblocks, occ * sms));
    };
    PDAL_WITH_S(S_it_, {
        if (staged_rows()) {
            constexpr size_t s32 = sizeof(PrimalTmaSmem<SB, float, true>),
                             s64 = sizeof(PrimalTmaSmem<SB, double, true>);
            staged_grid_[0][0] = wave(k_primal_tma<float, SB, false, true>, s32);
            staged_grid_[0][1] = wave(k_primal_tma<float, SB, true, true>, s32);
            staged_grid_[1][0] = wave(k_primal_tma<double, SB, false, true>, s64);
            staged_grid_[1][1] = wave(k_primal_tma<double, SB, true, true>, s64);
        } else {
            constexpr size_t s32 = sizeof(PrimalTmaSmem<SB, float, false>),
                             s64 = sizeof(PrimalTmaSmem<SB, double, false>);
            staged_grid_[0][0] = wave(k_primal_tma<float, SB, false, false>, s32);
            staged_grid_[0][1] = wave(k_primal_tma<float, SB, true, false>, s32);
            staged_grid_[1][0] = wave(k_primal_tma<double, SB, false, false>, s64);
            staged_grid_[1][1] = wave(k_primal_tma<double, SB, true, false>, s64);
        }
    });
}

/* The persistent loop runs small LPs (row blocks of at most 1,024 nonzeros)
 * on the default iteration path: no column panels, staged or hot-row primal
 * product, restart target selection, infeasibility rays or per-launch
 * timing, all of which the graph path carries.  Its grid is what the device
 * holds at once (a cooperative launch), capped by the work. */
#define PDAL_WITH_S_LOOP(Sval, ...)                   \
    switch (Sval) {                                   \
    case 256: {                                       \
        constexpr int SL = 256;                       \
        __VA_ARGS__;                                  \
    } break;                                          \
    case 512: {                                       \
        constexpr int SL = 512;                       \
        __VA_ARGS__;                                  \
    } break;                                          \
    case 1024: {                                      \
        constexpr int SL = 1024;                      \
        __VA_ARGS__;                                  \
    } break;                                          \
    default:                                          \
        throw Error("persistent loop: unsupported row-block budget"); \
    }

void CpalSolver::setup_loop() {
    const bool eligible = S_it_ <= 1024 && S_ev_ == S_it_ && !use_panels_ && !use_hot_ && !use_staged_ &&
                          cp_.restart_select == 0 && !cp_.infeas && O_.timing == 0 && !cp_.pulse && !cp_.trigger &&
                          !cp_.dyn;
    const bool want = O_.persistent_loop == 1;
    use_loop_ = eligible && want;
    if (!use_loop_) return;
    int dev = 0, sms = 0, coop = 0;
    PDAL_CUDA(cudaGetDevice(&dev));
    PDAL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PDAL_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) {
        use_loop_ = false;
        return;
    }
    const long long work = std::max({(long long)At_.it.hp.nblocks, (long long)A_.it.hp.nblocks,
                                     (long long)At_.ev.hp.nblocks, (long long)A_.ev.hp.nblocks,
                                     ((long long)std::max(n_, m_) + kThreads - 1) / kThreads, 1LL});
    auto wave = [&](auto kernel) {
        int occ = 0;
        PDAL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kThreads, 0));
        if (occ < 1) throw Error("persistent loop does not fit on one SM");
        return (int)std::min<long long>((long long)occ * sms, work);
    };
    PDAL_WITH_S_LOOP(S_it_, {
        if (beta_on_) {
            loop_grid_[0] = wave(k_cpal_loop<float, SL, SL, true>);
            loop_grid_[1] = wave(k_cpal_loop<double, SL, SL, true>);
        } else {
            loop_grid_[0] = wave(k_cpal_loop<float, SL, SL, false>);
            loop_grid_[1] = wave(k_cpal_loop<double, SL, SL, false>);
        }
    });
    PDAL_CUDA(cudaMemsetAsync(loop_bar_, 0, sizeof(LoopBar), stream_));
}

/* A device wait that ran out (a staging wait of k_primal_tma, a grid
 * barrier of k_cpal_loop) stops the solve (status kStatusDeviceError) and is
 * reported here as an error. */
void CpalSolver::check_device_error() {
    if (!dev_err_) return;
    int e = 0;
    PDAL_CUDA(cudaMemcpyAsync(&e, dev_err_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    if (e == 1) throw Error("a staged copy of the primal product did not complete in time; the solve was stopped");
    if (e) throw Error("a grid barrier of the persistent loop did not complete in time; the solve was stopped");
}

void CpalSolver::upload() {
    const double t_up = now_sec();
    if (O_.device >= 0) PDAL_CUDA(cudaSetDevice(O_.device));
    PDAL_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    PDAL_CUDA(cudaMallocHost(&h_st_, sizeof(CpalState)));
    PDAL_CUDA(cudaMallocHost(&h_ps_, sizeof(PowerState)));
    A_.nr = m_;
    A_.nc = n_;
    A_.nnz = nnz_;
    At_.nr = n_;
    At_.nc = m_;
    At_.nnz = nnz_;
    A_.it.hp = plan_rows(m_, prob_->constraint_matrix_row_pointers, S_it_);
    At_.it.hp = plan_rows(n_, At_host_.rp.data(), S_it_);
    A_.ev.hp = plan_rows(m_, prob_->constraint_matrix_row_pointers, S_ev_);
    At_.ev.hp = plan_rows(n_, At_host_.rp.data(), S_ev_);
    use_panels_ = false;
    use_hot_ = false;
    if (m_ > 0 && O_.dual_panels != 0 && A_.it.hp.nlong > 0) {
        const int *rp = prob_->constraint_matrix_row_pointers;
        long long long_nnz = 0;
        for (int q = 0; q < A_.it.hp.nlong; ++q) {
            const int r = A_.it.hp.linfo[4 * q];
            long_nnz += rp[r + 1] - rp[r];
        }
        if (O_.dual_panels == 1 || long_nnz >= (1ll << 20)) {
            const int W = O_.panel_width > 0 ? O_.panel_width : 16384;
            /* the FP64 phase stages W doubles per block */
            if (W % 4 != 0 || W > 65536 || panel_smem_bytes<double>(W) > 227 * 1024)
                throw Error("panel_width must be a multiple of 4 whose FP64 panel fits in shared memory "
                            "(at most 29,056)");
            /* one wave of two panel blocks per SM (64 KB of FP32 x-bar each) */
            pan_host_ = plan_panels(m_, n_, rp, prob_->constraint_matrix_col_indices, S_it_, W, 2 * 152);
            sh_r1_h.clear();
            sh_p1_h.clear();
            sh_c1_h.clear();
            sh_r2_h.clear();
            sh_r3_h.clear();
            const int *cip = prob_->constraint_matrix_col_indices;
            {
                size_t n1 = 0, n2 = 0, n3 = 0;
                for (int r = 0; r < m_; ++r) {
                    const int len = rp[r + 1] - rp[r];
                    n1 += len <= 1;
                    n2 += len > 1 && len <= kShortMidLen;
                    n3 += len > kShortMidLen && len <= S_it_;
                }
                sh_r1_h.reserve(n1);
                sh_p1_h.reserve(n1);
                sh_c1_h.reserve(n1);
                sh_r2_h.reserve(n2);
                sh_r3_h.reserve(n3);
            }
            for (int r = 0; r < m_; ++r) {
                const int len = rp[r + 1] - rp[r];
                if (len <= 1) {
                    sh_r1_h.push_back(r);
                    sh_p1_h.push_back(len ? rp[r] : -1);
                    sh_c1_h.push_back(len ? cip[rp[r]] : 0);
                } else if (len <= kShortMidLen) {
                    sh_r2_h.push_back(r);
                } else if (len <= S_it_) {
                    sh_r3_h.push_back(r);
                }
            }
            use_hot_ = O_.primal_hot_rows != 0 && pan_host_.H > 0 &&
                       pan_host_.H <= kHotRows;
            /* the warp rows longest first, so that the longest start in the
             * first round of the grid-stride loop (a counting sort by length:
             * rows of equal length keep their order) */
            {
                const int span = S_it_ - kShortMidLen; /* lengths kShortMidLen + 1 .. S_it_ */
                std::vector<int> at((size_t)span + 1, 0);
                for (int r : sh_r3_h) at[(size_t)(S_it_ - (rp[r + 1] - rp[r])) + 1]++;
                for (int q = 0; q < span; ++q) at[q + 1] += at[q];
                std::vector<int> sorted(sh_r3_h.size());
                for (int r : sh_r3_h) sorted[(size_t)at[(size_t)(S_it_ - (rp[r + 1] - rp[r]))]++] = r;
                sh_r3_h.swap(sorted);
            }
            /* a fixed number of blocks per part, each looping over its rows */
            auto blocks = [](long long rows, long long per_block, long long cap) {
                return (int)std::min<long long>((rows + per_block - 1) / per_block, cap);
            };
            sh_b1_ = blocks((long long)sh_r1_h.size(), kThreads * kShortUnroll, 152 * 3);
            sh_b2_ = blocks((long long)sh_r2_h.size(), kThreads / 8, 152 * 1);
            sh_b3_ = blocks((long long)sh_r3_h.size(), kThreads / 32, 152 * 2);
            use_panels_ = pan_host_.H > 0;
            fuse_finish_ = O_.dual_fused_finish == 1;
            /* measured: the FP64 dual step 0.212 -> 0.200 ms, the FP32 one no faster */
            dual_fork_ = use_panels_ && !fuse_finish_ && O_.dual_concurrent != 0;
            dual_fork32_ = dual_fork_ && O_.dual_concurrent == 1;
            if (dual_fork_ && !side_) {
                PDAL_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
                PDAL_CUDA(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
                PDAL_CUDA(cudaEventCreateWithFlags(&join_ev_, cudaEventDisableTiming));
            }
        }
    }
    {
        auto longs = [](int nr, const int *rp, std::vector<int> &out) {
            out.clear();
            for (int r = 0; r < nr; ++r)
                if (rp[r + 1] - rp[r] > kEqShort) out.push_back(r);
        };
        longs(m_, prob_->constraint_matrix_row_pointers, eq_long_h_[0]);
        longs(n_, At_host_.rp.data(), eq_long_h_[1]);
    }
    const double t_alloc = now_sec();
    upload_plan_sec = t_alloc - t_up;
    arena_.begin_measure();
    alloc_all();
    arena_.reserve_measured();
    alloc_all();
    upload_alloc_sec = now_sec() - t_alloc;
    PDAL_CUDA(cudaMemsetAsync(dev_err_, 0, sizeof(int), stream_));
    for (int q = 0; q < 2; ++q)
        if (!eq_long_h_[q].empty())
            PDAL_CUDA(cudaMemcpyAsync(eq_long_[q], eq_long_h_[q].data(), eq_long_h_[q].size() * sizeof(int),
                                      cudaMemcpyHostToDevice, stream_));
    setup_staged();

    const size_t n = n_, m = m_, nnz = nnz_;
    auto up = [&](void *dst, const void *src, size_t b) {
        if (b == 0) return;
        PDAL_CUDA(cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, stream_));
        h2d += (int64_t)b;
    };
    up(A_.rp, prob_->constraint_matrix_row_pointers, (m + 1) * sizeof(int));
    up(A_.ci, prob_->constraint_matrix_col_indices, nnz * sizeof(int));
    up(Av0_, prob_->constraint_matrix_values, nnz * sizeof(double));
    up(At_.rp, At_host_.rp.data(), (n + 1) * sizeof(int));
    if (device_transpose_) {
        PDAL_CUDA(cudaMemcpyAsync(at_cursor_, At_.rp, (n + 1) * sizeof(int), cudaMemcpyDeviceToDevice, stream_));
        const int nla = (int)eq_long_h_[0].size(), nlt = (int)eq_long_h_[1].size();
        if (m > 0)
            k_transpose_scatter<<<grid_for(std::max<long long>(m, 32LL * nla)), kThreads, 0, stream_>>>(
                m_, A_.rp, A_.ci, Av0_, at_cursor_, At_.ci, Atv0_, eq_long_[0], nla);
        k_transpose_sort_short<<<grid_for(n), kThreads, 0, stream_>>>(n_, At_.rp, At_.ci, Atv0_);
        if (nlt > 0)
            k_transpose_sort_long<<<std::min(nlt, 152 * 4), kThreads, 0, stream_>>>(At_.rp, At_.ci, Atv0_, eq_long_[1],
                                                                                 nlt);
        PDAL_LAUNCH_CHECK();
    } else {
        up(At_.ci, At_host_.ci.data(), nnz * sizeof(int));
        up(Atv0_, At_host_.v.data(), nnz * sizeof(double));
    }
    upload_plan(A_.it);
    upload_plan(At_.it);
    upload_plan(A_.ev);
    upload_plan(At_.ev);
    if (use_panels_) {
        const size_t len = (size_t)pan_host_.len, hp = (size_t)pan_host_.H * pan_host_.P;
        up(sh_r1_, sh_r1_h.data(), sh_r1_h.size() * sizeof(int));
        up(sh_p1_, sh_p1_h.data(), sh_p1_h.size() * sizeof(int));
        up(sh_c1_, sh_c1_h.data(), sh_c1_h.size() * sizeof(int));
        up(sh_r2_, sh_r2_h.data(), sh_r2_h.size() * sizeof(int));
        up(sh_r3_, sh_r3_h.data(), sh_r3_h.size() * sizeof(int));
        if (use_hot_) {
            std::vector<int> hot_id(m, -1);
            for (int h = 0; h < pan_host_.H; ++h) hot_id[pan_host_.rows[h]] = h;
            if (device_transpose_) {
                up(hot_id_d_, hot_id.data(), m * sizeof(int));
                k_hot_indices<<<grid_for((long long)nnz), kThreads, 0, stream_>>>((long long)nnz, At_.ci, hot_id_d_,
                                                                                 At_ci_hot_);
                PDAL_LAUNCH_CHECK();
            } else {
                std::vector<int> cih(At_host_.ci.size());
                const int nt = host_threads((long long)cih.size());
                parallel_for(nt, [&](int t) {
                    const size_t k0 = cih.size() * t / nt, k1 = cih.size() * (t + 1) / nt;
                    for (size_t k = k0; k < k1; ++k) {
                        const int r = At_host_.ci[k];
                        cih[k] = hot_id[r] >= 0 ? -1 - hot_id[r] : r;
                    }
                });
                up(At_ci_hot_, cih.data(), cih.size() * sizeof(int));
            }
            PDAL_CUDA(cudaStreamSynchronize(stream_)); /* hot_id / cih leave scope */
            int dev = 0, sms = 0;
            PDAL_CUDA(cudaGetDevice(&dev));
            PDAL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            auto wave = [&](auto kernel) {
                int occ = 0;
                PDAL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kThreads, 0));
                return std::max(1, std::min(At_.it.hp.nblocks, std::max(1, occ) * sms));
            };
            PDAL_WITH_S(S_it_, {
                hot_grid_[0][0] = wave(k_primal_hot<float, SB, false>);
                hot_grid_[0][1] = wave(k_primal_hot<float, SB, true>);
                hot_grid_[1][0] = wave(k_primal_hot<double, SB, false>);
                hot_grid_[1][1] = wave(k_primal_hot<double, SB, true>);
            });
        }
        up(pan_rows_, pan_host_.rows.data(), pan_host_.rows.size() * sizeof(int));
        up(pan_pmap_, pan_host_.pmap.data(), len * sizeof(int));
        up(pan_seg_, pan_host_.seg.data(), pan_host_.seg.size() * sizeof(int));
        up(pan_piece_, pan_host_.piece.data(), pan_host_.piece.size() * sizeof(int));
        up(pan_cta_, pan_host_.cta.data(), pan_host_.cta.size() * sizeof(int));
        up(pan_off_, pan_host_.off.data(), len * sizeof(uint16_t));
        /* (row, panel) pairs without a segment keep a zero partial */
        PDAL_CUDA(cudaMemsetAsync(pan_part64_, 0, hp * sizeof(double), stream_));
        {
            /* segments per long row: a row's last one finishes it */
            std::vector<int> nseg(std::max(pan_host_.H, 1), 0);
            for (size_t q = 0; q + 3 < pan_host_.seg.size(); q += 4) nseg[pan_host_.seg[q]]++;
            up(pan_nseg_, nseg.data(), nseg.size() * sizeof(int));
            PDAL_CUDA(cudaMemsetAsync(pan_cnt_, 0, nseg.size() * sizeof(unsigned), stream_));
            PDAL_CUDA(cudaStreamSynchronize(stream_)); /* nseg leaves scope */
        }
        if (pan_part32_) PDAL_CUDA(cudaMemsetAsync(pan_part32_, 0, hp * sizeof(float), stream_));
    }
    up(c0_, prob_->objective_vector, n * sizeof(double));
    up(vlb0_, prob_->variable_lower_bound, n * sizeof(double));
    up(vub0_, prob_->variable_upper_bound, n * sizeof(double));
    up(clb0_, prob_->constraint_lower_bound, m * sizeof(double));
    up(cub0_, prob_->constraint_upper_bound, m * sizeof(double));
    if (prob_->primal_start)
        up(x00_, prob_->primal_start, n * sizeof(double));
    else
        PDAL_CUDA(cudaMemsetAsync(x00_, 0, std::max<size_t>(n, 1) * sizeof(double), stream_));
    if (prob_->dual_start)
        up(y00_, prob_->dual_start, m * sizeof(double));
    else
        PDAL_CUDA(cudaMemsetAsync(y00_, 0, std::max<size_t>(m, 1) * sizeof(double), stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    At_host_ = HostCsr(); /* host transpose no longer needed */
    pan_host_.pmap = decltype(pan_host_.pmap)();
    pan_host_.off = decltype(pan_host_.off)();
    upload_sec = now_sec() - t_up;
}

/* A kernel launched with programmatic stream serialization (the iteration
 * and FP32 power kernels begin with pdl_enter): its launch is prepared while
 * the previous kernel finishes, which hides part of the launch latency that
 * bounds small problems (measured: 6,800 iterations of a 2,000 x 5,000 LP
 * 67.4 -> 62.3 ms).  Stream capture records the same programmatic edges. */
template <typename... KArgs, typename... Args>
static void launch_pdl_cfg(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t stream,
                           Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PDAL_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
}

template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kern)(KArgs...), int grid, cudaStream_t stream, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PDAL_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
}

void CpalSolver::power_iteration() {
    PowerState h{};
    h.max_iter = P_.sv_max_iter;
    h.tol = P_.sv_tol;
    h.done = (h.max_iter <= 0) ? 1 : 0;
    /* start vector: std::normal_distribution over std::mt19937(1), as the
     * reference draws it in a fresh process (LP/CP_AL/src/utils.cu:27-28, 102-106) */
    std::vector<double> v0(m_);
    std::mt19937 gen(1);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (int i = 0; i < m_; ++i) v0[i] = dist(gen);
    /* plain form: FP64 over the evaluation plans; chosen form: FP32 over the
     * iteration plans and the FP32 matrix copies (made before this call) */
    const bool f32 = fp32_phase_;
    if (f32) {
        std::vector<float> v0f(v0.begin(), v0.end());
        PDAL_CUDA(cudaMemcpyAsync(tmp_m_, v0f.data(), sizeof(float) * m_, cudaMemcpyHostToDevice, stream_));
        h2d += sizeof(float) * m_;
    } else {
        PDAL_CUDA(cudaMemcpyAsync(tmp_m_, v0.data(), sizeof(double) * m_, cudaMemcpyHostToDevice, stream_));
        h2d += sizeof(double) * m_;
    }
    *h_ps_ = h;
    PDAL_CUDA(cudaMemcpyAsync(ps_, h_ps_, sizeof(PowerState), cudaMemcpyHostToDevice, stream_));
    if (f32)
        k_power_start<float><<<1, kThreads, 0, stream_>>>(m_, (const float *)tmp_m_, ps_);
    else
        k_power_start<double><<<1, kThreads, 0, stream_>>>(m_, tmp_m_, ps_);
    PDAL_LAUNCH_CHECK();
    launches += 1;
    const int gres = grid_for(m_);
    const int steps_per_graph = 16;
    cudaGraphExec_t exec = nullptr;
    PDAL_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    for (int st = 0; st < steps_per_graph; ++st) {
        if (f32) {
            /* fused step: two products and one finishing block; v and vn
             * alternate between the two buffers (an even number of steps per
             * graph, so every launch starts from the first) */
            float *bufa = (float *)tmp_m_, *bufb = (float *)tmp_m2_, *dp = (float *)tmp_n_;
            float *v = (st % 2 == 0) ? bufa : bufb, *vn = (st % 2 == 0) ? bufb : bufa;
            const int *Arp = A_.rp, *Aci = A_.ci, *Atrp = At_.rp, *Atci = At_.ci;
            const float *Av = A_.vf, *Atv = At_.vf;
            const PowerState *psc = ps_;
            PDAL_WITH_S(S_it_, {
                launch_pdl(k_power_at<SB, float>, At_.it.d.nblocks, stream_, At_.it.d, Atrp, Atci, Atv,
                           (const float *)v, dp, psc);
                launch_pdl(k_power_a<SB, float, true>, A_.it.d.nblocks, stream_, A_.it.d, Arp, Aci, Av,
                           (const float *)dp, (const float *)v, vn, part_misc_, psc);
            });
            launch_pdl(k_power_fin, 1, stream_, (const double *)part_misc_, A_.it.d.nblocks + A_.it.d.nlong, ps_);
        } else {
            double *v = tmp_m_, *vn = tmp_m2_, *dp = tmp_n_;
            PDAL_WITH_SE(S_ev_, {
                k_power_at<SE, double><<<At_.ev.d.nblocks, kThreads, 0, stream_>>>(At_.ev.d, At_.rp, At_.ci, At_.v,
                                                                                   v, dp, ps_);
                k_power_a<SE, double><<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(A_.ev.d, A_.rp, A_.ci, A_.v, dp, v,
                                                                                 vn, part_misc_, ps_);
            });
            const int nparts = A_.ev.d.nblocks + A_.ev.d.nlong;
            k_power_dot<<<1, kThreads, 0, stream_>>>(part_misc_, nparts, ps_);
            k_power_resid<double><<<gres, kThreads, 0, stream_>>>(m_, v, vn, part_misc_, ps_);
            k_power_check<<<1, kThreads, 0, stream_>>>(part_misc_, gres, ps_);
        }
    }
    cudaGraph_t graph;
    PDAL_CUDA(cudaStreamEndCapture(stream_, &graph));
    PDAL_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    PDAL_CUDA(cudaGraphDestroy(graph));
    const int max_launch = P_.sv_max_iter / steps_per_graph + 2;
    for (int it = 0; it < max_launch; ++it) {
        PDAL_CUDA(cudaGraphLaunch(exec, stream_));
        launches += (f32 ? 3 : 5) * steps_per_graph;
        PDAL_CUDA(cudaMemcpyAsync(h_ps_, ps_, sizeof(PowerState), cudaMemcpyDeviceToHost, stream_));
        d2h += sizeof(PowerState);
        PDAL_CUDA(cudaStreamSynchronize(stream_));
        if (h_ps_->done) break;
    }
    cudaGraphExecDestroy(exec);
    power_iters = h_ps_->iters;
    const double smax = std::sqrt(h_ps_->s2);
    host_state.lambda_est = smax * smax;
}

/* sigma_max(A)^2 by Lanczos on A A^T with FP32 products (the chosen form;
 * k_lz_* in cpal_kernels.cuh): the power iteration's start vector, steps in
 * CUDA graphs of kLanczosChunk, and after each graph the largest Ritz value;
 * it stops when that value moves by less than 1e-8 relative over a chunk, at
 * an invariant subspace, or after min(kLanczosMax, sv_max_iter) steps. */
void CpalSolver::lanczos() {
    std::vector<double> v0(m_);
    std::mt19937 gen(1);
    std::normal_distribution<double> dist(0.0, 1.0);
    for (int i = 0; i < m_; ++i) v0[i] = dist(gen);
    PDAL_CUDA(cudaMemcpyAsync(tmp_m_, v0.data(), sizeof(double) * m_, cudaMemcpyHostToDevice, stream_));
    h2d += sizeof(double) * m_;
    PowerState h{};
    h.inv = 1.0; /* the product kernels scale their input by inv */
    h.max_iter = 1 << 30;
    *h_ps_ = h;
    PDAL_CUDA(cudaMemcpyAsync(ps_, h_ps_, sizeof(PowerState), cudaMemcpyHostToDevice, stream_));
    PDAL_CUDA(cudaMemsetAsync(lz_j_, 0, sizeof(int), stream_));
    /* FP32 buffers the iteration has not started to use */
    float *qf = v32_.ybar, *w = v32_.u, *dp = reinterpret_cast<float *>(tmp_n_);
    const LanczosDev lz{lz_alpha_, lz_beta_, lz_j_};
    k_lz_start<float><<<1, kThreads, 0, stream_>>>(m_, tmp_m_, qf, tmp_m2_);
    PDAL_LAUNCH_CHECK();
    launches += 1;
    const int gm = grid_for(m_);
    const int nparts = A_.it.d.nblocks + A_.it.d.nlong;
    cudaGraphExec_t exec = nullptr;
    PDAL_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    for (int st = 0; st < kLanczosChunk; ++st) {
        /* q_j and q_{j-1} alternate between the two FP64 buffers */
        double *q = (st % 2 == 0) ? tmp_m_ : tmp_m2_, *p = (st % 2 == 0) ? tmp_m2_ : tmp_m_;
        const int *Arp = A_.rp, *Aci = A_.ci, *Atrp = At_.rp, *Atci = At_.ci;
        const float *Av = A_.vf, *Atv = At_.vf;
        const PowerState *psc = ps_;
        PDAL_WITH_S(S_it_, {
            launch_pdl(k_power_at<SB, float>, At_.it.d.nblocks, stream_, At_.it.d, Atrp, Atci, Atv, (const float *)qf,
                       dp, psc);
            launch_pdl(k_power_a<SB, float, false>, A_.it.d.nblocks, stream_, A_.it.d, Arp, Aci, Av,
                       (const float *)dp, (const float *)qf, w, part_misc_, psc);
        });
        launch_pdl(k_lz_alpha, 1, stream_, (const double *)part_misc_, nparts, lz);
        launch_pdl(k_lz_update<float>, gm, stream_, m_, (const float *)w, (const double *)q, p, lz, part_misc_);
        launch_pdl(k_lz_beta, 1, stream_, (const double *)part_misc_, gm, lz);
        launch_pdl(k_lz_next<float>, gm, stream_, m_, p, qf, lz);
    }
    cudaGraph_t graph;
    PDAL_CUDA(cudaStreamEndCapture(stream_, &graph));
    PDAL_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    PDAL_CUDA(cudaGraphDestroy(graph));
    /* a multiple of the chunk, at most kLanczosMax: every step's slot exists */
    const int jmax = std::max(kLanczosChunk, std::min(kLanczosMax, std::max(P_.sv_max_iter, 1)));
    std::vector<double> a(kLanczosMax), b(kLanczosMax);
    double theta = 0.0, prev = -1.0;
    int steps = 0;
    for (;;) {
        PDAL_CUDA(cudaGraphLaunch(exec, stream_));
        launches += 6 * kLanczosChunk;
        steps += kLanczosChunk;
        PDAL_CUDA(cudaMemcpyAsync(a.data(), lz_alpha_, sizeof(double) * steps, cudaMemcpyDeviceToHost, stream_));
        PDAL_CUDA(cudaMemcpyAsync(b.data(), lz_beta_, sizeof(double) * steps, cudaMemcpyDeviceToHost, stream_));
        PDAL_CUDA(cudaStreamSynchronize(stream_));
        d2h += 2 * sizeof(double) * steps;
        /* an invariant subspace (zero beta): T up to that step holds the answer */
        int k = steps;
        for (int i = 0; i < steps; ++i)
            if (!(b[i] > 0.0)) {
                k = i + 1;
                break;
            }
        theta = tridiag_max_eig(a, b, k);
        const bool invariant = k < steps || b[k - 1] <= 1e-12 * std::max(theta, 1e-300);
        if (invariant || steps >= jmax || steps >= m_ || (prev > 0.0 && std::fabs(theta - prev) <= 1e-8 * theta))
            break;
        prev = theta;
    }
    cudaGraphExecDestroy(exec);
    power_iters = steps;
    host_state.lambda_est = theta;
}

void CpalSolver::setup_device() {
    const double t0 = now_sec();
    for (auto &r : sum_ms)
        for (auto &x : r) x = 0;
    for (auto &r : sub_ms)
        for (auto &x : r) x = 0;
    timed[0] = timed[1] = 0;
    launches = 0;
    fp32_iters = 0;
    fp32_phase_ = O_.precision == CP_AL_GB300_FP32_REFINE;
    const size_t n = n_, m = m_, nnz = nnz_;
    auto d2d = [&](void *dst, const void *src, size_t b) {
        if (b) PDAL_CUDA(cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToDevice, stream_));
    };
    d2d(A_.v, Av0_, nnz * sizeof(double));
    d2d(At_.v, Atv0_, nnz * sizeof(double));
    d2d(c_, c0_, n * sizeof(double));
    d2d(vlb_, vlb0_, n * sizeof(double));
    d2d(vub_, vub0_, n * sizeof(double));
    d2d(x0_, x00_, n * sizeof(double));
    d2d(clb_, clb0_, m * sizeof(double));
    d2d(cub_, cub0_, m * sizeof(double));
    d2d(y0_, y00_, m * sizeof(double));

    /* equilibration: LP/CP_AL/src/preconditioner.cu:379-475 */
    const int gn = grid_for(n), gm = grid_for(m);
    const int gwr_m = grid_for((long long)m * 32), gwr_n = grid_for((long long)n * 32);
    std::vector<double> ones_n(n, 1.0), ones_m(m, 1.0);
    PDAL_CUDA(cudaMemcpyAsync(dsc_, ones_n.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream_));
    if (m) PDAL_CUDA(cudaMemcpyAsync(rsc_, ones_m.data(), m * sizeof(double), cudaMemcpyHostToDevice, stream_));
    double *rstep = tmp_m_, *dstep = tmp_n_;
    /* reciprocal scales: an m- and an n-sized buffer the iteration has not
     * started to use (x_bar is cleared before the first iteration) */
    double *rinv = tmp_m2_, *dinv = v64_.xbar;
    const int nla = (int)eq_long_h_[0].size(), nlt = (int)eq_long_h_[1].size();
    const int geq_m = grid_for(std::max<long long>(m, 32LL * nla)), geq_n = grid_for(std::max<long long>(n, 32LL * nlt));
    auto scale_pass = [&](int mode, double deg_rows, double deg_cols) {
        if (m)
            k_row_scale<<<geq_m, kThreads, 0, stream_>>>(m_, A_.rp, A_.v, mode, deg_rows, rstep, rsc_, rinv, eq_long_[0],
                                                         nla);
        k_row_scale<<<geq_n, kThreads, 0, stream_>>>(n_, At_.rp, At_.v, mode, deg_cols, dstep, dsc_, dinv, eq_long_[1],
                                                     nlt);
        if (m) k_scale_matrix<<<geq_m, kThreads, 0, stream_>>>(m_, A_.rp, A_.ci, A_.v, rinv, dinv, 0, eq_long_[0], nla);
        k_scale_matrix<<<geq_n, kThreads, 0, stream_>>>(n_, At_.rp, At_.ci, At_.v, dinv, rinv, 1, eq_long_[1], nlt);
        k_scale_vectors<<<grid_for(std::max(n, m)), kThreads, 0, stream_>>>(n_, m_, dstep, rstep, c_, vlb_, vub_, x0_,
                                                                            clb_, cub_, y0_);
        PDAL_LAUNCH_CHECK();
        launches += 5;
    };
    /* Curtis-Reid before Ruiz (LP/CP_AL/src/preconditioner.cu:162-270,
     * 403-425): alternating row / column log-mean passes, then the scales
     * exp(log) clamped to [1e-30, 1e30] applied like a Ruiz pass; with early
     * stop (20 passes) the passes end after the fifth when no scaled entry's
     * log moved by more than the threshold */
    cr_passes = 0;
    if (O_.cr_iterations > 0) {
        double *lr = rstep, *lc = dstep, *dr = v64_.ybar, *dc = v64_.lam;
        if (m) PDAL_CUDA(cudaMemsetAsync(lr, 0, m * sizeof(double), stream_));
        PDAL_CUDA(cudaMemsetAsync(lc, 0, n * sizeof(double), stream_));
        const bool early = O_.cr_early_stop != 0 && O_.cr_iterations == 20;
        for (int it = 0; it < O_.cr_iterations; ++it) {
            if (m) k_cr_log_update<<<gwr_m, kThreads, 0, stream_>>>(m_, A_.rp, A_.ci, A_.v, lc, lr, early ? dr : nullptr);
            k_cr_log_update<<<gwr_n, kThreads, 0, stream_>>>(n_, At_.rp, At_.ci, At_.v, lr, lc, early ? dc : nullptr);
            PDAL_LAUNCH_CHECK();
            launches += 2;
            cr_passes = it + 1;
            if (early && it + 1 == 5) {
                /* a maximum over no rows is the lowest double: below any threshold */
                if (!m) break;
                const int ge = std::max(1, std::min(gwr_m, nmisc_));
                k_cr_edge_change<<<ge, kThreads, 0, stream_>>>(m_, A_.rp, A_.ci, dr, dc, part_misc_);
                PDAL_LAUNCH_CHECK();
                launches += 1;
                std::vector<double> part(ge);
                PDAL_CUDA(cudaMemcpyAsync(part.data(), part_misc_, ge * sizeof(double), cudaMemcpyDeviceToHost, stream_));
                PDAL_CUDA(cudaStreamSynchronize(stream_));
                d2h += ge * sizeof(double);
                double mx = 0.0;
                for (double v : part) mx = std::max(mx, v);
                if (mx <= O_.cr_early_stop_threshold) break;
            }
        }
        cp_.cr_early_stopped = early && cr_passes < O_.cr_iterations; /* preconditioner.cu:246 */
        if (m) k_cr_exp<<<gm, kThreads, 0, stream_>>>(m_, lr, rinv, rsc_);
        k_cr_exp<<<gn, kThreads, 0, stream_>>>(n_, lc, dinv, dsc_);
        if (m)
            k_scale_matrix<<<geq_m, kThreads, 0, stream_>>>(m_, A_.rp, A_.ci, A_.v, rinv, dinv, 0, eq_long_[0], nla);
        k_scale_matrix<<<geq_n, kThreads, 0, stream_>>>(n_, At_.rp, At_.ci, At_.v, dinv, rinv, 1, eq_long_[1], nlt);
        k_scale_vectors_inv<<<grid_for(std::max(n, m)), kThreads, 0, stream_>>>(n_, m_, lc, dinv, lr, rinv, c_, vlb_,
                                                                                vub_, x0_, clb_, cub_, y0_);
        PDAL_LAUNCH_CHECK();
        launches += 5;
    }
    for (int it = 0; it < P_.l_inf_ruiz_iterations; ++it) scale_pass(0, 0.0, 0.0);
    if (P_.has_pock_chambolle_alpha) scale_pass(1, P_.pock_chambolle_alpha, 2.0 - P_.pock_chambolle_alpha);
    const int gb = grid_for(std::max(n, m));
    k_boundobj_partials<<<gb, kThreads, 0, stream_>>>(n_, m_, clb_, cub_, c_, part_misc_);
    k_boundobj_finish<<<1, kThreads, 0, stream_>>>(part_misc_, gb, st_, P_.bound_objective_rescaling ? 1 : 0);
    if (P_.bound_objective_rescaling)
        k_scale_boundobj<<<gb, kThreads, 0, stream_>>>(n_, m_, st_, c_, vlb_, vub_, x0_, clb_, cub_, y0_);
    if (m) k_finite_bounds<<<gm, kThreads, 0, stream_>>>(m_, clb_, cub_, clbf_, cubf_);
    PDAL_LAUNCH_CHECK();
    launches += 4;
    (void)gn;
    /* cbr / ovr back to the host state */
    PDAL_CUDA(cudaMemcpyAsync(h_st_, st_, sizeof(CpalState), cudaMemcpyDeviceToHost, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    d2h += sizeof(CpalState);
    CpalState s{};
    s.cbr = h_st_->cbr;
    s.ovr = h_st_->ovr;
    equil_sec = now_sec() - t0;
    const double t_pow = now_sec();

    /* FP32 matrix copies of the equilibrated values (chosen form), which the
     * power iteration already uses */
    if (fp32_phase_) {
        if (nnz) k_convert<double, float><<<grid_for(nnz), kThreads, 0, stream_>>>(A_.v, A_.vf, (int)nnz);
        if (nnz) k_convert<double, float><<<grid_for(nnz), kThreads, 0, stream_>>>(At_.v, At_.vf, (int)nnz);
        PDAL_LAUNCH_CHECK();
        launches += 2;
    }
    /* the long rows' values in panel order, in each precision the
     * iteration runs in */
    if (use_panels_) {
        const long long len = pan_host_.len;
        k_panel_gather<double><<<grid_for(len), kThreads, 0, stream_>>>(pan_pmap_, A_.v, pan_v64_, len);
        if (fp32_phase_) k_panel_gather<float><<<grid_for(len), kThreads, 0, stream_>>>(pan_pmap_, A_.v, pan_v32_, len);
        const long long n1 = (long long)sh_r1_h.size();
        if (n1) {
            k_panel_gather<double><<<grid_for(n1), kThreads, 0, stream_>>>(sh_p1_, A_.v, sh_v64_, n1);
            if (fp32_phase_) k_panel_gather<float><<<grid_for(n1), kThreads, 0, stream_>>>(sh_p1_, A_.v, sh_v32_, n1);
        }
        {
            const int s64 = (int)panel_smem_bytes<double>(pan_host_.W), s32 = (int)panel_smem_bytes<float>(pan_host_.W);
            auto attr = [](auto kernel, int bytes) {
                PDAL_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
            };
            attr(k_dual_panels<double, false, false, false>, s64);
            attr(k_dual_panels<double, true, false, false>, s64);
            attr(k_dual_panels<double, true, false, true>, s64);
            attr(k_dual_panels<double, true, true, false>, s64);
            attr(k_dual_panels<double, true, true, true>, s64);
            attr(k_dual_panels<float, false, false, false>, s32);
            attr(k_dual_panels<float, true, false, false>, s32);
            attr(k_dual_panels<float, true, false, true>, s32);
            attr(k_dual_panels<float, true, true, false>, s32);
            attr(k_dual_panels<float, true, true, true>, s32);
        }
        PDAL_LAUNCH_CHECK();
        launches += fp32_phase_ ? 2 : 1;
    }
    /* step size and primal weight: LP/CP_AL/src/solver.cu:3538-3609 */
    if (nnz_ == 0) {
        host_state.lambda_est = 1.0;
        power_iters = 0;
    } else if (use_lanczos()) {
        lanczos();
    } else {
        power_iteration();
    }
    s.lambda_est = host_state.lambda_est;
    power_sec = now_sec() - t_pow;
    s.pw = P_.bound_objective_rescaling ? 1.0 : (cp_.obj_norm + 1.0) / (cp_.bnd_norm + 1.0);
    s.sigma_on = cp_.sigma_mode;
    s.sigma_adapt = 0;
    if (s.sigma_on) { /* solver.cu:3141-3164 */
        s.lambda_param = O_.lambda_param_set ? O_.lambda_param : O_.lambda_factor * std::fmax(s.lambda_est, 1e-12);
        s.lambda_param = std::fmax(s.lambda_param, (2.0 + 1e-12) * std::fmax(s.lambda_est, 1e-12));
        s.sigma_base = 1.0 / std::sqrt(std::fmax(s.lambda_param, 1e-16));
        s.sigma_min = O_.sigma_min_factor * s.sigma_base;
        s.sigma_max = O_.sigma_max_factor * s.sigma_base;
        s.sigma = O_.sigma_set ? O_.sigma : O_.sigma_init_factor * s.sigma_base;
        s.sigma = std::fmin(std::fmax(s.sigma, s.sigma_min), s.sigma_max);
        s.sigma_best = s.sigma;
        s.sigma_adapt = O_.sigma_adaptive != 0;
    }
    s.al_lambda = O_.al_lambda;
    cpal_refresh_step_schedule(s, cp_);
    s.best_pw = s.pw;
    s.best_gap = INFINITY;
    s.fp_last = INFINITY;
    s.refl = cp_.refl;
    s.fp32_switch_tol = fp32_phase_ ? O_.fp32_switch_tol : -1.0;
    s.fp32_stall_limit = O_.fp32_stall_evals;
    s.fp32_best_kkt = INFINITY;
    s.iter_limit = cp_.iteration_limit;
    /* the dynamic evaluation frequency's bootstrap starts with short blocks
     * (LP/CP_AL/src/solver.cu:1265-1268) */
    s.F = (cp_.dyn && cp_.dyn_boot > 0) ? cp_.dyn_fast : cp_.F;
    cpal_set_coefficients(s);
    beta_on_ = s.beta > 0.0;
    if (cp_.pulse) {
        /* LP/CP_AL/src/solver.cu:893-900 */
        fprintf(stderr,
                "[alpha-direct-pulse-config] enabled=1 alpha=2.000000000000e-03 pulse_iterations=200 "
                "history_epochs=2 deterministic_anchor_iter_ge=10000 wall_time_features=0 tail_only=1 "
                "force_pulse=%d\n",
                cp_.pulse_force);
        fflush(stderr);
    }
    host_state = s;
    *h_st_ = s;
    PDAL_CUDA(cudaMemcpyAsync(st_, h_st_, sizeof(CpalState), cudaMemcpyHostToDevice, stream_));
    h2d += sizeof(CpalState);
    k_fill_weights<<<1, kThreads, 0, stream_>>>(st_, wt_, wtf_, cp_.F);
    launches += 1;

    /* iterates start at the (scaled) warm start: solver.cu:1939-1974 */
    d2d(v64_.x, x0_, n * sizeof(double));
    d2d(v64_.xh, x0_, n * sizeof(double));
    d2d(v64_.y, y0_, m * sizeof(double));
    d2d(v64_.yh, y0_, m * sizeof(double));
    if (n) PDAL_CUDA(cudaMemsetAsync(v64_.lam, 0, n * sizeof(double), stream_));
    if (n) PDAL_CUDA(cudaMemsetAsync(v64_.xbar, 0, n * sizeof(double), stream_));
    if (m) PDAL_CUDA(cudaMemsetAsync(v64_.ybar, 0, m * sizeof(double), stream_));
    if (m) PDAL_CUDA(cudaMemsetAsync(v64_.u, 0, m * sizeof(double), stream_));
    if (fp32_phase_) {
        auto cv = [&](const double *src, float *dst, size_t len) {
            if (len) k_convert<double, float><<<grid_for(len), kThreads, 0, stream_>>>(src, dst, (int)len);
            launches += 1;
        };
        cv(c_, v32_.c, n);
        cv(vlb_, v32_.vlb, n);
        cv(vub_, v32_.vub, n);
        cv(x0_, v32_.x, n);
        cv(x0_, v32_.xh, n);
        cv(clb_, v32_.clb, m);
        cv(cub_, v32_.cub, m);
        cv(y0_, v32_.y, m);
        cv(y0_, v32_.yh, m);
        if (n) PDAL_CUDA(cudaMemsetAsync(v32_.lam, 0, n * sizeof(float), stream_));
        if (n) PDAL_CUDA(cudaMemsetAsync(v32_.xbar, 0, n * sizeof(float), stream_));
        if (m) PDAL_CUDA(cudaMemsetAsync(v32_.ybar, 0, m * sizeof(float), stream_));
        if (m) PDAL_CUDA(cudaMemsetAsync(v32_.u, 0, m * sizeof(float), stream_));
        if (n) k_split<<<grid_for(n), kThreads, 0, stream_>>>(x0_, x0f_, n_);
        if (m) k_split<<<grid_for(m), kThreads, 0, stream_>>>(y0_, y0f_, m_);
        launches += 2;
        PDAL_LAUNCH_CHECK();
        launch_init_ax<float>();
    } else {
        launch_init_ax<double>();
    }
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    setup_sec = now_sec() - t0;
}

template <typename T>
void CpalSolver::launch_init_ax() {
    if (m_ == 0) return;
    auto &v = vecs<T>();
    PDAL_WITH_SE(S_ev_, {
        float2 *axf = std::is_same<T, float>::value ? ax0f_ : nullptr;
        if (beta_on_)
            k_init_ax<T, SE, true><<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(
                A_.ev.d, A_.rp, A_.ci, A_.v, x0_, v.ax, ax0_, axf, v.u, v.y, v.clb, v.cub, st_);
        else
            k_init_ax<T, SE, false><<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(
                A_.ev.d, A_.rp, A_.ci, A_.v, x0_, v.ax, ax0_, axf, v.u, v.y, v.clb, v.cub, st_);
    });
    PDAL_LAUNCH_CHECK();
    launches += 1;
}

template <typename T>
static const T *matvals(const double *v64, const float *v32);
template <>
const double *matvals<double>(const double *v64, const float *) {
    return v64;
}
template <>
const float *matvals<float>(const double *, const float *v32) {
    return v32;
}

template <typename T>
static const typename AnchorT<T>::type *anchor(const double *a64, const float2 *a32);
template <>
const double *anchor<double>(const double *a64, const float2 *) {
    return a64;
}
template <>
const float2 *anchor<float>(const double *, const float2 *a32) {
    return a32;
}
template <typename T>
static const typename WeightT<T>::type *weights(const HalpernW *w64, const HalpernWf *w32);
template <>
const HalpernW *weights<double>(const HalpernW *w64, const HalpernWf *) {
    return w64;
}
template <>
const HalpernWf *weights<float>(const HalpernW *, const HalpernWf *w32) {
    return w32;
}

template <typename T>
void CpalSolver::launch_loop(int max_blocks) {
    auto &v = vecs<T>();
    LoopArgs<T> L{};
    L.at_it = At_.it.d;
    L.a_it = A_.it.d;
    L.at_ev = At_.ev.d;
    L.a_ev = A_.ev.d;
    if (m_ == 0) {
        L.a_it.nblocks = 0;
        L.a_ev.nblocks = 0;
    }
    L.at_rp = At_.rp;
    L.at_ci = At_.ci;
    L.a_rp = A_.rp;
    L.a_ci = A_.ci;
    L.at_val = matvals<T>(At_.v, At_.vf);
    L.a_val = matvals<T>(A_.v, A_.vf);
    L.at_v64 = At_.v;
    L.a_v64 = A_.v;
    L.pa = PrimalArgs<T>{v.x, v.xbar, v.xh, v.lam, anchor<T>(x0_, x0f_), v.c, v.vlb, v.vub};
    L.da = DualArgs<T>{v.y, v.yh, v.ybar, v.ax, v.u, anchor<T>(y0_, y0f_), anchor<T>(ax0_, ax0f_), v.clb, v.cub};
    L.gat = beta_on_ ? v.u : v.y;
    L.ra = EvalRowArgs<T>{v.xh, v.xbar, v.yh, v.ybar, x0_, y0_, ax0_, clb_, cub_, clbf_, cubf_, rsc_, phat_, part_row_,
                          A_.ev.d.nblocks, v.x, v.y, v.ax};
    L.ca = EvalColArgs<T>{v.xh, v.xbar, v.yh, v.ybar, v.lam, x0_, c_, dsc_, part_col_, At_.ev.d.nblocks, v.x, v.y, y0_};
    L.st = st_;
    L.p = cp_;
    L.wt = wt_;
    L.wtf = wtf_;
    L.nrow_slots = m_ > 0 ? A_.ev.d.nblocks + A_.ev.d.nlong : 0;
    L.ncol_slots = At_.ev.d.nblocks + At_.ev.d.nlong;
    L.n = n_;
    L.m = m_;
    const bool f32 = std::is_same<T, float>::value;
    L.x0 = x0_;
    L.y0 = y0_;
    L.ax0 = ax0_;
    L.x0f = f32 ? x0f_ : nullptr;
    L.y0f = f32 ? y0f_ : nullptr;
    L.ax0f = f32 ? ax0f_ : nullptr;
    L.phat = phat_;
    L.bar = loop_bar_;
    L.spin_limit = 1LL << 22; /* polls of an L2 round trip each: a barrier wait gives up after about 2 s */
    L.max_blocks = max_blocks;
    L.err = dev_err_;
    void *args[] = {(void *)&L};
    const int grid = loop_grid_[f32 ? 0 : 1];
    /* the barrier counter counts up from zero within a launch */
    PDAL_CUDA(cudaMemsetAsync(loop_bar_, 0, sizeof(LoopBar), stream_));
    PDAL_WITH_S_LOOP(S_it_, {
        const void *kern = beta_on_ ? (const void *)k_cpal_loop<T, SL, SL, true> : (const void *)k_cpal_loop<T, SL, SL, false>;
        PDAL_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(kThreads), args, 0, stream_));
    });
    launches += 1;
}

template <typename T>
void CpalSolver::launch_primal(int koff, bool major) {
    auto &v = vecs<T>();
    PrimalArgs<T> pa{v.x, v.xbar, v.xh, v.lam, anchor<T>(x0_, x0f_), v.c, v.vlb, v.vub};
    const T *gat = beta_on_ ? v.u : v.y;
    const T *Atv = matvals<T>(At_.v, At_.vf);
    const auto *wt = weights<T>(wt_, wtf_);
    if (hot_in<T>()) {
        T *hot = hot_ptr<T>();
        const int nh = pan_host_.H;
        /* the compact copy is rebuilt at the start of every block */
        if (koff == 1) launch_pdl(k_hot_refresh<T>, grid_for(nh), stream_, nh, (const int *)pan_rows_, gat, hot,
                                  (const CpalState *)st_);
        PDAL_WITH_S(S_it_, {
            const int *grid = hot_grid_[std::is_same<T, double>::value ? 1 : 0];
            if (major)
                launch_pdl(k_primal_hot<T, SB, true>, grid[1], stream_, At_.it.d, (const int *)At_.rp,
                           (const int *)At_ci_hot_, Atv, gat, (const T *)hot, nh, pa, (const CpalState *)st_, wt,
                           koff);
            else
                launch_pdl(k_primal_hot<T, SB, false>, grid[0], stream_, At_.it.d, (const int *)At_.rp,
                           (const int *)At_ci_hot_, Atv, gat, (const T *)hot, nh, pa, (const CpalState *)st_, wt,
                           koff);
        });
        return;
    }
    if (use_staged_) {
        PDAL_WITH_S(S_it_, {
            const int *grid = staged_grid_[std::is_same<T, double>::value ? 1 : 0];
            auto go = [&](auto kernel, size_t smem, int g) {
                launch_pdl_cfg(kernel, g, kThreads, smem, stream_, At_.it.d, (const int *)At_.rp,
                               (const int *)At_.ci, Atv, gat, pa, st_, wt, koff, dev_err_);
            };
            if (staged_rows()) {
                const size_t smem = sizeof(PrimalTmaSmem<SB, T, true>);
                if (major)
                    go(k_primal_tma<T, SB, true, true>, smem, grid[1]);
                else
                    go(k_primal_tma<T, SB, false, true>, smem, grid[0]);
            } else {
                const size_t smem = sizeof(PrimalTmaSmem<SB, T, false>);
                if (major)
                    go(k_primal_tma<T, SB, true, false>, smem, grid[1]);
                else
                    go(k_primal_tma<T, SB, false, false>, smem, grid[0]);
            }
        });
        return;
    }
    PDAL_WITH_S(S_it_, {
        if (major)
            launch_pdl(k_primal<T, SB, true>, At_.it.d.nblocks, stream_, At_.it.d, (const int *)At_.rp,
                       (const int *)At_.ci, Atv, gat, pa, (const CpalState *)st_, wt, koff);
        else
            launch_pdl(k_primal<T, SB, false>, At_.it.d.nblocks, stream_, At_.it.d, (const int *)At_.rp,
                       (const int *)At_.ci, Atv, gat, pa, (const CpalState *)st_, wt, koff);
    });
}

template <typename T>
void CpalSolver::launch_dual(int koff, bool major, bool timed) {
    if (m_ == 0) return;
    auto &v = vecs<T>();
    const T *Av = matvals<T>(A_.v, A_.vf);
    DualArgs<T> da{v.y, v.yh, v.ybar, v.ax, v.u, anchor<T>(y0_, y0f_), anchor<T>(ax0_, ax0f_), v.clb, v.cub};
    const auto *wt = weights<T>(wt_, wtf_);
    const T *xbar = v.xbar;
    const int *rp = A_.rp, *ci = A_.ci;
    const CpalState *st = st_;
    if (!use_panels_) {
        const PlanDev &pl = A_.it;
        PDAL_WITH_S(S_it_, {
            if (major) {
                if (beta_on_)
                    launch_pdl(k_dual<T, SB, true, true>, pl.d.nblocks, stream_, pl.d, rp, ci, Av, xbar, da, st, wt, koff);
                else
                    launch_pdl(k_dual<T, SB, true, false>, pl.d.nblocks, stream_, pl.d, rp, ci, Av, xbar, da, st, wt,
                               koff);
            } else {
                if (beta_on_)
                    launch_pdl(k_dual<T, SB, false, true>, pl.d.nblocks, stream_, pl.d, rp, ci, Av, xbar, da, st, wt,
                               koff);
                else
                    launch_pdl(k_dual<T, SB, false, false>, pl.d.nblocks, stream_, pl.d, rp, ci, Av, xbar, da, st, wt,
                               koff);
            }
        });
        return;
    }
    const PanelDev<T> pd = panel_dev<T>();
    const size_t psm = panel_smem_bytes<T>(pd.W);
    if (forked<T>()) {
        /* the panel partials on the side stream, concurrently with the short
         * rows: both only read x-bar and write disjoint outputs */
        PDAL_CUDA(cudaEventRecord(fork_ev_, stream_));
        PDAL_CUDA(cudaStreamWaitEvent(side_, fork_ev_, 0));
        k_dual_panels<T, false, false, false><<<pd.nblocks, kPanelThreads, psm, side_>>>(pd, xbar, n_, st, da, wt, koff);
        PDAL_LAUNCH_CHECK();
        PDAL_CUDA(cudaEventRecord(join_ev_, side_));
    }
    /* rows within the row-block budget, split by length */
    if (sh_b1_ + sh_b2_ + sh_b3_ > 0) {
        const ShortDev<T> sd = short_dev<T>();
        const int g = sh_b1_ + sh_b2_ + sh_b3_;
        if (major) {
            if (beta_on_)
                launch_pdl(k_dual_short<T, true, true>, g, stream_, sd, rp, ci, Av, xbar, da, st, wt, koff);
            else
                launch_pdl(k_dual_short<T, true, false>, g, stream_, sd, rp, ci, Av, xbar, da, st, wt, koff);
        } else {
            if (beta_on_)
                launch_pdl(k_dual_short<T, false, true>, g, stream_, sd, rp, ci, Av, xbar, da, st, wt, koff);
            else
                launch_pdl(k_dual_short<T, false, false>, g, stream_, sd, rp, ci, Av, xbar, da, st, wt, koff);
        }
    }
    /* the long rows: panel partials, then one warp per row for the sum and
     * the dual epilogue */
    const int gf = (pd.H * 32 + kThreads - 1) / kThreads;
    if (forked<T>()) {
        PDAL_CUDA(cudaStreamWaitEvent(stream_, join_ev_, 0));
        if (major) {
            if (beta_on_)
                k_dual_long_finish<T, true, true><<<gf, kThreads, 0, stream_>>>(pd, da, st, wt, koff);
            else
                k_dual_long_finish<T, true, false><<<gf, kThreads, 0, stream_>>>(pd, da, st, wt, koff);
        } else {
            if (beta_on_)
                k_dual_long_finish<T, false, true><<<gf, kThreads, 0, stream_>>>(pd, da, st, wt, koff);
            else
                k_dual_long_finish<T, false, false><<<gf, kThreads, 0, stream_>>>(pd, da, st, wt, koff);
        }
        PDAL_LAUNCH_CHECK();
        return;
    }
    if (timed) PDAL_CUDA(cudaEventRecordWithFlags(ev_[4], stream_, cudaEventRecordExternal));
    if (fuse_finish_) {
        /* the group that writes a long row's last partial finishes the row */
        if (major) {
            if (beta_on_)
                launch_pdl_cfg(k_dual_panels<T, true, true, true>, pd.nblocks, kPanelThreads, psm, stream_, pd, xbar,
                               n_, st, da, wt, koff);
            else
                launch_pdl_cfg(k_dual_panels<T, true, true, false>, pd.nblocks, kPanelThreads, psm, stream_, pd, xbar,
                               n_, st, da, wt, koff);
        } else {
            if (beta_on_)
                launch_pdl_cfg(k_dual_panels<T, true, false, true>, pd.nblocks, kPanelThreads, psm, stream_, pd, xbar,
                               n_, st, da, wt, koff);
            else
                launch_pdl_cfg(k_dual_panels<T, true, false, false>, pd.nblocks, kPanelThreads, psm, stream_, pd, xbar,
                               n_, st, da, wt, koff);
        }
        if (timed) PDAL_CUDA(cudaEventRecordWithFlags(ev_[5], stream_, cudaEventRecordExternal));
        return;
    }
    launch_pdl_cfg(k_dual_panels<T, false, false, false>, pd.nblocks, kPanelThreads, psm, stream_, pd, xbar, n_, st, da,
                   wt, koff);
    if (timed) PDAL_CUDA(cudaEventRecordWithFlags(ev_[5], stream_, cudaEventRecordExternal));
    if (major) {
        if (beta_on_)
            launch_pdl(k_dual_long_finish<T, true, true>, gf, stream_, pd, da, st, wt, koff);
        else
            launch_pdl(k_dual_long_finish<T, true, false>, gf, stream_, pd, da, st, wt, koff);
    } else {
        if (beta_on_)
            launch_pdl(k_dual_long_finish<T, false, true>, gf, stream_, pd, da, st, wt, koff);
        else
            launch_pdl(k_dual_long_finish<T, false, false>, gf, stream_, pd, da, st, wt, koff);
    }
}

template <typename T>
void CpalSolver::launch_iteration(int koff, bool major) {
    launch_primal<T>(koff, major);
    launch_dual<T>(koff, major);
}

template <typename T>
void CpalSolver::launch_eval_terms() {
    auto &v = vecs<T>();
    EvalRowArgs<T> ra{v.xh, v.xbar, v.yh, v.ybar, x0_, y0_, ax0_, clb_, cub_, clbf_, cubf_, rsc_, phat_, part_row_,
                      A_.ev.d.nblocks, v.x, v.y, v.ax};
    EvalColArgs<T> ca{v.xh, v.xbar, v.yh, v.ybar, v.lam, x0_, c_, dsc_, part_col_, At_.ev.d.nblocks, v.x, v.y, y0_};
    PDAL_WITH_SE(S_ev_, {
        if (m_ > 0) k_eval_rows<T, SE><<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(A_.ev.d, A_.rp, A_.ci, A_.v, ra, st_);
        k_eval_cols<T, SE><<<At_.ev.d.nblocks, kThreads, 0, stream_>>>(At_.ev.d, At_.rp, At_.ci, At_.v, ca, st_);
    });
}

template <typename T>
void CpalSolver::launch_eval() {
    auto &v = vecs<T>();
    EvalRowArgs<T> ra{v.xh, v.xbar, v.yh, v.ybar, x0_, y0_, ax0_, clb_, cub_, clbf_, cubf_, rsc_, phat_, part_row_,
                      A_.ev.d.nblocks, v.x, v.y, v.ax};
    EvalColArgs<T> ca{v.xh, v.xbar, v.yh, v.ybar, v.lam, x0_, c_, dsc_, part_col_, At_.ev.d.nblocks, v.x, v.y, y0_};
    if (cp_.restart_select && cp_.restart_threepoint) {
        PDAL_WITH_SE(S_ev_, {
            if (m_ > 0)
                k_eval_rows<T, SE, true>
                    <<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(A_.ev.d, A_.rp, A_.ci, A_.v, ra, st_);
            k_eval_cols<T, SE, true, true>
                <<<At_.ev.d.nblocks, kThreads, 0, stream_>>>(At_.ev.d, At_.rp, At_.ci, At_.v, ca, st_);
        });
    } else if (cp_.restart_select) {
        PDAL_WITH_SE(S_ev_, {
            if (m_ > 0)
                k_eval_rows<T, SE, true>
                    <<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(A_.ev.d, A_.rp, A_.ci, A_.v, ra, st_);
            k_eval_cols<T, SE, true>
                <<<At_.ev.d.nblocks, kThreads, 0, stream_>>>(At_.ev.d, At_.rp, At_.ci, At_.v, ca, st_);
        });
    } else {
        PDAL_WITH_SE(S_ev_, {
            if (m_ > 0)
                k_eval_rows<T, SE><<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(A_.ev.d, A_.rp, A_.ci, A_.v, ra, st_);
            k_eval_cols<T, SE><<<At_.ev.d.nblocks, kThreads, 0, stream_>>>(At_.ev.d, At_.rp, At_.ci, At_.v, ca, st_);
        });
    }
    const int nrow_slots = m_ > 0 ? A_.ev.d.nblocks + A_.ev.d.nlong : 0;
    const int ncol_slots = At_.ev.d.nblocks + At_.ev.d.nlong;
    if (cp_.infeas) {
        RayArgs<T> rr{v.xh, v.yh, x0_, y0_, vlb_, vub_, clb_, cub_, clbf_, cubf_, rsc_, dsc_, c_, part_ray_row_,
                      A_.ev.d.nblocks};
        RayArgs<T> rc = rr;
        rc.part = part_ray_col_;
        rc.nblocks = At_.ev.d.nblocks;
        PDAL_WITH_SE(S_ev_, {
            if (m_ > 0) k_ray_rows<T, SE><<<A_.ev.d.nblocks, kThreads, 0, stream_>>>(A_.ev.d, A_.rp, A_.ci, A_.v, rr, st_);
            k_ray_cols<T, SE><<<At_.ev.d.nblocks, kThreads, 0, stream_>>>(At_.ev.d, At_.rp, At_.ci, At_.v, rc, st_);
        });
    }
    k_control<<<1, kThreads, 0, stream_>>>(part_row_, nrow_slots, part_col_, ncol_slots, part_ray_row_,
                                           cp_.infeas ? nrow_slots : 0, part_ray_col_, cp_.infeas ? ncol_slots : 0,
                                           st_, cp_, wt_, wtf_);
    const int gr = grid_for(std::max(n_, m_));
    const bool f32 = std::is_same<T, float>::value;
    float2 *x0f = f32 ? x0f_ : nullptr, *y0f = f32 ? y0f_ : nullptr, *ax0f = f32 ? ax0f_ : nullptr;
    if (beta_on_)
        k_restart<T, true><<<gr, kThreads, 0, stream_>>>(st_, n_, m_, v.xh, v.x, x0_, x0f, v.yh, v.y, y0_, y0f, phat_,
                                                         v.ax, ax0_, ax0f, v.u, v.clb, v.cub, v.xbar, v.ybar);
    else
        k_restart<T, false><<<gr, kThreads, 0, stream_>>>(st_, n_, m_, v.xh, v.x, x0_, x0f, v.yh, v.y, y0_, y0f,
                                                          phat_, v.ax, ax0_, ax0f, v.u, v.clb, v.cub, v.xbar, v.ybar);
}

template <typename T>
void CpalSolver::capture_block(cudaGraphExec_t &exec, int F) {
    const int G = graph_blocks();
    const bool timing = O_.timing != 0;
    if (timing && !ev_[0])
        for (auto &e : ev_) PDAL_CUDA(cudaEventCreate(&e));
    PDAL_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    for (int g = 0; g < G; ++g) {
        if (timing && g == 0) PDAL_CUDA(cudaEventRecordWithFlags(ev_[3], stream_, cudaEventRecordExternal));
        for (int i = 1; i <= F; ++i) {
            /* one non-major iteration (F-1 >= 2) is bracketed by events */
            if (timing && g == 0 && i == F - 1) {
                PDAL_CUDA(cudaEventRecordWithFlags(ev_[0], stream_, cudaEventRecordExternal));
                launch_primal<T>(i, false);
                PDAL_CUDA(cudaEventRecordWithFlags(ev_[1], stream_, cudaEventRecordExternal));
                launch_dual<T>(i, false, use_panels_);
                PDAL_CUDA(cudaEventRecordWithFlags(ev_[2], stream_, cudaEventRecordExternal));
            } else {
                launch_iteration<T>(i, i == F);
            }
        }
        launch_eval<T>();
    }
    cudaGraph_t graph;
    PDAL_CUDA(cudaStreamEndCapture(stream_, &graph));
    PDAL_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    PDAL_CUDA(cudaGraphDestroy(graph));
}

void CpalSolver::switch_to_fp64() {
    /* FP64 refinement phase: restart from the FP32 iterate (x0 = x = x^,
     * y0 = y = y^), recompute A x0 and the predictor exactly in FP64, and
     * keep every controller scalar (weight, step, sigma, counters). */
    const size_t n = n_, m = m_;
    auto up = [&](const float *src, double *dst, size_t len) {
        if (len) k_convert<float, double><<<grid_for(len), kThreads, 0, stream_>>>(src, dst, (int)len);
        launches += 1;
    };
    up(v32_.xh, v64_.xh, n);
    up(v32_.xh, v64_.x, n);
    up(v32_.xh, x0_, n);
    up(v32_.xbar, v64_.xbar, n);
    up(v32_.lam, v64_.lam, n);
    up(v32_.yh, v64_.yh, m);
    up(v32_.yh, v64_.y, m);
    up(v32_.yh, y0_, m);
    up(v32_.ybar, v64_.ybar, m);
    PDAL_LAUNCH_CHECK();
    CpalState s = *h_st_;
    s.inner = 0;
    s.fp_last = INFINITY;
    if (!s.restart) s.fp0 = s.fp;
    s.phase_switch = 0;
    s.fp32_switch_tol = -1.0;
    s.restart = 0;
    *h_st_ = s;
    PDAL_CUDA(cudaMemcpyAsync(st_, h_st_, sizeof(CpalState), cudaMemcpyHostToDevice, stream_));
    h2d += sizeof(CpalState);
    k_fill_weights<<<1, kThreads, 0, stream_>>>(st_, wt_, wtf_, cp_.F);
    launches += 1;
    fp32_phase_ = false;
    launch_init_ax<double>();
}

/*
 * Feasibility polishing.  Primal phase: c = 0, the dual iterates at zero,
 * the primal ones as the solve left them; dual phase: every finite bound 0,
 * the primal iterates at zero, the dual ones as the solve left them.  Each
 * phase keeps the step size, the AL / sigma coefficients and the counters of
 * the solve except the primal weight (that of the start of the solve) and the
 * Halpern counter, and runs blocks of F iterations with the restart rule on a
 * one-sided fixed-point error until its relative residual is below
 * eps_feas_polish_relative.  The evaluation kernels of the loop supply the
 * residual terms; restarts reset one side's anchor and refresh A x0 and the
 * AL predictor.  A successful phase replaces that side's solution, residuals
 * and objective (the primal objective without the objective constant, as
 * utils.cu:1388-1391 computes it).  Runs in FP64: a solve still in its FP32
 * phase switches to FP64 first.
 */
void CpalSolver::polish() {
    const double t_start = now_sec();
    const double eps = P_.termination_criteria.eps_feas_polish_relative;
    const CpalState base = host_state;
    if (base.rel_p < eps && base.rel_d < eps) return; /* solver.cu:3915-3920 */
    if (fp32_phase_) {
        switch_to_fp64();
        PDAL_CUDA(cudaStreamSynchronize(stream_));
    }
    const size_t n = n_, m = m_, mm = std::max<size_t>(m, 1);
    const int F = cp_.F;
    auto &v = v64_;
    /* saved state of the solve: 8 n-vectors, 9 m-vectors, two scalars */
    double *sv = nullptr;
    const size_t total_doubles = 8 * n + 9 * mm + 2;
    PDAL_CUDA(cudaMalloc(&sv, total_doubles * sizeof(double)));
    PolishEval *pe_d = nullptr, *pe_h = nullptr;
    PDAL_CUDA(cudaMalloc(&pe_d, sizeof(PolishEval)));
    PDAL_CUDA(cudaMallocHost(&pe_h, sizeof(PolishEval)));
    struct Free {
        double *a;
        PolishEval *b, *c;
        ~Free() {
            if (a) cudaFree(a);
            if (b) cudaFree(b);
            if (c) cudaFreeHost(c);
        }
    } guard{sv, pe_d, pe_h};
    double *p = sv;
    double *s_x = p, *s_x0 = (p += n), *s_xh = (p += n), *s_xbar = (p += n), *s_lam = (p += n), *s_c = (p += n),
           *s_vlb = (p += n), *s_vub = (p += n);
    double *s_y = (p += n), *s_y0 = (p += mm), *s_yh = (p += mm), *s_ybar = (p += mm), *s_ax = (p += mm),
           *s_ax0 = (p += mm), *s_u = (p += mm), *s_clb = (p += mm), *s_cub = (p += mm);
    double *dot_out = (p += mm);
    auto cp = [&](double *dst, const double *src, size_t len) {
        if (len) PDAL_CUDA(cudaMemcpyAsync(dst, src, len * sizeof(double), cudaMemcpyDeviceToDevice, stream_));
    };
    auto zero = [&](double *dst, size_t len) {
        if (len) PDAL_CUDA(cudaMemsetAsync(dst, 0, len * sizeof(double), stream_));
    };
    auto save = [&]() {
        cp(s_x, v.x, n), cp(s_x0, x0_, n), cp(s_xh, v.xh, n), cp(s_xbar, v.xbar, n), cp(s_lam, v.lam, n);
        cp(s_c, c_, n), cp(s_vlb, vlb_, n), cp(s_vub, vub_, n);
        cp(s_y, v.y, m), cp(s_y0, y0_, m), cp(s_yh, v.yh, m), cp(s_ybar, v.ybar, m), cp(s_ax, v.ax, m);
        cp(s_ax0, ax0_, m), cp(s_u, v.u, m), cp(s_clb, clb_, m), cp(s_cub, cub_, m);
    };
    auto restore = [&]() {
        cp(v.x, s_x, n), cp(x0_, s_x0, n), cp(v.xh, s_xh, n), cp(v.xbar, s_xbar, n), cp(v.lam, s_lam, n);
        cp(c_, s_c, n), cp(vlb_, s_vlb, n), cp(vub_, s_vub, n);
        cp(v.y, s_y, m), cp(y0_, s_y0, m), cp(v.yh, s_yh, m), cp(v.ybar, s_ybar, m), cp(v.ax, s_ax, m);
        cp(ax0_, s_ax0, m), cp(v.u, s_u, m), cp(clb_, s_clb, m), cp(cub_, s_cub, m);
    };
    save();
    const double pw0 = P_.bound_objective_rescaling ? 1.0 : (cp_.obj_norm + 1.0) / (cp_.bnd_norm + 1.0);
    const int gm = grid_for(std::max<size_t>(m, 1)), gn = grid_for(std::max<size_t>(n, 1));
    const int nrow_slots = m_ > 0 ? A_.ev.d.nblocks + A_.ev.d.nlong : 0;
    const int ncol_slots = At_.ev.d.nblocks + At_.ev.d.nlong;
    auto evaluate = [&]() {
        launch_eval_terms<double>();
        k_polish_reduce<<<1, kThreads, 0, stream_>>>(part_row_, nrow_slots, part_col_, ncol_slots, pe_d);
        PDAL_LAUNCH_CHECK();
        launches += 3;
        PDAL_CUDA(cudaMemcpyAsync(pe_h, pe_d, sizeof(PolishEval), cudaMemcpyDeviceToHost, stream_));
        PDAL_CUDA(cudaStreamSynchronize(stream_));
        return *pe_h;
    };
    auto refresh_predictor = [&]() {
        if (beta_on_ && m) {
            k_predictor<<<gm, kThreads, 0, stream_>>>(m_, v.ax, v.y, clb_, cub_, v.u, st_);
            PDAL_LAUNCH_CHECK();
            launches += 1;
        }
    };
    auto dot = [&](const double *a, const double *b) {
        k_dot_block<<<1, kThreads, 0, stream_>>>(n_, a, b, dot_out);
        PDAL_LAUNCH_CHECK();
        launches += 1;
        double h = 0.0;
        PDAL_CUDA(cudaMemcpyAsync(&h, dot_out, sizeof(double), cudaMemcpyDeviceToHost, stream_));
        PDAL_CUDA(cudaStreamSynchronize(stream_));
        return h;
    };
    const bool linf = cp_.norm_linf;
    /* one phase; returns its termination_reason_t code and fills the
     * residuals of its side */
    auto phase = [&](bool primal, double &abs_r, double &rel_r, int &total, PolishEval &last) {
        CpalState s = base;
        s.status = 0;
        s.restart = 0;
        s.pw = pw0;
        s.best_pw = pw0;
        s.pw_esum = s.pw_last = 0.0;
        s.best_gap = INFINITY;
        s.fp = s.fp0 = s.fp_last = INFINITY;
        s.inner = 0;
        s.total = 0;
        s.fp32_switch_tol = -1.0;
        cpal_set_coefficients(s);
        auto push = [&]() {
            *h_st_ = s;
            PDAL_CUDA(cudaMemcpyAsync(st_, h_st_, sizeof(CpalState), cudaMemcpyHostToDevice, stream_));
            k_fill_weights<<<1, kThreads, 0, stream_>>>(st_, wt_, wtf_, F);
            PDAL_LAUNCH_CHECK();
            launches += 1;
        };
        push();
        refresh_predictor();
        const int limit = cp_.iteration_limit;
        bool do_restart = false;
        int status = 0;
        auto fpe = [&](const PolishEval &e) { return primal ? e.dx2 * s.pw : e.dy2 / s.pw; };
        for (;;) { /* solver.cu:3988-4051 (primal), 4063-4126 (dual) */
            launch_iteration<double>(1, true);
            launches += iter_launches() + (hot_in<double>() ? 1 : 0);
            if (do_restart) {
                s.fp = fpe(evaluate());
                s.fp0 = s.fp;
                do_restart = false;
            }
            for (int k = 2; k <= F - 1; ++k) launch_iteration<double>(k, false);
            launch_iteration<double>(F, true);
            launches += (int64_t)iter_launches() * (F - 1);
            last = evaluate();
            s.fp = fpe(last);
            if (primal) { /* utils.cu:1341-1392 */
                abs_r = (linf ? last.rpmax : std::sqrt(last.rp2)) / s.cbr;
                rel_r = abs_r / (1.0 + cp_.bnd_norm);
            } else { /* utils.cu:1394-1453 */
                abs_r = (linf ? last.rdmax : std::sqrt(last.rd2)) / s.ovr;
                rel_r = abs_r / (1.0 + cp_.obj_norm);
            }
            s.inner += F;
            s.total += F;
            /* utils.cu:1194-1226; the time limit is the solve's */
            if (rel_r <= eps) {
                status = TERMINATION_REASON_FEAS_POLISH_SUCCESS;
                break;
            }
            if (s.total >= limit) {
                status = TERMINATION_REASON_ITERATION_LIMIT;
                break;
            }
            if (now_sec() - loop_t0_ >= cp_.time_limit) {
                status = TERMINATION_REASON_TIME_LIMIT;
                break;
            }
            do_restart = cpal_should_restart(s, cp_, cp_.F);
            if (do_restart) { /* solver.cu:4376-4404 */
                if (primal) {
                    cp(v.x, v.xh, n);
                    cp(x0_, v.xh, n);
                    push();
                    launch_init_ax<double>(); /* A x0 = A x and the predictor */
                } else {
                    cp(v.y, v.yh, m);
                    cp(y0_, v.yh, m);
                }
                s.inner = 0;
                s.fp_last = INFINITY;
            }
            push();
            if (do_restart && !primal) refresh_predictor();
        }
        total = s.total;
        return status;
    };
    CpalState out = base;
    int iters = 0;
    {   /* primal phase (solver.cu:4131-4200 state) */
        zero(c_, n);
        zero(v.y, m), zero(y0_, m), zero(v.yh, m), zero(v.ybar, m), zero(v.lam, n);
        double abs_r = 0, rel_r = 0;
        int total = 0;
        PolishEval last{};
        const int st = phase(true, abs_r, rel_r, total, last);
        polish_status[0] = st;
        if (st == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
            out.abs_p = abs_r;
            out.rel_p = rel_r;
            out.pobj = dot(s_c, v.xh) / (base.cbr * base.ovr);
            cp(s_xh, v.xh, n);
        }
        iters += total - 1;
        restore();
    }
    {   /* dual phase (solver.cu:4247-4330 state) */
        for (double *b : {clb_, cub_})
            if (m) k_zero_finite<<<gm, kThreads, 0, stream_>>>(m_, b);
        for (double *b : {vlb_, vub_}) k_zero_finite<<<gn, kThreads, 0, stream_>>>(n_, b);
        PDAL_LAUNCH_CHECK();
        launches += 4;
        zero(v.x, n), zero(x0_, n), zero(v.xh, n), zero(v.xbar, n), zero(v.ax, m), zero(ax0_, m);
        double abs_r = 0, rel_r = 0;
        int total = 0;
        PolishEval last{};
        const int st = phase(false, abs_r, rel_r, total, last);
        polish_status[1] = st;
        if (st == TERMINATION_REASON_FEAS_POLISH_SUCCESS) {
            out.abs_d = abs_r;
            out.rel_d = rel_r;
            out.dobj = (dot(v.lam, s_xh) + last.contrib) / (base.cbr * base.ovr) + cp_.obj_const;
            cp(s_yh, v.yh, m);
        }
        iters += total - 1;
        restore();
    }
    out.gap = std::fabs(out.pobj - out.dobj);
    out.rel_gap = out.gap / (1.0 + std::fabs(out.pobj) + std::fabs(out.dobj));
    host_state.abs_p = out.abs_p;
    host_state.rel_p = out.rel_p;
    host_state.pobj = out.pobj;
    host_state.abs_d = out.abs_d;
    host_state.rel_d = out.rel_d;
    host_state.dobj = out.dobj;
    host_state.gap = out.gap;
    host_state.rel_gap = out.rel_gap;
    /* the device state returns to the solve's, for the result kernels */
    *h_st_ = host_state;
    PDAL_CUDA(cudaMemcpyAsync(st_, h_st_, sizeof(CpalState), cudaMemcpyHostToDevice, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    polish_iters = iters;
    polish_sec = now_sec() - t_start;
}

void CpalSolver::run_loop() {
    const double t0 = now_sec();
    loop_t0_ = t0;
    const int F = cp_.F;
    const int G = graph_blocks();
    const int F0 = h_st_->F;
    k_start_clock<<<1, 1, 0, stream_>>>(st_);
    PDAL_LAUNCH_CHECK();
    launches += 1;
    const int fp32_cap = O_.fp32_max_iterations;
    setup_loop();
    for (;;) {
        if (use_loop_) {
            /* evaluation blocks on the device until a termination, the end
             * of the FP32 phase or this many blocks (the host then checks
             * its wall-clock guard and prints the verbose line) */
            int chunk = (P_.verbose || (fp32_phase_ && fp32_cap >= 0)) ? 1 : 50;
            /* the launch's barrier counter (blocks x barriers) stays below 2^31 */
            const long long per = (2LL * F + 3) * std::max(loop_grid_[0], loop_grid_[1]);
            chunk = (int)std::max(1LL, std::min<long long>(chunk, (1LL << 31) / std::max(per, 1LL)));
            if (fp32_phase_)
                launch_loop<float>(chunk);
            else
                launch_loop<double>(chunk);
        } else {
            const int Fb = h_st_->F; /* this block's length (the dynamic evaluation frequency may shorten it) */
            const int64_t per_block = (int64_t)iter_launches() * Fb + (m_ > 0 ? 4 : 3) +
                                      (cp_.infeas ? (m_ > 0 ? 2 : 1) : 0);
            cudaGraphExec_t *exec;
            if (fp32_phase_) {
                exec = &exec32_[beta_on_ ? 1 : 0][Fb != F ? 1 : 0];
                if (!*exec) capture_block<float>(*exec, Fb);
            } else {
                exec = &exec64_[beta_on_ ? 1 : 0][Fb != F ? 1 : 0];
                if (!*exec) capture_block<double>(*exec, Fb);
            }
            PDAL_CUDA(cudaGraphLaunch(*exec, stream_));
            launches += (per_block + ((fp32_phase_ ? hot_in<float>() : hot_in<double>()) ? 1 : 0)) * G;
        }
        PDAL_CUDA(cudaMemcpyAsync(h_st_, st_, sizeof(CpalState), cudaMemcpyDeviceToHost, stream_));
        d2h += sizeof(CpalState);
        PDAL_CUDA(cudaStreamSynchronize(stream_));
        if (!use_loop_ && O_.timing && F >= 3 && ev_[0]) {
            float a = 0, b = 0, c = 0;
            PDAL_CUDA(cudaEventElapsedTime(&a, ev_[0], ev_[1]));
            PDAL_CUDA(cudaEventElapsedTime(&b, ev_[1], ev_[2]));
            PDAL_CUDA(cudaEventElapsedTime(&c, ev_[3], ev_[2]));
            const int ph = fp32_phase_ ? 1 : 0;
            sum_ms[ph][0] += a;
            sum_ms[ph][1] += b;
            sum_ms[ph][2] += c;
            if (use_panels_ && !(fp32_phase_ ? forked<float>() : forked<double>())) {
                float d = 0, e = 0;
                PDAL_CUDA(cudaEventElapsedTime(&d, ev_[1], ev_[4]));
                PDAL_CUDA(cudaEventElapsedTime(&e, ev_[4], ev_[5]));
                sub_ms[ph][0] += d;
                sub_ms[ph][1] += e;
            }
            timed[ph] += 1;
        }
        if (fp32_phase_) fp32_iters = h_st_->total;
        if (P_.verbose) {
            /* one line per block, the columns of display_iteration_stats
             * (LP/CP_AL/src/utils.cu:613-634) plus weight, step and phase */
            const CpalState &q = *h_st_;
            printf("%8d %.2e | %+.6e %+.6e | %.1e %.1e %.1e | %.1e | pw %.3e eta %.3e beta %.3e rs %d %s\n", q.total,
                   now_sec() - t0, q.pobj, q.dobj, q.rel_p, q.rel_d, q.rel_gap, q.fp, q.pw, q.step, q.beta,
                   q.restarts, fp32_phase_ ? "fp32" : "fp64");
            fflush(stdout);
        }
        if (h_st_->status == kStatusDeviceError) check_device_error();
        if (cp_.pulse) pulse_report();
        if (cp_.dyn && h_st_->F != F0 && !dyn_reported_) {
            /* LP/CP_AL/src/solver.cu:1557-1569 */
            dyn_reported_ = true;
            if (P_.verbose || cp_.dyn_sec > 0.0 || cp_.dyn_iters > 0)
                printf("[dynamic-eval] iter=%d solve_sec=%.12e eval_frequency=%d->%d relative_primal=%.12e "
                       "relative_dual=%.12e\n",
                       h_st_->total, h_st_->elapsed, F0, h_st_->F, h_st_->rel_p, h_st_->rel_d);
        }
        if (cp_.trigger && h_st_->trigger_iter && P_.verbose && h_st_->restart && h_st_->trigger_iter == h_st_->total)
            printf("sigma-trigger iter %d rpr %.12e rdr %.12e sigma %.12e base %.12e\n", h_st_->total, h_st_->rel_p,
                   h_st_->rel_d, h_st_->sigma, h_st_->sigma_base);
        if (h_st_->status) break;
        /* the device enforces the time limit; this host guard only covers a
         * device clock that does not advance */
        if (now_sec() - t0 > cp_.time_limit + 60.0) {
            h_st_->status = TERMINATION_REASON_TIME_LIMIT;
            break;
        }
        /* the alpha pulse and the sigma trigger change the AL penalty only at
         * a restart (x = x0): the next block runs the iteration form of the
         * new penalty, starting from A x0 and the predictor recomputed */
        const bool beta_now = h_st_->beta > 0.0;
        const bool beta_up = beta_now && !beta_on_;
        beta_on_ = beta_now;
        if (fp32_phase_ && (h_st_->phase_switch || (fp32_cap >= 0 && h_st_->total >= fp32_cap))) {
            switch_to_fp64();
        } else if (beta_up) {
            if (fp32_phase_)
                launch_init_ax<float>();
            else
                launch_init_ax<double>();
        }
    }
    if (fp32_phase_) {
        /* finished inside the FP32 phase: promote the reported iterate */
        const size_t n = n_, m = m_;
        if (n) k_convert<float, double><<<grid_for(n), kThreads, 0, stream_>>>(v32_.xh, v64_.xh, n_);
        if (m) k_convert<float, double><<<grid_for(m), kThreads, 0, stream_>>>(v32_.yh, v64_.yh, m_);
        PDAL_LAUNCH_CHECK();
        launches += 2;
    }
    host_state = *h_st_;
    loop_sec = now_sec() - t0;
    if (cp_.pulse) {
        /* LP/CP_AL/src/solver.cu:1009-1032 */
        const CpalState &q = host_state;
        const int started = q.pulse_phase != 0, completed = q.pulse_phase == 2;
        const int aborted = completed && q.pulse_status != 0 && q.pulse_status != TERMINATION_REASON_OPTIMAL;
        fprintf(stderr,
                "[alpha-direct-pulse-final] charged_iter=%d trajectory_iter=%d started=%d completed=%d aborted=%d "
                "gate_evaluated=%d gate_passed=%d gate_rejected=%d gate_anchor_charged_iter=%d gate_previous_K=%d "
                "gate_recent_K=%d gate_delta_fp_rate=%.12e positive_charged_iters=%d final_alpha=%.12e "
                "final_penalty=%.12e\n",
                q.total, q.total, started, completed, aborted, q.pulse_gate != 0, q.pulse_gate == 1, q.pulse_gate == 2,
                pulse_gate_iter_, pulse_gate_k_[0], pulse_gate_k_[1], pulse_gate_rate_[1] - pulse_gate_rate_[0],
                completed ? cp_.F : 0, q.al_lambda, q.beta);
        fflush(stderr);
    }
}

/* The alpha pulse's stderr lines (LP/CP_AL/src/solver.cu:893-988, 1017-1028),
 * printed from the state after each evaluation block: the gate when it was
 * evaluated, the start of the positive block and its end. */
void CpalSolver::pulse_report() {
    const CpalState &q = *h_st_;
    if (q.pulse_gate && !pulse_seen_gate_) {
        pulse_seen_gate_ = q.pulse_gate;
        pulse_gate_iter_ = q.total;
        for (int i = 0; i < 2; ++i) {
            pulse_gate_k_[i] = q.hist_iters[i];
            pulse_gate_rate_[i] = q.hist_fp_rate[i];
        }
        fprintf(stderr,
                "[alpha-deterministic-tail-anchor] charged_iter=%d trajectory_iter=%d previous_K=%d recent_K=%d "
                "previous_fp_rate=%.12e recent_fp_rate=%.12e delta_fp_rate=%.12e pass=%d force_pulse=%d\n",
                q.total, q.total, q.hist_iters[0], q.hist_iters[1], q.hist_fp_rate[0], q.hist_fp_rate[1],
                q.hist_fp_rate[1] - q.hist_fp_rate[0], q.pulse_gate == 1, cp_.pulse_force);
    }
    if (q.pulse_phase >= 1 && pulse_seen_phase_ < 1)
        fprintf(stderr,
                "[alpha-direct-pulse-start] charged_iter=%d trajectory_iter=%d alpha=2.000000000000e-03 "
                "pulse_iterations=%d\n",
                q.pulse_start, q.pulse_start, cp_.F);
    if (q.pulse_phase == 2 && pulse_seen_phase_ < 2)
        fprintf(stderr,
                "[alpha-direct-pulse-complete] charged_iter=%d trajectory_iter=%d positive_iters=%d fp0map=%.12e "
                "primal=%.12e dual=%.12e gap=%.12e term=%d\n",
                q.total, q.total, cp_.F, q.pulse_fp, q.pulse_p, q.pulse_d, q.pulse_g, q.pulse_status);
    pulse_seen_phase_ = q.pulse_phase;
    fflush(stderr);
}

bool CpalSolver::extend(int n) {
    if (n <= 0) return false;
    const CpalState &q = host_state;
    if (q.status != 0 && q.status != TERMINATION_REASON_ITERATION_LIMIT) return false;
    const int F = cp_.F;
    const int blocks = (n + F - 1) / F;
    CpalState s = *h_st_;
    s.status = 0;
    s.iter_limit = s.total + blocks * F;
    *h_st_ = s;
    PDAL_CUDA(cudaMemcpyAsync(st_, h_st_, sizeof(CpalState), cudaMemcpyHostToDevice, stream_));
    h2d += sizeof(CpalState);
    return true;
}

void CpalSolver::result_on_device() {
    ResultColEpi epi;
    epi.xh = v64_.xh;
    epi.c = c_;
    epi.cscale = dsc_;
    epi.vlb = vlb_;
    epi.vub = vub_;
    epi.st = st_;
    epi.x_out = xout_;
    epi.rc_out = rcout_;
    PDAL_WITH_SE(S_ev_, {
        k_result_cols<SE><<<At_.ev.d.nblocks, kThreads, 0, stream_>>>(At_.ev.d, At_.rp, At_.ci, At_.v, v64_.yh, epi);
    });
    if (m_) k_result_rows<<<grid_for(m_), kThreads, 0, stream_>>>(m_, v64_.yh, rsc_, st_, yout_);
    PDAL_LAUNCH_CHECK();
    launches += 2;
}

void CpalSolver::fetch_vectors(double *x, double *y, double *rc) {
    if (x) PDAL_CUDA(cudaMemcpyAsync(x, xout_, sizeof(double) * n_, cudaMemcpyDeviceToHost, stream_));
    if (y && m_) PDAL_CUDA(cudaMemcpyAsync(y, yout_, sizeof(double) * m_, cudaMemcpyDeviceToHost, stream_));
    if (rc) PDAL_CUDA(cudaMemcpyAsync(rc, rcout_, sizeof(double) * n_, cudaMemcpyDeviceToHost, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    d2h += (int64_t)sizeof(double) * ((x ? n_ : 0) + (y ? m_ : 0) + (rc ? n_ : 0));
}

void CpalSolver::fetch_scaling(double *vals, double *rsc, double *csc, double *bo) {
    if (vals && nnz_) PDAL_CUDA(cudaMemcpyAsync(vals, A_.v, sizeof(double) * nnz_, cudaMemcpyDeviceToHost, stream_));
    if (rsc && m_) PDAL_CUDA(cudaMemcpyAsync(rsc, rsc_, sizeof(double) * m_, cudaMemcpyDeviceToHost, stream_));
    if (csc) PDAL_CUDA(cudaMemcpyAsync(csc, dsc_, sizeof(double) * n_, cudaMemcpyDeviceToHost, stream_));
    PDAL_CUDA(cudaStreamSynchronize(stream_));
    if (bo) {
        bo[0] = host_state.cbr;
        bo[1] = host_state.ovr;
    }
}

void CpalSolver::download(cp_al_result_t *res, bool vectors) {
    check_device_error();
    const CpalState &s = host_state;
    res->num_variables = n_;
    res->num_constraints = m_;
    res->num_nonzeros = nnz_;
    res->total_count = s.total;
    res->rescaling_time_sec = setup_sec;
    res->cumulative_time_sec = loop_sec;
    res->presolve_time = 0.0;
    res->presolve_status = 0;
    res->absolute_primal_residual = s.abs_p;
    res->relative_primal_residual = s.rel_p;
    res->absolute_dual_residual = s.abs_d;
    res->relative_dual_residual = s.rel_d;
    res->primal_objective_value = s.pobj;
    res->dual_objective_value = s.dobj;
    res->objective_gap = s.gap;
    res->relative_objective_gap = s.rel_gap;
    res->termination_reason = (termination_reason_t)s.status;
    res->max_primal_ray_infeasibility = s.ray_pinf;
    res->max_dual_ray_infeasibility = s.ray_dinf;
    res->primal_ray_linear_objective = s.ray_pobj;
    res->dual_ray_objective = s.ray_dobj;
    if (vectors) {
        res->primal_solution = (double *)malloc(sizeof(double) * std::max(n_, 1));
        res->dual_solution = (double *)malloc(sizeof(double) * std::max(m_, 1));
        res->reduced_cost = (double *)malloc(sizeof(double) * std::max(n_, 1));
        if (!res->primal_solution || !res->dual_solution || !res->reduced_cost) throw Error("out of host memory");
        fetch_vectors(res->primal_solution, res->dual_solution, res->reduced_cost);
    }
}

} // namespace pdal

/* ---------------------------------------------------------------------- */
/* C entry points                                                          */
/* ---------------------------------------------------------------------- */
namespace {
thread_local std::string g_last_error;

void set_error(const std::string &msg) {
    g_last_error = msg;
    fprintf(stderr, "[cp_al_gb300] %s\n", msg.c_str());
}
} // namespace

namespace pdal {
void set_last_error(const std::string &msg) { set_error(msg); }
void clear_last_error() { g_last_error.clear(); }
} // namespace pdal

struct cp_al_gb300_session {
    std::unique_ptr<pdal::CpalSolver> solver;
    lp_problem_t prob_copy;
};

extern "C" {

const char *cp_al_gb300_last_error(void) { return g_last_error.c_str(); }

void cp_al_gb300_last_stats(cp_al_gb300_stats_t *out) {
    if (out) *out = pdal::g_stats;
}

static void fill_stats(const pdal::CpalSolver &s, double total) {
    cp_al_gb300_stats_t &st = pdal::g_stats;
    memset(&st, 0, sizeof(st));
    st.setup_sec = s.setup_sec;
    st.loop_sec = s.loop_sec;
    st.total_sec = total;
    st.lambda_est = s.host_state.lambda_est;
    st.power_iterations = s.power_iters;
    st.restarts = s.host_state.restarts;
    st.fp32_iterations = s.fp32_iters;
    st.kernel_launches = s.launches;
    st.h2d_bytes = s.h2d;
    st.d2h_bytes = s.d2h;
    st.primal_weight = s.host_state.pw;
    if (s.timed[0] > 0) {
        st.avg_primal_ms = s.sum_ms[0][0] / s.timed[0];
        st.avg_dual_ms = s.sum_ms[0][1] / s.timed[0];
        st.avg_block_ms = s.sum_ms[0][2] / s.timed[0];
        st.timed_blocks = s.timed[0];
    }
    if (s.timed[1] > 0) {
        st.avg_primal32_ms = s.sum_ms[1][0] / s.timed[1];
        st.avg_dual32_ms = s.sum_ms[1][1] / s.timed[1];
        st.avg_block32_ms = s.sum_ms[1][2] / s.timed[1];
        st.timed_blocks32 = s.timed[1];
    }
    st.step_size = s.host_state.step;
    st.al_penalty = s.host_state.beta;
    st.prepare_sec = s.prepare_sec;
    st.upload_sec = s.upload_sec;
    st.upload_plan_sec = s.upload_plan_sec;
    st.upload_alloc_sec = s.upload_alloc_sec;
    st.equilibration_sec = s.equil_sec;
    st.power_sec = s.power_sec;
    st.polish_primal_status = s.polish_status[0];
    st.polish_dual_status = s.polish_status[1];
    st.cr_passes = s.cr_passes;
    if (s.timed[0]) {
        st.avg_dual_rows_ms = s.sub_ms[0][0] / s.timed[0];
        st.avg_dual_panels_ms = s.sub_ms[0][1] / s.timed[0];
    }
    if (s.timed[1]) {
        st.avg_dual_rows32_ms = s.sub_ms[1][0] / s.timed[1];
        st.avg_dual_panels32_ms = s.sub_ms[1][1] / s.timed[1];
    }
    st.panel_rows = s.panel_rows();
    st.panels = s.panels();
    st.pulse_start_iteration = s.host_state.pulse_phase ? s.host_state.pulse_start : -1;
    st.pulse_gate = s.host_state.pulse_gate;
    st.sigma_trigger_iteration = s.host_state.trigger_iter;
    st.dynamic_eval_iteration = s.host_state.dyn_iter;
}

/* Options from the environment, unless a switch of a controller this library
 * lacks is set (then false, with the message). */
static bool options_from_env_checked(cp_al_gb300_options_t &o, const char *who) {
    if (const char *sw = cp_al_gb300_unbuilt_switch()) {
        set_error(std::string(who) + ": " + sw + " is set, but the controller it enables is not part of this library");
        return false;
    }
    cp_al_gb300_options_from_env(&o);
    return true;
}

cp_al_result_t *cp_al_gb300_solve(lp_problem_t *prob, const cp_al_parameters_t *params,
                                  const cp_al_gb300_options_t *opts) {
    g_last_error.clear();
    if (!prob) {
        set_error("solve_lp_problem: invalid arguments.");
        return nullptr;
    }
    cp_al_parameters_t local;
    if (params)
        local = *params;
    else
        set_default_parameters(&local);
    cp_al_gb300_options_t o;
    if (opts)
        o = *opts;
    else if (!options_from_env_checked(o, "solve_lp_problem"))
        return nullptr;
    const double t0 = pdal::now_sec();
    cp_al_result_t *res = (cp_al_result_t *)calloc(1, sizeof(cp_al_result_t));
    if (!res) {
        set_error("out of host memory");
        return nullptr;
    }
    try {
        pdal::CpalSolver s(prob, &local, &o);
        s.prepare();
        s.upload();
        s.setup_device();
        s.run_loop();
        /* solver.cu:1715-1719: no polishing after an infeasibility status
         * (only infeasibility detection, off by default, produces one) */
        if (local.feasibility_polishing && s.host_state.status != TERMINATION_REASON_PRIMAL_INFEASIBLE &&
            s.host_state.status != TERMINATION_REASON_DUAL_INFEASIBLE)
            s.polish();
        s.result_on_device();
        s.download(res, true);
        res->feasibility_polishing_time = s.polish_sec;
        res->feasibility_iteration = s.polish_iters;
        fill_stats(s, pdal::now_sec() - t0);
        if (local.verbose) {
            printf("Solution Summary\n  Status                 : %d\n  Iterations             : %d\n"
                   "  Primal objective       : %.10g\n  Dual objective         : %.10g\n",
                   (int)res->termination_reason, res->total_count, res->primal_objective_value,
                   res->dual_objective_value);
        }
        return res;
    } catch (const std::exception &e) {
        set_error(e.what());
        free(res->primal_solution);
        free(res->dual_solution);
        free(res->reduced_cost);
        free(res);
        return nullptr;
    }
}

cp_al_result_t *solve_lp_problem(lp_problem_t *prob, const cp_al_parameters_t *params) {
    return cp_al_gb300_solve(prob, params, nullptr);
}

cp_al_gb300_session_t *cp_al_gb300_session_create(const lp_problem_t *prob, const cp_al_parameters_t *params,
                                                  const cp_al_gb300_options_t *opts) {
    g_last_error.clear();
    if (!prob) {
        set_error("session_create: invalid arguments.");
        return nullptr;
    }
    cp_al_gb300_options_t o;
    if (opts)
        o = *opts;
    else if (!options_from_env_checked(o, "session_create"))
        return nullptr;
    try {
        auto *sess = new cp_al_gb300_session;
        cp_al_parameters_t local;
        if (params)
            local = *params;
        else
            set_default_parameters(&local);
        sess->prob_copy = *prob;
        sess->solver.reset(new pdal::CpalSolver(&sess->prob_copy, &local, &o));
        sess->solver->prepare();
        sess->solver->upload();
        PDAL_CUDA(cudaDeviceSynchronize());
        return sess;
    } catch (const std::exception &e) {
        set_error(e.what());
        return nullptr;
    }
}

int cp_al_gb300_session_solve(cp_al_gb300_session_t *s, cp_al_result_t *summary) {
    if (!s) return -1;
    try {
        const double t0 = pdal::now_sec();
        s->solver->setup_device();
        s->solver->run_loop();
        s->solver->result_on_device();
        PDAL_CUDA(cudaDeviceSynchronize());
        if (summary) s->solver->download(summary, false);
        fill_stats(*s->solver, pdal::now_sec() - t0);
        return 0;
    } catch (const std::exception &e) {
        set_error(e.what());
        return -1;
    }
}

int cp_al_gb300_session_fetch(cp_al_gb300_session_t *s, double *primal, double *dual, double *reduced_cost) {
    if (!s) return -1;
    try {
        s->solver->fetch_vectors(primal, dual, reduced_cost);
        return 0;
    } catch (const std::exception &e) {
        set_error(e.what());
        return -1;
    }
}

void cp_al_gb300_session_free(cp_al_gb300_session_t *s) { delete s; }

int cp_al_gb300_session_start(cp_al_gb300_session_t *s) {
    if (!s) return -1;
    try {
        s->solver->setup_device();
        s->solver->host_state.status = TERMINATION_REASON_ITERATION_LIMIT;
        s->solver->started = true;
        return 0;
    } catch (const std::exception &e) {
        set_error(e.what());
        return -1;
    }
}

int cp_al_gb300_session_iterate(cp_al_gb300_session_t *s, int iterations, cp_al_result_t *summary) {
    if (!s || iterations < 0) return -1;
    try {
        if (!s->solver->started) {
            set_error("session_iterate: call cp_al_gb300_session_start first");
            return -1;
        }
        const double t0 = pdal::now_sec();
        if (s->solver->extend(iterations)) s->solver->run_loop();
        PDAL_CUDA(cudaDeviceSynchronize());
        if (summary) s->solver->download(summary, false);
        fill_stats(*s->solver, pdal::now_sec() - t0);
        return 0;
    } catch (const std::exception &e) {
        set_error(e.what());
        return -1;
    }
}

int cp_al_gb300_session_scaling(cp_al_gb300_session_t *s, double *scaled_values, double *row_scale,
                                double *col_scale, double *bound_obj_factors, double *lambda_est) {
    if (!s) return -1;
    try {
        s->solver->setup_device();
        s->solver->fetch_scaling(scaled_values, row_scale, col_scale, bound_obj_factors);
        if (lambda_est) *lambda_est = s->solver->host_state.lambda_est;
        return 0;
    } catch (const std::exception &e) {
        set_error(e.what());
        return -1;
    }
}

} // extern "C"

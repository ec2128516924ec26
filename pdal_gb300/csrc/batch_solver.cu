/*
 * batch_solver.cu -- host side of the batched CP_AL solver
 * (cp_al_gb300_batch_solve): validation, transposes and row-block plans per
 * instance (host threads), one packed image of every instance's arrays
 * uploaded with a single copy, the persistent launch of batch_kernels.cuh,
 * and the per-instance results.
 */
#include "../../include/cp_al.h"
#include "../../include/cp_al_gb300.h"
#include "batch_kernels.cuh"
#include "common.h"
#include "cpal_setup.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <functional>
#include <mutex>
#include <random>
#include <thread>
#include <vector>
#include <tuple>
#include <map>

namespace pdal {
namespace {

using namespace batch;

/* Candidate schedules of the persistent launch: row-block nonzero budget x
 * resident blocks per SM (every pair has a kernel instantiation; 2,048 x 4
 * does not fit the SM's shared memory). */
struct Schedule {
    int bs, minb;
};
constexpr Schedule kSchedules[] = {{2048, 2}, {2048, 3}, {1024, 2}, {1024, 3}, {1024, 4}};

double now_sec() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

/* Offsets (bytes from the image base) of one instance's arrays. */
struct Layout {
    size_t Arp, Aci, Av, Atrp, Atci, Atv, Adesc, Alinfo, Alpart, Alcount, Atdesc, Atlinfo, Atlpart, Atlcount;
    size_t c, vlb, vub, clb, cub, x0, y0, x, xbar, xh, lam, y, yh, ybar, ax, u, ax0, phat;
    size_t dsc, rsc, clbf, cubf, tn, tm, tm2, pv0;
    size_t Avf, Atvf, cf, vlbf, vubf, clbF, cubF, xf, xbarf, xhf, lamf, yf, yhf, ybarf, axf, uf, x0f, y0f, ax0f;
    size_t out_x, out_y, out_rc;
};

struct Prepared {
    HostCsr At;
    HostPlan pa, pat;
    CpalParams cp;
};

class Packer {
  public:
    size_t take(size_t bytes) {
        const size_t o = off_;
        off_ += (std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
        return o;
    }
    size_t size() const { return off_; }

  private:
    size_t off_ = 0;
};

void run_threads(int count, const std::function<void(int)> &fn) {
    const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), 32));
    std::atomic<int> next{0};
    std::vector<std::thread> th;
    std::exception_ptr err = nullptr;
    std::mutex mu;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&]() {
            for (;;) {
                const int i = next.fetch_add(1);
                if (i >= count) break;
                try {
                    fn(i);
                } catch (...) {
                    std::lock_guard<std::mutex> lk(mu);
                    if (!err) err = std::current_exception();
                }
            }
        });
    for (auto &t : th) t.join();
    if (err) std::rethrow_exception(err);
}

int run_batch(int count, lp_problem_t *const *problems, const cp_al_parameters_t &P, const cp_al_gb300_options_t &O,
              const double *sigma0, cp_al_result_t **results, cp_al_gb300_instance_info_t *info,
              cp_al_gb300_batch_stats_t *stats, int bs, int minb) {
    const double t_begin = now_sec();
    if (count <= 0) throw Error("batch_solve: count must be positive");
    if (!problems || !results) throw Error("batch_solve: missing problem or result array");
    if (P.termination_evaluation_frequency < 3) throw Error("termination_evaluation_frequency must be >= 3");
    std::vector<Prepared> prep(count);
    run_threads(count, [&](int i) {
        const lp_problem_t *q = problems[i];
        if (!q) throw Error("batch_solve: NULL problem " + std::to_string(i));
        const int n = q->num_variables, m = q->num_constraints, nnz = q->constraint_matrix_num_nonzeros;
        if (n <= 0 || m < 0) throw Error("batch_solve: instance " + std::to_string(i) + " has no variables");
        if (!q->objective_vector || !q->variable_lower_bound || !q->variable_upper_bound ||
            (m > 0 && (!q->constraint_lower_bound || !q->constraint_upper_bound)))
            throw Error("batch_solve: instance " + std::to_string(i) + " misses a vector");
        csr_validate(m, n, q->constraint_matrix_row_pointers, q->constraint_matrix_col_indices, nnz,
                     "constraint matrix");
        Prepared &p = prep[i];
        p.At = csr_transpose(m, n, q->constraint_matrix_row_pointers, q->constraint_matrix_col_indices,
                             q->constraint_matrix_values);
        p.pa = plan_rows(m, q->constraint_matrix_row_pointers, bs);
        p.pat = plan_rows(n, p.At.rp.data(), bs);
        p.cp = resolve_cpal_params(P, O, q);
        p.cp.infeas = 0; /* the batch controller evaluates no rays */
        /* nor runs the alpha pulse or the sigma trigger (their step changes
         * switch the iteration's kernel form, fixed per batch launch) */
        p.cp.pulse = 0;
        p.cp.trigger = 0;
        p.cp.dyn = 0; /* nor a changing block length */
    });

    /* image layout */
    Packer pk;
    std::vector<Layout> L(count);
    for (int i = 0; i < count; ++i) {
        const lp_problem_t *q = problems[i];
        const size_t n = q->num_variables, m = q->num_constraints, nnz = q->constraint_matrix_num_nonzeros;
        const Prepared &p = prep[i];
        Layout &l = L[i];
        l.Arp = pk.take((m + 1) * 4);
        l.Aci = pk.take((nnz + 8) * 4);
        l.Av = pk.take((nnz + 8) * 8);
        l.Atrp = pk.take((n + 1) * 4);
        l.Atci = pk.take((nnz + 8) * 4);
        l.Atv = pk.take((nnz + 8) * 8);
        l.Adesc = pk.take(p.pa.desc.size() * 4);
        l.Alinfo = pk.take(p.pa.linfo.size() * 4);
        l.Alpart = pk.take((size_t)kLongStride * std::max(p.pa.npieces, 1) * 8);
        l.Alcount = pk.take((size_t)std::max(p.pa.nlong, 1) * 4);
        l.Atdesc = pk.take(p.pat.desc.size() * 4);
        l.Atlinfo = pk.take(p.pat.linfo.size() * 4);
        l.Atlpart = pk.take((size_t)kLongStride * std::max(p.pat.npieces, 1) * 8);
        l.Atlcount = pk.take((size_t)std::max(p.pat.nlong, 1) * 4);
        for (size_t *f : {&l.c, &l.vlb, &l.vub, &l.x0, &l.x, &l.xbar, &l.xh, &l.lam, &l.dsc, &l.tn}) *f = pk.take(n * 8);
        for (size_t *f : {&l.clb, &l.cub, &l.y0, &l.y, &l.yh, &l.ybar, &l.ax, &l.u, &l.ax0, &l.phat, &l.rsc, &l.clbf,
                          &l.cubf, &l.tm, &l.tm2, &l.pv0})
            *f = pk.take(m * 8);
        const bool f32 = O.precision == CP_AL_GB300_FP32_REFINE;
        const size_t fn = f32 ? n : 0, fm = f32 ? m : 0, fz = f32 ? nnz + 8 : 0;
        l.Avf = pk.take(fz * 4);
        l.Atvf = pk.take(fz * 4);
        for (size_t *f : {&l.cf, &l.vlbf, &l.vubf, &l.xf, &l.xbarf, &l.xhf, &l.lamf}) *f = pk.take(fn * 4);
        for (size_t *f : {&l.clbF, &l.cubF, &l.yf, &l.yhf, &l.ybarf, &l.axf, &l.uf}) *f = pk.take(fm * 4);
        l.x0f = pk.take(fn * 8);
        l.y0f = pk.take(fm * 8);
        l.ax0f = pk.take(fm * 8);
    }
    /* outputs last, contiguous: one download */
    const size_t out_begin = pk.size();
    for (int i = 0; i < count; ++i) {
        const lp_problem_t *q = problems[i];
        L[i].out_x = pk.take((size_t)q->num_variables * 8);
        L[i].out_rc = pk.take((size_t)q->num_variables * 8);
        L[i].out_y = pk.take((size_t)q->num_constraints * 8);
    }
    const size_t outs_off = pk.take(sizeof(BOut) * count);
    const size_t out_end = pk.size();
    const size_t insts_off = pk.take(sizeof(BInst) * count);
    const size_t order_off = pk.take(sizeof(int) * count);
    const size_t queue_off = pk.take(sizeof(unsigned));
    const size_t total = pk.size();

    char *dev = nullptr, *host = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    struct Guard {
        char *&d, *&h;
        cudaStream_t &s;
        cudaEvent_t &a, &b;
        ~Guard() {
            if (d) cudaFree(d);
            if (h) cudaFreeHost(h);
            if (s) cudaStreamDestroy(s);
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } guard{dev, host, stream, e0, e1};
    if (O.device >= 0) PDAL_CUDA(cudaSetDevice(O.device));
    PDAL_CUDA(cudaMalloc(&dev, total));
    PDAL_CUDA(cudaMallocHost(&host, total));
    PDAL_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    PDAL_CUDA(cudaEventCreate(&e0));
    PDAL_CUDA(cudaEventCreate(&e1));

    /* fill the image (host threads) */
    std::vector<BInst> insts(count);
    run_threads(count, [&](int i) {
        const lp_problem_t *q = problems[i];
        const int n = q->num_variables, m = q->num_constraints, nnz = q->constraint_matrix_num_nonzeros;
        const Prepared &p = prep[i];
        const Layout &l = L[i];
        auto put = [&](size_t off, const void *src, size_t bytes) {
            if (bytes) memcpy(host + off, src, bytes);
        };
        auto zero = [&](size_t off, size_t bytes) { memset(host + off, 0, bytes); };
        put(l.Arp, q->constraint_matrix_row_pointers, (size_t)(m + 1) * 4);
        zero(l.Aci, (size_t)(nnz + 8) * 4);
        zero(l.Av, (size_t)(nnz + 8) * 8);
        put(l.Aci, q->constraint_matrix_col_indices, (size_t)nnz * 4);
        put(l.Av, q->constraint_matrix_values, (size_t)nnz * 8);
        put(l.Atrp, p.At.rp.data(), (size_t)(n + 1) * 4);
        zero(l.Atci, (size_t)(nnz + 8) * 4);
        zero(l.Atv, (size_t)(nnz + 8) * 8);
        put(l.Atci, p.At.ci.data(), (size_t)nnz * 4);
        put(l.Atv, p.At.v.data(), (size_t)nnz * 8);
        put(l.Adesc, p.pa.desc.data(), p.pa.desc.size() * 4);
        put(l.Alinfo, p.pa.linfo.data(), p.pa.linfo.size() * 4);
        zero(l.Alcount, (size_t)std::max(p.pa.nlong, 1) * 4);
        put(l.Atdesc, p.pat.desc.data(), p.pat.desc.size() * 4);
        put(l.Atlinfo, p.pat.linfo.data(), p.pat.linfo.size() * 4);
        zero(l.Atlcount, (size_t)std::max(p.pat.nlong, 1) * 4);
        put(l.c, q->objective_vector, (size_t)n * 8);
        put(l.vlb, q->variable_lower_bound, (size_t)n * 8);
        put(l.vub, q->variable_upper_bound, (size_t)n * 8);
        if (q->primal_start)
            put(l.x0, q->primal_start, (size_t)n * 8);
        else
            zero(l.x0, (size_t)n * 8);
        put(l.clb, q->constraint_lower_bound, (size_t)m * 8);
        put(l.cub, q->constraint_upper_bound, (size_t)m * 8);
        if (q->dual_start)
            put(l.y0, q->dual_start, (size_t)m * 8);
        else
            zero(l.y0, (size_t)m * 8);
        /* power-iteration start: std::normal_distribution over
         * std::mt19937(1), what a fresh reference process draws */
        {
            std::mt19937 gen(1);
            std::normal_distribution<double> dist(0.0, 1.0);
            double *v = reinterpret_cast<double *>(host + l.pv0);
            for (int k = 0; k < m; ++k) v[k] = dist(gen);
        }
        BInst &I = insts[i];
        I.m = m;
        I.n = n;
        I.nnz = nnz;
        I.nbA = p.pa.nblocks;
        I.nlA = p.pa.nlong;
        I.nbAt = p.pat.nblocks;
        I.nlAt = p.pat.nlong;
        auto D = [&](size_t off) { return dev + off; };
        I.Arp = (const int *)D(l.Arp);
        I.Aci = (const int *)D(l.Aci);
        I.Av = (double *)D(l.Av);
        I.Atrp = (const int *)D(l.Atrp);
        I.Atci = (const int *)D(l.Atci);
        I.Atv = (double *)D(l.Atv);
        I.Adesc = (const int4 *)D(l.Adesc);
        I.Alinfo = (const int4 *)D(l.Alinfo);
        I.Alpart = (double *)D(l.Alpart);
        I.Alcount = (unsigned *)D(l.Alcount);
        I.Atdesc = (const int4 *)D(l.Atdesc);
        I.Atlinfo = (const int4 *)D(l.Atlinfo);
        I.Atlpart = (double *)D(l.Atlpart);
        I.Atlcount = (unsigned *)D(l.Atlcount);
        I.c = (double *)D(l.c);
        I.vlb = (double *)D(l.vlb);
        I.vub = (double *)D(l.vub);
        I.clb = (double *)D(l.clb);
        I.cub = (double *)D(l.cub);
        I.x0 = (double *)D(l.x0);
        I.y0 = (double *)D(l.y0);
        I.x = (double *)D(l.x);
        I.xbar = (double *)D(l.xbar);
        I.xh = (double *)D(l.xh);
        I.lam = (double *)D(l.lam);
        I.y = (double *)D(l.y);
        I.yh = (double *)D(l.yh);
        I.ybar = (double *)D(l.ybar);
        I.ax = (double *)D(l.ax);
        I.u = (double *)D(l.u);
        I.ax0 = (double *)D(l.ax0);
        I.phat = (double *)D(l.phat);
        I.dsc = (double *)D(l.dsc);
        I.rsc = (double *)D(l.rsc);
        I.clbf = (double *)D(l.clbf);
        I.cubf = (double *)D(l.cubf);
        I.tn = (double *)D(l.tn);
        I.tm = (double *)D(l.tm);
        I.tm2 = (double *)D(l.tm2);
        I.pv0 = (const double *)D(l.pv0);
        I.Avf = (float *)D(l.Avf);
        I.Atvf = (float *)D(l.Atvf);
        I.cf = (float *)D(l.cf);
        I.vlbf = (float *)D(l.vlbf);
        I.vubf = (float *)D(l.vubf);
        I.clbF = (float *)D(l.clbF);
        I.cubF = (float *)D(l.cubF);
        I.xf = (float *)D(l.xf);
        I.xbarf = (float *)D(l.xbarf);
        I.xhf = (float *)D(l.xhf);
        I.lamf = (float *)D(l.lamf);
        I.yf = (float *)D(l.yf);
        I.yhf = (float *)D(l.yhf);
        I.ybarf = (float *)D(l.ybarf);
        I.axf = (float *)D(l.axf);
        I.uf = (float *)D(l.uf);
        I.x0f = (float2 *)D(l.x0f);
        I.y0f = (float2 *)D(l.y0f);
        I.ax0f = (float2 *)D(l.ax0f);
        I.out_x = (double *)D(l.out_x);
        I.out_y = (double *)D(l.out_y);
        I.out_rc = (double *)D(l.out_rc);
        I.obj_norm = p.cp.obj_norm;
        I.bnd_norm = p.cp.bnd_norm;
        I.obj_const = p.cp.obj_const;
        I.sigma0 = (sigma0 && std::isfinite(sigma0[i])) ? sigma0[i] : 0.0;
    });
    memcpy(host + insts_off, insts.data(), sizeof(BInst) * count);
    std::vector<int> order(count);
    for (int i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const long long wa = (long long)problems[a]->constraint_matrix_num_nonzeros + problems[a]->num_variables;
        const long long wb = (long long)problems[b]->constraint_matrix_num_nonzeros + problems[b]->num_variables;
        return wa > wb;
    });
    memcpy(host + order_off, order.data(), sizeof(int) * count);
    memset(host + queue_off, 0, sizeof(unsigned));
    const double t_prep = now_sec();

    PDAL_CUDA(cudaMemcpyAsync(dev, host, total, cudaMemcpyHostToDevice, stream));
    PDAL_CUDA(cudaStreamSynchronize(stream));
    const double t_up = now_sec();

    BOpts bo{};
    bo.ruiz = P.l_inf_ruiz_iterations;
    bo.pc = P.has_pock_chambolle_alpha ? 1 : 0;
    bo.pc_alpha = P.pock_chambolle_alpha;
    bo.boundobj = P.bound_objective_rescaling ? 1 : 0;
    bo.sv_max_iter = P.sv_max_iter;
    bo.sv_tol = P.sv_tol;
    bo.al_lambda = O.al_lambda;
    bo.sigma_mode = O.sigma_mode;
    bo.sigma_set = O.sigma_set;
    bo.sigma_adaptive = O.sigma_adaptive;
    bo.lambda_param_set = O.lambda_param_set;
    bo.sigma = O.sigma;
    bo.sigma_init_factor = O.sigma_init_factor;
    bo.sigma_min_factor = O.sigma_min_factor;
    bo.sigma_max_factor = O.sigma_max_factor;
    bo.lambda_param = O.lambda_param;
    bo.fp32 = O.precision == CP_AL_GB300_FP32_REFINE ? 1 : 0;
    bo.fp32_stall_evals = O.fp32_stall_evals;
    bo.fp32_switch_tol = O.fp32_switch_tol;
    CpalParams cp = prep[0].cp; /* instance-specific norms are overridden per instance in the kernel */
    if (cp.restart_select != 0) throw Error("batch_solve: restart_select is not supported by the batched solver");
    if (O.cr_iterations > 0) throw Error("batch_solve: Curtis-Reid scaling is not supported by the batched solver");
    if (O.alpha_direct_pulse || O.sigma_trigger || O.dynamic_eval || O.dynamic_eval_after_sec > 0.0 ||
        O.dynamic_eval_after_iters > 0)
        throw Error("batch_solve: the alpha pulse, the sigma trigger and the dynamic evaluation frequency are not "
                    "supported by the batched solver");

    int dev_id = 0, sms = 0, per_sm = 0;
    PDAL_CUDA(cudaGetDevice(&dev_id));
    PDAL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
    using KernT = void (*)(const BInst *, int, const int *, unsigned *, CpalParams, BOpts, BOut *);
    KernT kern;
    size_t dsm;
    if (bs == 2048) {
        if (minb > 3) throw Error("batch_solve: 2,048-nonzero blocks fit at most 3 per SM");
        kern = minb == 3 ? k_batch_lp<3, 2048> : k_batch_lp<2, 2048>; /* 3: ~70 KB of staging each */
        dsm = sizeof(BSmem<2048>);
    } else {
        kern = minb == 4 ? k_batch_lp<4, 1024> : (minb == 3 ? k_batch_lp<3, 1024> : k_batch_lp<2, 1024>);
        dsm = sizeof(BSmem<1024>);
    }
    PDAL_CUDA(cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm));
    PDAL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, dsm));
    if (per_sm < 1) throw Error("the batch kernel does not fit on one SM");
    const int grid = std::max(1, std::min(count, per_sm * sms));
    PDAL_CUDA(cudaEventRecord(e0, stream));
    kern<<<grid, kThreads, dsm, stream>>>((const BInst *)(dev + insts_off), count, (const int *)(dev + order_off),
                                          (unsigned *)(dev + queue_off), cp, bo, (BOut *)(dev + outs_off));
    PDAL_CUDA(cudaGetLastError());
    PDAL_CUDA(cudaEventRecord(e1, stream));
    PDAL_CUDA(cudaMemcpyAsync(host + out_begin, dev + out_begin, out_end - out_begin, cudaMemcpyDeviceToHost, stream));
    PDAL_CUDA(cudaStreamSynchronize(stream));
    float kms = 0.f;
    PDAL_CUDA(cudaEventElapsedTime(&kms, e0, e1));
    const double t_kernel_end = now_sec();

    const BOut *outs = reinterpret_cast<const BOut *>(host + outs_off);
    std::vector<int> iters(count);
    int optimal = 0;
    long long total_iters = 0;
    for (int i = 0; i < count; ++i) {
        const lp_problem_t *q = problems[i];
        const int n = q->num_variables, m = q->num_constraints;
        const BOut &o = outs[i];
        cp_al_result_t *r = (cp_al_result_t *)calloc(1, sizeof(cp_al_result_t));
        r->primal_solution = (double *)malloc(sizeof(double) * std::max(n, 1));
        r->dual_solution = (double *)malloc(sizeof(double) * std::max(m, 1));
        r->reduced_cost = (double *)malloc(sizeof(double) * std::max(n, 1));
        memcpy(r->primal_solution, host + L[i].out_x, sizeof(double) * n);
        memcpy(r->reduced_cost, host + L[i].out_rc, sizeof(double) * n);
        if (m) memcpy(r->dual_solution, host + L[i].out_y, sizeof(double) * m);
        r->num_variables = n;
        r->num_constraints = m;
        r->num_nonzeros = q->constraint_matrix_num_nonzeros;
        r->num_reduced_variables = n;
        r->num_reduced_constraints = m;
        r->num_reduced_nonzeros = q->constraint_matrix_num_nonzeros;
        r->total_count = o.iterations;
        r->rescaling_time_sec = o.setup_sec;
        r->cumulative_time_sec = o.elapsed;
        r->absolute_primal_residual = o.abs_p;
        r->relative_primal_residual = o.rel_p;
        r->absolute_dual_residual = o.abs_d;
        r->relative_dual_residual = o.rel_d;
        r->primal_objective_value = o.pobj;
        r->dual_objective_value = o.dobj;
        r->objective_gap = std::fabs(o.pobj - o.dobj);
        r->relative_objective_gap = o.rel_gap;
        r->termination_reason = (termination_reason_t)o.status;
        results[i] = r;
        if (info) {
            cp_al_gb300_instance_info_t &f = info[i];
            f.sigma = o.sigma;
            f.sigma_best = o.sigma_best;
            f.primal_weight = o.pw;
            f.step_size = o.step;
            f.lambda_est = o.lambda_est;
            f.restarts = o.restarts;
            f.power_iterations = o.power_iters;
            f.fp32_iterations = o.fp32_iterations;
        }
        iters[i] = o.iterations;
        total_iters += o.iterations;
        if (o.status == TERMINATION_REASON_OPTIMAL) ++optimal;
    }
    const double t_end = now_sec();
    if (stats) {
        std::vector<int> sorted = iters;
        std::sort(sorted.begin(), sorted.end());
        auto pct = [&](double f) {
            const size_t k = (size_t)std::min<double>(sorted.size() - 1, std::ceil(f * sorted.size()) - 1);
            return sorted[k];
        };
        memset(stats, 0, sizeof(*stats));
        stats->instances = count;
        stats->optimal = optimal;
        stats->grid_blocks = grid;
        stats->host_prep_sec = t_prep - t_begin;
        stats->upload_sec = t_up - t_prep;
        stats->kernel_sec = kms * 1e-3;
        stats->download_sec = t_end - t_kernel_end;
        stats->total_sec = t_end - t_begin;
        stats->solves_per_sec = count / stats->total_sec;
        stats->iterations_p50 = pct(0.5);
        stats->iterations_p99 = pct(0.99);
        stats->iterations_max = sorted.back();
        stats->total_iterations = total_iters;
        stats->device_bytes = (long long)total;
        stats->block_nnz = bs;
        stats->blocks_per_sm = minb;
    }
    return 0;
}

/* Schedules chosen for earlier batches of the same shape (instance count,
 * nonzeros in total and in the largest instance, precision). */
std::mutex g_sched_mu;
std::map<std::tuple<int, long long, long long, int>, Schedule> g_sched;

/*
 * The autotuner: the largest instances bound the makespan (each runs on one
 * block from start to end), so every candidate schedule solves the same probe
 * -- the SM-count largest instances, 100 iterations and at most 8 power
 * iterations each -- and the fastest kernel time wins.  A schedule the caller
 * fixes (spmv_nnz_per_block, batch_blocks_per_sm) restricts the candidates.
 */
Schedule tune_schedule(int count, lp_problem_t *const *problems, const cp_al_parameters_t &P,
                       const cp_al_gb300_options_t &O, double &tune_sec) {
    const int want_bs = O.spmv_nnz_per_block, want_mb = O.batch_blocks_per_sm;
    if (want_bs != 0 && want_bs != 1024 && want_bs != 2048)
        throw Error("batch_solve: spmv_nnz_per_block must be 0, 1024 or 2048");
    if (want_mb != 0 && (want_mb < 2 || want_mb > 4)) throw Error("batch_solve: batch_blocks_per_sm must be 0 or 2-4");
    std::vector<Schedule> cand;
    for (const Schedule &c : kSchedules)
        if ((want_bs == 0 || c.bs == want_bs) && (want_mb == 0 || c.minb == want_mb)) cand.push_back(c);
    if (cand.empty()) throw Error("batch_solve: no schedule with 2,048-nonzero blocks at 4 blocks per SM");
    tune_sec = 0.0;
    if (cand.size() == 1) return cand[0];
    long long tot = 0, mx = 0;
    for (int i = 0; i < count; ++i) {
        const long long w = problems[i] ? problems[i]->constraint_matrix_num_nonzeros : 0;
        tot += w;
        mx = std::max(mx, w);
    }
    const auto key = std::make_tuple(count, tot, mx, O.precision * 16 + want_bs / 1024 * 4 + want_mb);
    {
        std::lock_guard<std::mutex> lk(g_sched_mu);
        auto it = g_sched.find(key);
        if (it != g_sched.end()) return it->second;
    }
    const double t0 = now_sec();
    int dev_id = 0, sms = 0;
    if (O.device >= 0) PDAL_CUDA(cudaSetDevice(O.device));
    PDAL_CUDA(cudaGetDevice(&dev_id));
    PDAL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
    std::vector<int> idx(count);
    for (int i = 0; i < count; ++i) idx[i] = i;
    auto weight = [&](int i) {
        return problems[i] ? (long long)problems[i]->constraint_matrix_num_nonzeros + problems[i]->num_variables : 0;
    };
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return weight(a) > weight(b); });
    const int k = std::min(count, sms);
    std::vector<lp_problem_t *> probe(k);
    for (int i = 0; i < k; ++i) probe[i] = problems[idx[i]];
    cp_al_parameters_t pp = P;
    pp.termination_criteria.iteration_limit = std::min(P.termination_criteria.iteration_limit, 100);
    pp.sv_max_iter = std::min(P.sv_max_iter, 8);
    std::vector<cp_al_result_t *> res(k, nullptr);
    Schedule best = cand[0];
    double best_t = INFINITY;
    for (const Schedule &c : cand) {
        cp_al_gb300_batch_stats_t st{};
        run_batch(k, probe.data(), pp, O, nullptr, res.data(), nullptr, &st, c.bs, c.minb);
        for (cp_al_result_t *&r : res) {
            cp_al_result_free(r);
            r = nullptr;
        }
        if (st.kernel_sec < best_t) {
            best_t = st.kernel_sec;
            best = c;
        }
    }
    tune_sec = now_sec() - t0;
    std::lock_guard<std::mutex> lk(g_sched_mu);
    g_sched[key] = best;
    return best;
}

int batch_solve(int count, lp_problem_t *const *problems, const cp_al_parameters_t &P, const cp_al_gb300_options_t &O,
                const double *sigma0, cp_al_result_t **results, cp_al_gb300_instance_info_t *info,
                cp_al_gb300_batch_stats_t *stats) {
    if (count <= 0) throw Error("batch_solve: count must be positive");
    if (!problems || !results) throw Error("batch_solve: missing problem or result array");
    double tune_sec = 0.0;
    const Schedule sc = tune_schedule(count, problems, P, O, tune_sec);
    const int rc = run_batch(count, problems, P, O, sigma0, results, info, stats, sc.bs, sc.minb);
    if (stats) {
        stats->tune_sec = tune_sec;
        stats->total_sec += tune_sec;
        stats->solves_per_sec = count / stats->total_sec;
    }
    return rc;
}

} // namespace
} // namespace pdal

extern "C" int cp_al_gb300_batch_tune(int count, lp_problem_t *const *problems, const cp_al_parameters_t *params,
                                      const cp_al_gb300_options_t *opts, cp_al_gb300_batch_stats_t *stats) {
    pdal::clear_last_error();
    cp_al_parameters_t p;
    if (params)
        p = *params;
    else
        set_default_parameters(&p);
    cp_al_gb300_options_t o;
    if (opts)
        o = *opts;
    else
        cp_al_gb300_default_options(&o);
    try {
        if (count <= 0 || !problems) throw pdal::Error("batch_tune: no problems");
        double t = 0.0;
        const pdal::Schedule sc = pdal::tune_schedule(count, problems, p, o, t);
        if (stats) {
            memset(stats, 0, sizeof(*stats));
            stats->instances = count;
            stats->block_nnz = sc.bs;
            stats->blocks_per_sm = sc.minb;
            stats->tune_sec = t;
        }
        return 0;
    } catch (const std::exception &e) {
        pdal::set_last_error(e.what());
        return -1;
    }
}

extern "C" int cp_al_gb300_batch_solve(int count, lp_problem_t *const *problems, const cp_al_parameters_t *params,
                                       const cp_al_gb300_options_t *opts, const double *sigma0,
                                       cp_al_result_t **results, cp_al_gb300_instance_info_t *info,
                                       cp_al_gb300_batch_stats_t *stats) {
    pdal::clear_last_error();
    cp_al_parameters_t p;
    if (params)
        p = *params;
    else
        set_default_parameters(&p);
    cp_al_gb300_options_t o;
    if (opts)
        o = *opts;
    else
        cp_al_gb300_default_options(&o);
    try {
        return pdal::batch_solve(count, problems, p, o, sigma0, results, info, stats);
    } catch (const std::exception &e) {
        pdal::set_last_error(e.what());
        return -1;
    }
}

// C ABI of libpffrg_gpu.so: context, device-resident actions and the
// sequencing of the flow right-hand side (src/Flow/compute.jl,
// src/Flow/flow_self.jl, src/Flow/SDE.jl, src/Launcher/launcher_{1l,2l,ml}.jl).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pffrg_gpu.h"
#include "pffrg_internal.h"

using namespace pffrg;

namespace {
thread_local std::string g_create_error;
constexpr int kPartials = 512;
}  // namespace

struct pffrg_ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    Layout L{};
    int symmetry = 0;
    double S = 0.5;
    int precision = PFFRG_FP64;
    DevLattice lat;
    double* mesh = nullptr;  // [σ|Ωs|νs|Ωt|νt]
    double* mesh_new = nullptr;  // the next step's meshes during a resampling
    float* mesh_ff = nullptr;    // float-float meshes of the mixed path's node setup
    long long* scan_arg = nullptr;  // [3 C] argmax of |q3| per component and channel
    double* scan_cuts = nullptr;    // [3 C][NO + 3 Nn] cuts through the maxima
    double* slot[PFFRG_NUM_SLOTS] = {};
    double* da_l = nullptr;
    double* da_c = nullptr;
    double* da_temp = nullptr;
    double* da_sig = nullptr;
    double* sig_tmp = nullptr;  // [Nsig]
    float* f_a = nullptr;       // FP32 copies for the mixed path
    float* f_da = nullptr;
    float* f_dal = nullptr;
    float* f_dtemp = nullptr;
    // the FP64 action each FP32 copy was last made from (the FP64 pass of the mixed path reads it)
    const float* f_copy[4] = {nullptr, nullptr, nullptr, nullptr};
    const double* f_src[4] = {nullptr, nullptr, nullptr, nullptr};
    double esc_eps = 1e-6;  // FP64 hand-off margin of the mixed path (0: off)
    long long chi_cluster_min = 32768;  // χ region capacity from which a cluster runs each integral
    int chi_cluster_blocks = 8;         // blocks of such a cluster (8 or 16)
    // χ integrand in FP64 on both paths (default): near the 10^7-evaluation cap the cubature does not
    // converge and FP32 rounding of the integrand changes which regions it refines
    int chi_fp64 = 1;
    std::vector<double> h_mesh;    // host copy of [σ|Ωs|νs|Ωt|νt]
    double* log_bounds = nullptr;  // [2][NO][eval+1]
    int bounds_cap = 0;            // eval the buffer holds
    std::vector<double> h_bounds;
    double* corrs = nullptr;       // [2,3,NO]
    double* corrs_sde = nullptr;   // corrs left by the last SDE call
    double* partial = nullptr;     // [kPartials]
    double* scalars = nullptr;     // [4]
    double* h_scalars = nullptr;   // pinned [4]
    int* status = nullptr;
    unsigned long long* counter = nullptr;
    // Gauss-Kronrod segment scratch: gk_slots integrals of gk_cap segments
    double* gk_seg = nullptr;
    long long gk_cap = 0, gk_slots = 0;
    int gk_overflow = 0;
    int async_waves = 1;  // device-driven quadrature levels (no host round trip per level)
    long long queue_cap_req = 0;  // chunk-queue capacity of the passes (0: queue_factor nsub + 65536)
    long long queue_factor = 8;   // chunks per subdomain of the default queue, grown after an overflow
    int queue_grow = 0;           // the last call's queue overflowed (the call is repeated with a bigger one)
    int rows_mode = 0;            // overlap rows: 0 staged by size, 1 read through L1/L2, 2 staged when they fit
    int team_T = 0, team_SPL = 0;  // requested team shape of the passes (0: chosen by Ns)
    int64_t chi_evals = 0, chi_regions_max = 0, chi_rounds = 0, chi_rounds_max = 0;
    // wave workspace of the passes (device scratch) and its host-visible counters
    void* wave_mem = nullptr;
    size_t wave_bytes = 0;
    long long wave_nsub = 0, wave_qcap = 0;
    int* h_wave_counters = nullptr;  // pinned [8]
    int queue_overflow = 0;
    int4* tasks_sym = nullptr;
    int4* tasks_full = nullptr;
    int4* tasks_red = nullptr;
    int n_sym = 0, n_full = 0, n_red = 0;
    int64_t last_evals = 0;
    int64_t last_alg_values = 0;
    // optional CUDA-event timing of the pass kernels and of whole right-hand sides
    int timing = 0;
    std::vector<cudaEvent_t> ev;  // pairs (start, stop) of the pass launches since the last reset
    int ev_used = 0;
    cudaEvent_t rhs_ev[2] = {nullptr, nullptr};
    double pass_ms = 0.0, rhs_ms = 0.0;
    int64_t pass_launches = 0, launches = 0;
    // correlations: region records of the cubature and the ω mesh of χ
    double* chi_reg = nullptr;
    int* chi_split = nullptr;
    size_t chi_reg_bytes = 0;
    int* chi_jobs = nullptr;  // job list of a cubature launch
    int* chi_over = nullptr;  // per job: 1 overflow, else minus the regions it needed
    int* chi_ctl = nullptr;   // per-job round orders of a cluster
    // the integrals that needed a cluster's capacity at the previous call run first, on a second
    // stream with their own region records, alongside the others
    cudaStream_t st_chi = nullptr;
    cudaEvent_t ev_chi = nullptr;
    double* chi_reg2 = nullptr;
    int* chi_split2 = nullptr;
    size_t chi_reg_bytes2 = 0;
    int* chi_jobs2 = nullptr;
    int* chi_over2 = nullptr;
    int* chi_ctl2 = nullptr;
    long long chi_n2 = 0;             // jobs the second stream's job and overflow words hold
    std::vector<long long> chi_need;  // per integral: the capacity it needed at the previous call
    double* chi_box = nullptr;
    double* chi_out = nullptr;
    double* chi_mesh = nullptr;
    int chi_n = 0;
    std::string err;

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
};

#define CK_PASS(call)                                                                                     \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            if (ctx->queue_overflow) {                                                                    \
                ctx->queue_overflow = 0;                                                                  \
                ctx->queue_grow = 1;                                                                      \
                return ctx->fail(PFFRG_E_LIMIT, "quadrature chunk queue capacity exceeded");              \
            }                                                                                             \
            return ctx->fail(PFFRG_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                             __LINE__);                                                                   \
        }                                                                                                 \
    } while (0)

#define CK(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return ctx->fail(PFFRG_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                             __LINE__);                                                                   \
    } while (0)

namespace {

// free a device buffer the context's stream may still be reading: wait for the stream first
cudaError_t stream_free(cudaStream_t st, void* p) {
    if (!p) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    return cudaFree(p);
}

std::vector<int4> make_tasks(int NO, int Nn, int mode) {
    // mode 0: w2 >= w3 (compute.jl:73-107), 1: all w2 (compute.jl:135-170), 2: reduced s bubble (SDE.jl:76-86)
    std::vector<int4> T;
    for (int w1 = 0; w1 < NO; ++w1) {
        T.push_back(make_int4(1, w1, -1, -1));
        for (int w3 = 0; w3 < Nn; ++w3) {
            if (mode != 2) T.push_back(make_int4(2, w1, w3, -1));
            T.push_back(make_int4(3, w1, -1, w3));
            if (mode == 2) continue;
            for (int w2 = (mode == 0 ? w3 : 0); w2 < Nn; ++w2) T.push_back(make_int4(4, w1, w2, w3));
        }
    }
    return T;
}

int check_mesh(pffrg_ctx* ctx, const pffrg_mesh_view* m) {
    if (!m || !m->sigma || !m->omega_s || !m->nu_s || !m->omega_t || !m->nu_t)
        return ctx->fail(PFFRG_E_ARGS, "mesh view has null arrays");
    if (m->num_sigma < 2 || m->num_omega < 2 || m->num_nu < 2)
        return ctx->fail(PFFRG_E_ARGS, "meshes need at least two frequencies");
    if (m->num_sigma > kMaxMesh || m->num_omega > kMaxMesh || m->num_nu > kMaxMesh)
        return ctx->fail(PFFRG_E_LIMIT, "mesh longer than %d frequencies", kMaxMesh);
    return 0;
}

int upload_mesh(pffrg_ctx* ctx, const pffrg_mesh_view* m) {
    if (int rc = check_mesh(ctx, m)) return rc;
    if (m->num_sigma != ctx->L.Nsig || m->num_omega != ctx->L.NO || m->num_nu != ctx->L.Nn)
        return ctx->fail(PFFRG_E_ARGS, "mesh sizes differ from the context's");
    std::vector<double> h;
    h.insert(h.end(), m->sigma, m->sigma + m->num_sigma);
    h.insert(h.end(), m->omega_s, m->omega_s + m->num_omega);
    h.insert(h.end(), m->nu_s, m->nu_s + m->num_nu);
    h.insert(h.end(), m->omega_t, m->omega_t + m->num_omega);
    h.insert(h.end(), m->nu_t, m->nu_t + m->num_nu);
    ctx->h_mesh = h;
    const std::vector<float> hf = mesh_block_ff(h, ctx->L.Nsig, ctx->L.NO, ctx->L.Nn);
    append_inverse_spacings(h, ctx->L.Nsig, ctx->L.NO, ctx->L.Nn);
    CK(cudaMemcpyAsync(ctx->mesh, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->mesh_ff, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

// Subdomain end points ξ^k a of integrate_log! (quadrature.jl:113-139) for every task
// frequency w1 of both bosonic meshes at cutoff Λ, with libm's pow as in the reference.
int upload_log_bounds(pffrg_ctx* ctx, double Lam, int eval) {
    const Layout& L = ctx->L;
    if (eval > ctx->bounds_cap) {
        CK(stream_free(ctx->st, ctx->log_bounds));
        ctx->log_bounds = nullptr;
        CK(cudaMalloc(&ctx->log_bounds, sizeof(double) * 2 * L.NO * (eval + 1)));
        ctx->bounds_cap = eval;
    }
    const double* Os = ctx->h_mesh.data() + L.Nsig;
    const double* ns = Os + L.NO;
    const double* Ot = ns + L.Nn;
    const double* nt = Ot + L.NO;
    std::vector<double>& hb = ctx->h_bounds;
    hb.assign((size_t)2 * L.NO * (eval + 1), 0.0);
    for (int m = 0; m < 2; ++m) {
        const double* Om = m ? Ot : Os;
        const double* nu = m ? nt : ns;
        const double val = Om[L.NO - 1] + nu[L.Nn - 1];
        for (int w1 = 0; w1 < L.NO; ++w1) {
            const double ref = Lam + 0.5 * Om[w1];
            const double a = 2.0 * ref, b = 1.0 * val;
            if (!(b > a)) continue;
            const double xi = std::pow(b / a, 1.0 / eval);
            double* o = hb.data() + (size_t)(m * L.NO + w1) * (eval + 1);
            for (int k = 0; k <= eval; ++k) o[k] = std::pow(xi, (double)k) * a;
        }
    }
    CK(cudaMemcpyAsync(ctx->log_bounds, hb.data(), sizeof(double) * hb.size(), cudaMemcpyHostToDevice, ctx->st));
    return 0;
}

// host view <-> device packed action (one copy per array, or one copy when packed)
int copy_view(pffrg_ctx* ctx, double* dev, const pffrg_action_view* v, bool to_device) {
    const Layout& L = ctx->L;
    if (!v || !v->sigma) return ctx->fail(PFFRG_E_ARGS, "action view has null arrays");
    auto kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    // packed fast path: every array at its packed offset from sigma
    bool packed = true;
    for (int c = 0; c < L.C && packed; ++c) {
        if (v->bare[c] != v->sigma + L.bare(c)) packed = false;
        for (int ch = 0; ch < 3 && packed; ++ch) {
            if (v->q1[c][ch] != v->sigma + L.qbase(c, ch, 0) || v->q2_1[c][ch] != v->sigma + L.qbase(c, ch, 1) ||
                v->q2_2[c][ch] != v->sigma + L.qbase(c, ch, 2) || v->q3[c][ch] != v->sigma + L.qbase(c, ch, 3))
                packed = false;
        }
    }
    if (packed) {
        if (to_device) CK(cudaMemcpyAsync(dev, v->sigma, sizeof(double) * L.total, kind, ctx->st));
        else CK(cudaMemcpyAsync(v->sigma, dev, sizeof(double) * L.total, kind, ctx->st));
        return 0;
    }
    auto cp = [&](double* host, int64_t off, int64_t n) -> int {
        if (!host) return ctx->fail(PFFRG_E_ARGS, "action view has a null array");
        if (to_device) CK(cudaMemcpyAsync(dev + off, host, sizeof(double) * n, kind, ctx->st));
        else CK(cudaMemcpyAsync(host, dev + off, sizeof(double) * n, kind, ctx->st));
        return 0;
    };
    if (int rc = cp(v->sigma, 0, L.Nsig)) return rc;
    for (int c = 0; c < L.C; ++c) {
        if (int rc = cp(v->bare[c], L.bare(c), L.Ns)) return rc;
        for (int ch = 0; ch < 3; ++ch) {
            if (int rc = cp(v->q1[c][ch], L.qbase(c, ch, 0), L.K1)) return rc;
            if (int rc = cp(v->q2_1[c][ch], L.qbase(c, ch, 1), L.K2)) return rc;
            if (int rc = cp(v->q2_2[c][ch], L.qbase(c, ch, 2), L.K2)) return rc;
            if (int rc = cp(v->q3[c][ch], L.qbase(c, ch, 3), L.K3)) return rc;
        }
    }
    return 0;
}

// make sure the wave workspace holds a pass of ntasks x nchan tasks at this eval
cudaError_t ensure_wave_space(pffrg_ctx* ctx, long long nsub) {
    const long long qcap = ctx->queue_cap_req > 0 ? ctx->queue_cap_req : ctx->queue_factor * nsub + 65536;
    if (nsub <= ctx->wave_nsub && ctx->wave_mem && (ctx->queue_cap_req <= 0 || qcap == ctx->wave_qcap))
        return cudaSuccess;
    if (ctx->wave_mem) {
        cudaError_t e = stream_free(ctx->st, ctx->wave_mem);
        if (e != cudaSuccess) return e;
        ctx->wave_mem = nullptr;
    }
    const size_t bytes = wave_space_bytes(nsub, ctx->L.Ns, qcap, ctx->L.C);
    cudaError_t e = cudaMalloc(&ctx->wave_mem, bytes);
    if (e != cudaSuccess) return e;
    ctx->wave_bytes = bytes;
    ctx->wave_nsub = nsub;
    ctx->wave_qcap = qcap;
    return cudaSuccess;
}

template <typename R>
cudaError_t launch_waves(pffrg_ctx* ctx, const PassArgs<R>& p) {
    const long long nsub = (long long)p.ntasks * p.nchan * (4 * p.eval + 1);
    cudaError_t e = ensure_wave_space(ctx, nsub);
    if (e != cudaSuccess) return e;
    WaveSpace W;
    wave_space_carve(W, ctx->wave_mem, nsub, ctx->L.Ns, ctx->wave_qcap, ctx->L.C);
    // this pass uses its own subdomain count; the queues keep the allocated capacity
    W.nsub = (int)nsub;
    ctx->h_wave_counters[7] = 0;
    e = launch_pass<R>(p, W, ctx->h_wave_counters, ctx->st);
    ctx->launches += ctx->h_wave_counters[7];  // the kernels of the pass
    if (e == cudaErrorLaunchOutOfResources && ctx->h_wave_counters[4]) ctx->queue_overflow = 1;
    return e;
}

// the FP64 action an FP32 copy of the mixed path was made from
const double* fp64_source(const pffrg_ctx* ctx, const float* y) {
    if (!y) return nullptr;
    for (int k = 0; k < 4; ++k)
        if (ctx->f_copy[k] == y) return ctx->f_src[k];
    return nullptr;
}

// One pass; on the mixed path the FP32 waves hand the subdomains whose Simpson decisions FP32
// rounding could flip to the same pass in FP64 on the FP64 actions, which also sums the results.
template <typename R>
cudaError_t launch_pass_all(pffrg_ctx* ctx, const PassArgs<R>& p0) {
    PassArgs<R> p = p0;
    // the FP64 Σ and dΣ of the propagators (node setup in FP64)
    if constexpr (sizeof(R) == 8) {
        p.prop_a64 = p.prop_a;
        p.prop_da64 = p.prop_da;
    } else {
        p.prop_a64 = fp64_source(ctx, p.prop_a);
        p.prop_da64 = fp64_source(ctx, p.prop_da);
        if ((p.prop_a && !p.prop_a64) || (p.prop_da && !p.prop_da64)) return cudaErrorInvalidValue;
    }
    if constexpr (sizeof(R) == 4) {
        if (ctx->esc_eps > 0.0) {
            static_assert(sizeof(PassArgs<float>) == sizeof(PassArgs<double>), "R appears only in pointers");
            PassArgs<float> p32 = p;
            p32.esc_mode = 1;
            p32.esc_eps = ctx->esc_eps;
            PassArgs<double> p64;
            std::memcpy(&p64, &p32, sizeof(p64));
            for (int k = 0; k < 4; ++k) {
                p64.src[k] = fp64_source(ctx, p32.src[k]);
                if (p32.src[k] && !p64.src[k]) return cudaErrorInvalidValue;
            }
            p64.prop_a = p32.prop_a64;
            p64.prop_da = p32.prop_da64;
            p64.esc_mode = 2;
            cudaError_t e = launch_waves<float>(ctx, p32);
            if (e != cudaSuccess) return e;
            return launch_waves<double>(ctx, p64);
        }
    }
    return launch_waves<R>(ctx, p);
}

// pass launch, bracketed by CUDA events on the context's stream when timing is on
template <typename R>
cudaError_t run_pass(pffrg_ctx* ctx, const PassArgs<R>& p) {
    ++ctx->pass_launches;  // the kernels of the pass are added to ctx->launches by launch_waves
    if (!ctx->timing) return launch_pass_all<R>(ctx, p);
    while ((int)ctx->ev.size() < 2 * (ctx->ev_used + 1)) {
        cudaEvent_t e;
        cudaError_t er = cudaEventCreate(&e);
        if (er != cudaSuccess) return er;
        ctx->ev.push_back(e);
    }
    cudaEvent_t e0 = ctx->ev[2 * ctx->ev_used], e1 = ctx->ev[2 * ctx->ev_used + 1];
    ++ctx->ev_used;
    cudaError_t er = cudaEventRecord(e0, ctx->st);
    if (er != cudaSuccess) return er;
    er = launch_pass_all<R>(ctx, p);
    if (er != cudaSuccess) return er;
    return cudaEventRecord(e1, ctx->st);
}

// accumulate the recorded pass durations (stream already synchronised)
int collect_pass_times(pffrg_ctx* ctx) {
    for (int k = 0; k < ctx->ev_used; ++k) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->ev[2 * k], ctx->ev[2 * k + 1]));
        ctx->pass_ms += ms;
    }
    ctx->ev_used = 0;
    return 0;
}

template <typename R>
PassArgs<R> base_pass(pffrg_ctx* ctx, double Lam, int eval, double atol, double rtol) {
    PassArgs<R> p;
    std::memset(&p, 0, sizeof(p));
    p.L = ctx->L;
    p.exch = ctx->lat.exch;
    p.ov_off = ctx->lat.ov_off;
    p.ov_rows = ctx->lat.ov_rows;
    p.rows_total = ctx->lat.rows;
    p.rows_in_smem = 0;
    p.rows_mode = ctx->rows_mode;
    p.mesh = ctx->mesh;
    p.mesh_ff = ctx->mesh_ff;
    p.log_bounds = ctx->log_bounds;
    p.corrs = ctx->corrs;
    p.Lam = Lam;
    p.eval = eval;
    p.atol = atol;
    p.rtol = rtol;
    p.twoS = 2.0 * ctx->S;
    p.nchan = 3;
    p.chan_of_y[0] = 1;  // t-channel CTAs (the heaviest) first
    p.chan_of_y[1] = 0;
    p.chan_of_y[2] = 2;
    p.node_counter = ctx->counter;
    p.async_waves = ctx->async_waves;
    p.team_T = ctx->team_T;
    p.team_SPL = ctx->team_SPL;
    p.status = ctx->status;
    return p;
}

template <typename R>
void set_tasks(PassArgs<R>& p, pffrg_ctx* ctx, bool full) {
    p.tasks = full ? ctx->tasks_full : ctx->tasks_sym;
    p.ntasks = full ? ctx->n_full : ctx->n_sym;
}

// slot sources and, per channel X = s, t, u, the channels each slot reads
template <typename R>
void set_slots(PassArgs<R>& p, const R* s0, const R* s1, const R* s2, const R* s3, const int (&m)[3][4]) {
    p.src[0] = s0;
    p.src[1] = s1;
    p.src[2] = s2;
    p.src[3] = s3;
    for (int X = 0; X < 3; ++X)
        for (int k = 0; k < 4; ++k) p.mask[X][k] = m[X][k];
}

// Katanin kernels (flow_su2_{s,t,u}.jl:2-55): every slot reads all channels
constexpr int kMaskKat[3][4] = {{CH_ALL, CH_ALL, CH_ALL, CH_ALL}, {CH_ALL, CH_ALL, CH_ALL, CH_ALL},
                                {CH_ALL, CH_ALL, CH_ALL, CH_ALL}};
// left kernels (flow_su2_s.jl:57-109, flow_su2_t.jl:89-173, flow_su2_u.jl:57-109) and the parquet BSE
// kernels (BSE_su2_{s,t,u}.jl): slot 1 without the own channel, t-channel slot 3 without u
constexpr int kMaskLeft[3][4] = {{CH_T | CH_U, CH_ALL, CH_ALL, CH_ALL},
                                 {CH_S | CH_U, CH_ALL, CH_S | CH_T, CH_ALL},
                                 {CH_S | CH_T, CH_ALL, CH_ALL, CH_ALL}};
// central kernels (flow_su2_s.jl:112-159, flow_su2_t.jl:176-255, flow_su2_u.jl:112-159): slot 2 only
// the own channel of da_l, t-channel slot 4 only its u channel
constexpr int kMaskCentral[3][4] = {{CH_ALL, CH_S, CH_ALL, CH_ALL},
                                    {CH_ALL, CH_T, CH_ALL, CH_U},
                                    {CH_ALL, CH_U, CH_ALL, CH_ALL}};
// reduced s bubble (SDE_su2.jl:2-42): slot 1 is the bare vertex
constexpr int kMaskReduced[3][4] = {{0, CH_ALL, CH_ALL, CH_ALL}, {0, CH_ALL, CH_ALL, CH_ALL},
                                    {0, CH_ALL, CH_ALL, CH_ALL}};

// typed views of the vertex sources: FP64 uses the action itself, FP32 its converted copy
template <typename R>
struct Src {
    const R* a;
    const R* da;
    const R* dal;
    const R* dtemp;
};

// Gauss-Kronrod segment scratch for `slots` integrals at the context's capacity
int ensure_gk(pffrg_ctx* ctx, long long slots) {
    if (ctx->gk_cap == 0) ctx->gk_cap = kGkCap0;
    if (ctx->gk_seg && slots <= ctx->gk_slots) return 0;
    slots = std::max(slots, ctx->gk_slots);
    CK(stream_free(ctx->st, ctx->gk_seg));
    ctx->gk_seg = nullptr;
    CK(cudaMalloc(&ctx->gk_seg, sizeof(double) * 4 * (size_t)ctx->gk_cap * (size_t)slots));
    ctx->gk_slots = slots;
    return 0;
}

// after a Gauss-Kronrod overflow: 8x the segments per integral (up to QuadGK's evaluation cap)
bool grow_gk(pffrg_ctx* ctx) {
    if (!ctx->gk_overflow || ctx->gk_cap >= kGkCapMax) return false;
    ctx->gk_overflow = 0;
    ctx->gk_cap = std::min(ctx->gk_cap * 8, kGkCapMax);
    stream_free(ctx->st, ctx->gk_seg);
    ctx->gk_seg = nullptr;
    return true;
}

// after a chunk-queue overflow of the default-sized queue: 4x the chunks per subdomain (up to 128;
// a queue size the caller set with pffrg_set_capacities is kept)
bool grow_queue(pffrg_ctx* ctx) {
    if (!ctx->queue_grow || ctx->queue_cap_req > 0 || ctx->queue_factor >= 128) return false;
    ctx->queue_grow = 0;
    ctx->queue_factor *= 4;
    ctx->wave_nsub = 0;  // the next pass allocates the bigger queue
    return true;
}

template <typename R>
int corrs_run(pffrg_ctx* ctx, int kind, double Lam, const R* a, const R* da, double atol, double rtol,
              double* out) {
    if (int rc = ensure_gk(ctx, 6ll * ctx->L.NO)) return rc;
    CorrsArgs<R> c;
    c.NO = ctx->L.NO;
    c.Nn = ctx->L.Nn;
    c.Nsig = ctx->L.Nsig;
    c.kind = kind;
    c.a = a;
    c.da = da;
    c.mesh = ctx->mesh;
    c.Lam = Lam;
    c.atol = atol;
    c.rtol = rtol;
    c.corrs = out;
    c.seg = ctx->gk_seg;
    c.seg_cap = ctx->gk_cap;
    c.status = ctx->status;
    ++ctx->launches;
    CK(launch_corrs<R>(c, ctx->st));
    return 0;
}

template <typename R>
int sigma_run(pffrg_ctx* ctx, int kind, double Lam, const R* a, const R* aux, double* out, double atol,
              double rtol) {
    if (int rc = ensure_gk(ctx, ctx->L.Nsig)) return rc;
    SigmaArgs<R> s;
    s.L = ctx->L;
    s.kind = kind;
    s.a = a;
    s.aux = aux;
    s.out = out;
    s.exch = ctx->lat.exch;
    s.mult = ctx->lat.mult;
    s.mesh = ctx->mesh;
    s.Lam = Lam;
    s.atol = atol;
    s.rtol = rtol;
    s.twoS = 2.0 * ctx->S;
    s.seg = ctx->gk_seg;
    s.seg_cap = ctx->gk_cap;
    s.status = ctx->status;
    ++ctx->launches;
    CK(launch_sigma<R>(s, ctx->st));
    return 0;
}

// FP32 copy of an action for the mixed passes (SU(2): the pair layout of Layout::pq); the FP64
// source is remembered for the FP64 hand-off pass.  `plain` keeps the FP64 layout (the FP32 χ
// integrand reads it).
int to_f(pffrg_ctx* ctx, const double* x, float* y, bool plain = false) {
    for (int k = 0; k < 4; ++k)
        if (ctx->f_copy[k] == y || !ctx->f_copy[k]) {
            ctx->f_copy[k] = y;
            ctx->f_src[k] = x;
            break;
        }
    ++ctx->launches;
    if (ctx->L.C == 2 && !plain) CK(launch_to_float_pairs(ctx->L, x, y, ctx->st));
    else CK(launch_to_float(x, y, ctx->L.total, ctx->st));
    return 0;
}

int check_status(pffrg_ctx* ctx) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, ctx->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (h) {
        CK(cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->st));
        if (h & 8) {
            ctx->queue_grow = 1;
            return ctx->fail(PFFRG_E_LIMIT, "quadrature chunk queue capacity exceeded");
        }
        if (h & ~16) {
            ctx->gk_overflow = 1;
            return ctx->fail(PFFRG_E_LIMIT, "adaptive Gauss-Kronrod segment capacity (%lld) exceeded", ctx->gk_cap);
        }
        return ctx->fail(PFFRG_E_NONFINITE, "the result holds NaN or infinite values (non-finite input state?)");
    }
    return 0;
}

// status bit 16 when the action holds a NaN or an infinity (read by check_status)
int check_finite(pffrg_ctx* ctx, const double* a) {
    ++ctx->launches;
    CK(launch_check_finite(a, ctx->L.total, ctx->status, ctx->st));
    return 0;
}

// compute_χ! (correlation_su2.jl:58-86, correlation_u1_dm.jl:152-190) on a
// device action.  Every (ω, site, component, box) integral starts with the
// region capacity it needed at the previous call (512 at the first); the
// integrals that run out of it are run again with 8x the capacity, up to the
// reference's bound of 10^7 integrand evaluations per cubature (10^7 / 34
// cuts).  The integrals that needed a cluster's capacity run on a second
// stream alongside the others, so the longest ones start first and the SMs
// their last waves leave idle take the small ones.  An integral's result
// does not depend on its capacity or on the stream.
int chi_dev(pffrg_ctx* ctx, double Lam, const double* a, const double* chi_mesh, int num_chi, double atol,
            double rtol, double* chi) {
    if (num_chi < 1 || !chi_mesh || !chi) return ctx->fail(PFFRG_E_ARGS, "empty correlation mesh or output");
    const int Ns = ctx->L.Ns;
    const int ncomp = ctx->L.C == 2 ? 1 : 3;  // χ, or χxx, χzz, χxy
    const long long njobs = 9ll * ncomp * Ns * num_chi;
    // a call that failed may have left integrals running on the second stream
    if (ctx->st_chi) CK(cudaStreamSynchronize(ctx->st_chi));
    if (num_chi > ctx->chi_n) {
        for (double** p : {&ctx->chi_mesh, &ctx->chi_box, &ctx->chi_out}) {
            CK(stream_free(ctx->st, *p));
            *p = nullptr;
        }
        for (int** p : {&ctx->chi_jobs, &ctx->chi_over, &ctx->chi_ctl}) {
            CK(stream_free(ctx->st, *p));
            *p = nullptr;
        }
        CK(cudaMalloc(&ctx->chi_mesh, sizeof(double) * num_chi));
        CK(cudaMalloc(&ctx->chi_box, sizeof(double) * 9 * 3 * (size_t)Ns * num_chi));
        CK(cudaMalloc(&ctx->chi_out, sizeof(double) * 3 * (size_t)Ns * num_chi));
        CK(cudaMalloc(&ctx->chi_jobs, sizeof(int) * 9 * 3 * (size_t)Ns * num_chi));
        CK(cudaMalloc(&ctx->chi_over, sizeof(int) * 9 * 3 * (size_t)Ns * num_chi));
        CK(cudaMalloc(&ctx->chi_ctl, sizeof(int) * 4 * 9 * 3 * (size_t)Ns * num_chi));
        ctx->chi_n = num_chi;
    }
    CK(cudaMemcpyAsync(ctx->chi_mesh, chi_mesh, sizeof(double) * num_chi, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->st));
    ChiArgs c;
    c.L = ctx->L;
    c.a = a;
    c.af = nullptr;
    if (ctx->precision == PFFRG_MIXED && !ctx->chi_fp64) {
        // FP32 integrand on the FP32 copy (float-float node setup), cubature sums and errors in FP64
        if (int rc = to_f(ctx, a, ctx->f_a, true)) return rc;
        c.af = ctx->f_a;
    }
    c.mesh = ctx->mesh;
    c.chi_mesh = ctx->chi_mesh;
    c.mesh_ff = ctx->mesh_ff;
    c.num_chi = num_chi;
    c.ncomp = ncomp;
    c.exch = ctx->lat.exch;
    c.Lam = Lam;
    c.atol = atol;
    c.rtol = rtol;
    c.twoS = 2.0 * ctx->S;
    c.box_out = ctx->chi_box;
    c.chi = ctx->chi_out;
    c.status = ctx->status;
    c.evals = ctx->counter + 2;  // [2..5] of the context's counters
    CK(cudaMemsetAsync(c.evals, 0, 4 * sizeof(unsigned long long), ctx->st));
    const long long cap_max = 10000000 / 34 + 2;
    const size_t budget = (size_t)16 << 30;  // region records of one launch (each stream)
    const size_t rec = 10 * sizeof(double) + 4 * sizeof(int);
    // capacity ladder: 512, 4096, 32768, 262144 regions, then the bound of 10^7 evaluations; an
    // integral that outgrows a capacity starts again from its first region with the next one
    auto next_cap = [&](long long cap) { return cap * 64 > cap_max ? cap_max : cap * 8; };
    auto cap_for = [&](long long n) {
        long long cap = 512;
        while (cap < n && cap < cap_max) cap = next_cap(cap);
        return cap;
    };
    // every integral starts at the capacity it needed at the previous call on the same jobs (with
    // a quarter's room to grow): a flow measures χ after every step, on a state that changes
    // little, so the integrals that need clusters are known before they are run
    if ((long long)ctx->chi_need.size() != njobs) ctx->chi_need.assign(njobs, 512);
    auto record = [&](int job, int ov) { ctx->chi_need[job] = cap_for((long long)(-ov) + (-ov) / 4); };
    auto ensure_reg = [&](double*& reg, int*& split, size_t& bytes, cudaStream_t st, long long cap,
                          long long batch) -> int {
        const size_t need = (size_t)cap * rec * (size_t)batch;
        if (need <= bytes) return 0;
        CK(stream_free(st, reg));
        CK(stream_free(st, split));
        reg = nullptr;
        split = nullptr;
        bytes = 0;
        CK(cudaMalloc(&reg, sizeof(double) * 10 * (size_t)cap * batch));
        CK(cudaMalloc(&split, sizeof(int) * 4 * (size_t)cap * batch));
        bytes = need;
        return 0;
    };
    auto launch = [&](ChiArgs cc, const int* jobs_dev, int nb, int* over_dev, long long cap, cudaStream_t st) -> int {
        ++ctx->launches;
        // the integrals that need large capacities are few and long: a cluster of blocks evaluates
        // each round's regions of one integral
        const int cl = cap >= ctx->chi_cluster_min ? ctx->chi_cluster_blocks : 1;
        cc.cap = cap;
        cudaError_t le = launch_chi_boxes(cc, jobs_dev, nb, over_dev, cl, st);
        if (le != cudaSuccess && cl > 8) {
            // a 16-block cluster did not launch (non-portable size): clusters of 8 from now on
            // (measured on the GB300: 16-block clusters were 20-30 % slower than 8, so 8 is the default)
            cudaGetLastError();
            ctx->chi_cluster_blocks = 8;
            le = launch_chi_boxes(cc, jobs_dev, nb, over_dev, 8, st);
        }
        CK(le);
        return 0;
    };
    // 1. the integrals that needed a cluster last time: one launch per capacity on the second
    //    stream, their overflow words read after the rest
    std::vector<std::vector<int>> big(8);
    std::vector<long long> big_cap(8, 0);
    std::vector<int> todo;
    for (long long j = 0; j < njobs; ++j) {
        const long long cap = ctx->chi_need[j];
        if (cap < ctx->chi_cluster_min) {
            todo.push_back((int)j);
            continue;
        }
        int level = 0;
        for (long long c2 = 512; c2 < cap; c2 = next_cap(c2)) ++level;
        big[level].push_back((int)j);
        big_cap[level] = cap;
    }
    std::vector<int> big_jobs;  // in launch order, each launch's words at its offset
    std::vector<long long> big_cap_of;
    for (int l = 7; l >= 0; --l)
        for (int j : big[l]) {
            big_jobs.push_back(j);
            big_cap_of.push_back(big_cap[l]);
        }
    if (!big_jobs.empty()) {
        if (!ctx->st_chi) {
            CK(cudaStreamCreateWithFlags(&ctx->st_chi, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&ctx->ev_chi, cudaEventDisableTiming));
        }
        if (!ctx->chi_jobs2 || ctx->chi_n2 < njobs) {
            for (int** q : {&ctx->chi_jobs2, &ctx->chi_over2, &ctx->chi_ctl2}) {
                CK(stream_free(ctx->st_chi, *q));
                *q = nullptr;
            }
            CK(cudaMalloc(&ctx->chi_jobs2, sizeof(int) * (size_t)njobs));
            CK(cudaMalloc(&ctx->chi_over2, sizeof(int) * (size_t)njobs));
            CK(cudaMalloc(&ctx->chi_ctl2, sizeof(int) * 4 * (size_t)njobs));
            ctx->chi_n2 = njobs;
        }
        long long reg_cap = 0, reg_batch = 0;
        for (size_t k = 0; k < big_jobs.size();) {
            size_t e = k;
            while (e < big_jobs.size() && big_cap_of[e] == big_cap_of[k]) ++e;
            const long long cap = big_cap_of[k];
            const long long batch = std::max<long long>(1, std::min<long long>((long long)(e - k),
                                                                               (long long)(budget / (cap * rec))));
            if ((size_t)cap * batch > (size_t)reg_cap * reg_batch) reg_cap = cap, reg_batch = batch;
            k = e;
        }
        if (int rc = ensure_reg(ctx->chi_reg2, ctx->chi_split2, ctx->chi_reg_bytes2, ctx->st_chi, reg_cap, reg_batch))
            return rc;
        // the second stream starts after the inputs of this call (mesh, status, counters, FP32 copy)
        CK(cudaEventRecord(ctx->ev_chi, ctx->st));
        CK(cudaStreamWaitEvent(ctx->st_chi, ctx->ev_chi, 0));
        CK(cudaMemcpyAsync(ctx->chi_jobs2, big_jobs.data(), sizeof(int) * big_jobs.size(), cudaMemcpyHostToDevice,
                           ctx->st_chi));
        ChiArgs c2 = c;
        c2.reg = ctx->chi_reg2;
        c2.reg_split = ctx->chi_split2;
        c2.ctl = ctx->chi_ctl2;
        for (size_t k = 0; k < big_jobs.size();) {
            const long long cap = big_cap_of[k];
            size_t e = k;
            while (e < big_jobs.size() && big_cap_of[e] == cap) ++e;
            const long long batch = std::max<long long>(1, (long long)(budget / (cap * rec)));
            for (size_t b = k; b < e; b += (size_t)batch) {
                const int nb = (int)std::min<size_t>((size_t)batch, e - b);
                if (int rc = launch(c2, ctx->chi_jobs2 + b, nb, ctx->chi_over2 + b, cap, ctx->st_chi)) return rc;
            }
            k = e;
        }
    }
    // 2. the rest on the context's stream, up the ladder from their capacities
    std::vector<int> over;
    long long cap = 512;
    for (int j : todo) cap = std::max(cap, ctx->chi_need[j]);
    auto run_ladder = [&](std::vector<int>& jobs, long long cap) -> int {
        while (!jobs.empty()) {
            const long long batch = std::max<long long>(1, std::min<long long>((long long)jobs.size(),
                                                                               (long long)(budget / (cap * rec))));
            if (int rc = ensure_reg(ctx->chi_reg, ctx->chi_split, ctx->chi_reg_bytes, ctx->st, cap, batch)) return rc;
            c.reg = ctx->chi_reg;
            c.reg_split = ctx->chi_split;
            c.ctl = ctx->chi_ctl;
            std::vector<int> next;
            for (size_t s0 = 0; s0 < jobs.size(); s0 += (size_t)batch) {
                const int nb = (int)std::min<size_t>((size_t)batch, jobs.size() - s0);
                CK(cudaMemcpyAsync(ctx->chi_jobs, jobs.data() + s0, sizeof(int) * nb, cudaMemcpyHostToDevice,
                                   ctx->st));
                if (int rc = launch(c, ctx->chi_jobs, nb, ctx->chi_over, cap, ctx->st)) return rc;
                over.resize(nb);
                CK(cudaMemcpyAsync(over.data(), ctx->chi_over, sizeof(int) * nb, cudaMemcpyDeviceToHost, ctx->st));
                CK(cudaStreamSynchronize(ctx->st));
                for (int q = 0; q < nb; ++q) {
                    if (over[q] > 0) next.push_back(jobs[s0 + q]);
                    else record(jobs[s0 + q], over[q]);
                }
            }
            jobs.swap(next);
            if (!jobs.empty()) {
                if (cap >= cap_max)
                    return ctx->fail(PFFRG_E_LIMIT, "cubature of χ needs more than %lld regions", cap_max);
                cap = next_cap(cap);
            }
        }
        return 0;
    };
    // the small integrals all start at the largest of their remembered capacities (a launch has
    // one capacity; an integral's result does not depend on it)
    if (int rc = run_ladder(todo, cap)) return rc;
    // 3. the second stream's integrals: those that outgrew their capacity go up the ladder here
    if (!big_jobs.empty()) {
        CK(cudaStreamSynchronize(ctx->st_chi));
        over.resize(big_jobs.size());
        CK(cudaMemcpy(over.data(), ctx->chi_over2, sizeof(int) * big_jobs.size(), cudaMemcpyDeviceToHost));
        std::vector<std::vector<int>> grow(8);
        for (size_t k = 0; k < big_jobs.size(); ++k) {
            if (over[k] <= 0) {
                record(big_jobs[k], over[k]);
                continue;
            }
            if (big_cap_of[k] >= cap_max)
                return ctx->fail(PFFRG_E_LIMIT, "cubature of χ needs more than %lld regions", cap_max);
            int level = 0;
            for (long long c2 = 512; c2 < next_cap(big_cap_of[k]); c2 = next_cap(c2)) ++level;
            grow[level].push_back(big_jobs[k]);
        }
        for (int l = 0; l < 8; ++l) {
            if (grow[l].empty()) continue;
            long long cl = 512;
            for (int q = 0; q < l; ++q) cl = next_cap(cl);
            if (int rc = run_ladder(grow[l], cl)) return rc;
        }
    }
    for (;;) {
        if (int rc = ensure_gk(ctx, num_chi)) return rc;
        c.seg = ctx->gk_seg;
        c.seg_cap = ctx->gk_cap;
        ++ctx->launches;
        CK(launch_chi_sum(c, ctx->st));
        int h = 0;
        CK(cudaMemcpyAsync(&h, ctx->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        if (!h) break;
        CK(cudaMemsetAsync(ctx->status, 0, sizeof(int), ctx->st));
        ctx->gk_overflow = 1;
        if (!grow_gk(ctx))
            return ctx->fail(PFFRG_E_LIMIT, "adaptive Gauss-Kronrod segment capacity exceeded in χ");
    }
    CK(cudaMemcpyAsync(chi, ctx->chi_out, sizeof(double) * ncomp * (size_t)Ns * num_chi, cudaMemcpyDeviceToHost,
                       ctx->st));
    unsigned long long ev[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(ev, c.evals, sizeof(ev), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->chi_evals = (int64_t)ev[0];
    ctx->chi_regions_max = (int64_t)ev[1];
    ctx->chi_rounds = (int64_t)ev[2];
    ctx->chi_rounds_max = (int64_t)ev[3];
    return 0;
}

// compute_dΣ! on device actions.  The Gauss-Kronrod integrals run in FP64 on both paths: their
// adaptive bisection stops on |K15 - G7|, which FP32 rounding of the integrand keeps above the
// tolerance at small Λ (the segments then grow to the capacity limit)
int dsigma_dev(pffrg_ctx* ctx, double Lam, const double* a, double* da, double atol, double rtol) {
    return sigma_run<double>(ctx, SIG_FLOW, Lam, a, nullptr, da, atol, rtol);
}

// compute_dΓ_{1l,2l,ml}! (+ compute_dΣ_corr!) on device actions
template <typename R>
int dgamma_dev(pffrg_ctx* ctx, int loops, double Lam, const double* a, double* da, int eval, double gatol,
               double grtol, int sigma_corr, double satol, double srtol) {
    const Layout& L = ctx->L;
    Src<R> s;
    if constexpr (sizeof(R) == 8) {
        s.a = (const R*)a;
        s.da = (const R*)da;
        s.dal = (const R*)ctx->da_l;
        s.dtemp = (const R*)ctx->da_temp;
    } else {
        if (int rc = to_f(ctx, a, ctx->f_a)) return rc;
        if (int rc = to_f(ctx, da, ctx->f_da)) return rc;  // dΣ for the Katanin propagator
        s.a = (const R*)ctx->f_a;
        s.da = (const R*)ctx->f_da;
        s.dal = (const R*)ctx->f_dal;
        s.dtemp = (const R*)ctx->f_dtemp;
    }
    CK(cudaMemsetAsync(ctx->counter, 0, 2 * sizeof(unsigned long long), ctx->st));
    if (int rc = upload_log_bounds(ctx, Lam, eval)) return rc;
    // 1 loop (compute.jl:57-112)
    if (int rc = corrs_run<double>(ctx, PROP_KAT, Lam, a, da, gatol, grtol, ctx->corrs)) return rc;
    {
        PassArgs<R> p = base_pass<R>(ctx, Lam, eval, gatol, grtol);
        set_tasks(p, ctx, false);
        set_slots<R>(p, s.a, s.a, s.a, s.a, kMaskKat);
        p.prop_kind = PROP_KAT;
        p.prop_a = s.a;
        p.prop_da = s.da;
        p.out = da;
        CK_PASS(run_pass<R>(ctx, p));
        CK((++ctx->launches, launch_symmetrize)(L, ctx->lat.exch, da, ctx->st));
    }
    if (loops >= 2) {
        // 2 loop (compute.jl:115-174)
        if constexpr (sizeof(R) == 4) {
            if (int rc = to_f(ctx, da, ctx->f_da)) return rc;
        }
        if (int rc = corrs_run<double>(ctx, PROP_PLAIN, Lam, a, a, gatol, grtol, ctx->corrs)) return rc;
        PassArgs<R> p = base_pass<R>(ctx, Lam, eval, gatol, grtol);
        set_tasks(p, ctx, true);
        set_slots<R>(p, s.da, s.a, s.da, s.a, kMaskLeft);
        p.prop_kind = PROP_PLAIN;
        p.prop_a = s.a;
        p.prop_da = s.a;
        p.out = ctx->da_l;
        CK_PASS(run_pass<R>(ctx, p));
        CK((++ctx->launches, launch_symmetrize_add_to)(L, ctx->lat.exch, ctx->da_l, da, ctx->st));
    }
    if (loops >= 3) {
        // multiloop (compute.jl:177-287)
        CK((++ctx->launches, launch_axpby)(L, 0.0, nullptr, 0.0, ctx->da_temp, false, true, ctx->st));
        CK((++ctx->launches, launch_axpby)(L, 0.0, nullptr, 0.0, ctx->da_sig, false, true, ctx->st));
        CK((++ctx->launches, launch_symmetrize_add_to)(L, ctx->lat.exch, ctx->da_l, ctx->da_temp, ctx->st));
        for (int loop = 3; loop <= loops; ++loop) {
            if constexpr (sizeof(R) == 4) {
                if (int rc = to_f(ctx, ctx->da_l, ctx->f_dal)) return rc;
                if (int rc = to_f(ctx, ctx->da_temp, ctx->f_dtemp)) return rc;
            }
            {
                // central kernels (flow_su2_s.jl:112-159, t :176-255, u :112-159)
                PassArgs<R> p = base_pass<R>(ctx, Lam, eval, gatol, grtol);
                set_tasks(p, ctx, false);
                p.prop_kind = PROP_PLAIN;
                p.prop_a = s.a;
                p.prop_da = s.a;
                p.out = ctx->da_c;
                set_slots<R>(p, s.a, s.dal, s.a, s.dal, kMaskCentral);
                CK_PASS(run_pass<R>(ctx, p));
            }
            {
                PassArgs<R> p = base_pass<R>(ctx, Lam, eval, gatol, grtol);
                set_tasks(p, ctx, true);
                p.prop_kind = PROP_PLAIN;
                p.prop_a = s.a;
                p.prop_da = s.a;
                p.out = ctx->da_l;
                set_slots<R>(p, s.dtemp, s.a, s.dtemp, s.a, kMaskLeft);
                CK_PASS(run_pass<R>(ctx, p));
            }
            CK((++ctx->launches, launch_symmetrize)(L, ctx->lat.exch, ctx->da_c, ctx->st));
            CK(cudaMemcpyAsync(ctx->da_temp, ctx->da_c, sizeof(double) * L.total, cudaMemcpyDeviceToDevice, ctx->st));
            CK((++ctx->launches, launch_symmetrize_add_to)(L, ctx->lat.exch, ctx->da_l, ctx->da_temp, ctx->st));
            CK((++ctx->launches, launch_axpby)(L, 1.0, ctx->da_c, 1.0, ctx->da_sig, false, true, ctx->st));
            CK((++ctx->launches, launch_axpby)(L, 1.0, ctx->da_temp, 1.0, da, false, true, ctx->st));
        }
        if (sigma_corr) {
            // compute_dΣ_corr! (flow_self.jl:23-51), in FP64 on both paths
            if (int rc = sigma_run<double>(ctx, SIG_CORR1, Lam, a, ctx->da_sig, ctx->da_sig, satol, srtol)) return rc;
            CK(cudaMemsetAsync(ctx->sig_tmp, 0, sizeof(double) * L.Nsig, ctx->st));
            if (int rc = sigma_run<double>(ctx, SIG_CORR2, Lam, a, ctx->da_sig, ctx->sig_tmp, satol, srtol)) return rc;
            // da.Σ += da_Σ.Σ + corr2 (index 0 included: both are zero there)
            CK((++ctx->launches, launch_axpby)(L, 1.0, ctx->da_sig, 1.0, da, true, false, ctx->st));
            CK((++ctx->launches, launch_axpby)(L, 1.0, ctx->sig_tmp, 1.0, da, true, false, ctx->st));
        }
    }
    return 0;
}

int rhs_dev(pffrg_ctx* ctx, int loops, double Lam, const double* a, double* da, int eval, double gatol,
            double grtol, double satol, double srtol, int sigma_corr) {
    int rc = dsigma_dev(ctx, Lam, a, da, satol, srtol);
    if (rc) return rc;
    rc = ctx->precision == PFFRG_FP64
             ? dgamma_dev<double>(ctx, loops, Lam, a, da, eval, gatol, grtol, sigma_corr, satol, srtol)
             : dgamma_dev<float>(ctx, loops, Lam, a, da, eval, gatol, grtol, sigma_corr, satol, srtol);
    if (rc) return rc;
    return check_finite(ctx, da);
}

int read_evals(pffrg_ctx* ctx) {
    unsigned long long h[2] = {0, 0};
    CK(cudaMemcpyAsync(h, ctx->counter, sizeof(h), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->last_evals = (int64_t)h[0];
    ctx->last_alg_values = (int64_t)h[1];
    return collect_pass_times(ctx);
}

int absmax(pffrg_ctx* ctx, const double* a, double* dst) {
    ctx->launches += 2;
    CK(launch_absmax_q3(ctx->L, a, ctx->partial, kPartials, dst, ctx->st));
    return 0;
}

}  // namespace

// rerun a call whose Gauss-Kronrod integrals ran out of segments with 8x the capacity, or whose
// quadrature levels overflowed the default chunk queue with a 4x bigger queue
template <class Fn>
int gk_retry(pffrg_ctx* ctx, Fn fn) {
    for (;;) {
        const int rc = fn();
        if (rc != PFFRG_E_LIMIT || !ctx || !(grow_gk(ctx) || grow_queue(ctx))) return rc;
    }
}

extern "C" {

const char* pffrg_last_error(const pffrg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int64_t pffrg_action_size(const pffrg_ctx* ctx) { return ctx ? ctx->L.total : 0; }

int64_t pffrg_last_integrand_evals(const pffrg_ctx* ctx) { return ctx ? ctx->last_evals : 0; }

int pffrg_set_timing(pffrg_ctx* ctx, int on) {
    if (!ctx) return PFFRG_E_ARGS;
    ctx->timing = on ? 1 : 0;
    return 0;
}

int pffrg_read_stats(pffrg_ctx* ctx, pffrg_stats* out, int reset) {
    if (!ctx || !out) return PFFRG_E_ARGS;
    out->integrand_evals = ctx->last_evals;
    out->algorithmic_values = ctx->last_alg_values;
    out->pass_ms = ctx->pass_ms;
    out->rhs_ms = ctx->rhs_ms;
    out->pass_launches = ctx->pass_launches;
    out->launches = ctx->launches;
    out->chi_evals = ctx->chi_evals;
    out->chi_regions_max = ctx->chi_regions_max;
    out->chi_rounds = ctx->chi_rounds;
    out->chi_rounds_max = ctx->chi_rounds_max;
    if (reset) {
        ctx->pass_ms = ctx->rhs_ms = 0.0;
        ctx->pass_launches = ctx->launches = 0;
    }
    return 0;
}

void pffrg_destroy(pffrg_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    if (ctx->st_chi) cudaStreamSynchronize(ctx->st_chi);
    void* ptrs[] = {ctx->lat.exch, ctx->lat.mult, ctx->lat.ov_off, ctx->lat.ov_rows, ctx->wave_mem,
                    ctx->mesh, ctx->log_bounds, ctx->da_l, ctx->da_c, ctx->da_temp, ctx->da_sig, ctx->sig_tmp, ctx->f_a, ctx->f_da,
                    ctx->f_dal, ctx->f_dtemp, ctx->corrs, ctx->corrs_sde, ctx->partial, ctx->scalars, ctx->status,
                    ctx->counter, ctx->tasks_sym, ctx->tasks_full, ctx->tasks_red, ctx->chi_reg, ctx->chi_split,
                    ctx->chi_box, ctx->chi_out, ctx->chi_mesh, ctx->chi_jobs, ctx->chi_over, ctx->chi_ctl, ctx->gk_seg,
                    ctx->mesh_new, ctx->mesh_ff, ctx->scan_arg, ctx->scan_cuts, ctx->chi_reg2, ctx->chi_split2,
                    ctx->chi_jobs2, ctx->chi_over2, ctx->chi_ctl2};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (int k = 0; k < PFFRG_NUM_SLOTS; ++k)
        if (ctx->slot[k]) cudaFree(ctx->slot[k]);
    if (ctx->h_scalars) cudaFreeHost(ctx->h_scalars);
    if (ctx->h_wave_counters) cudaFreeHost(ctx->h_wave_counters);
    for (cudaEvent_t e : ctx->ev) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->rhs_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->ev_chi) cudaEventDestroy(ctx->ev_chi);
    if (ctx->st_chi) cudaStreamDestroy(ctx->st_chi);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
}

pffrg_ctx* pffrg_create(const pffrg_lattice_view* lat, const pffrg_mesh_view* mesh, int symmetry, double S,
                        int precision, int device) {
    g_create_error.clear();
    if (!lat || !mesh || !lat->exchange || !lat->mult || !lat->overlap_offsets || lat->num_sites <= 0) {
        g_create_error = "invalid lattice view";
        return nullptr;
    }
    if (symmetry != PFFRG_SU2 && symmetry != PFFRG_U1_DM) {
        g_create_error = "unknown symmetry";
        return nullptr;
    }
    if (precision != PFFRG_FP64 && precision != PFFRG_MIXED) {
        g_create_error = "unknown precision";
        return nullptr;
    }
    if (lat->num_sites > 256) {
        g_create_error = "more than 256 irreducible sites";
        return nullptr;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= device || device < 0) {
        g_create_error = std::string("no usable CUDA device: ") + cudaGetErrorString(e);
        return nullptr;
    }
    pffrg_ctx* ctx = new pffrg_ctx();
    ctx->device = device;
    ctx->symmetry = symmetry;
    ctx->S = S;
    ctx->precision = precision;
    auto bail = [&](const std::string& msg) -> pffrg_ctx* {
        g_create_error = msg;
        pffrg_destroy(ctx);
        return nullptr;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail("cudaSetDevice failed");
    if (check_mesh(ctx, mesh)) return bail(ctx->err);
    const int Ns = (int)lat->num_sites;
    ctx->L = make_layout(Ns, (int)mesh->num_sigma, (int)mesh->num_omega, (int)mesh->num_nu,
                         symmetry == PFFRG_SU2 ? 2 : 6);
    const Layout& L = ctx->L;
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) return bail("stream creation failed");

    // lattice tables (0-based on the device)
    std::vector<int> exch(Ns), mult(Ns), off(Ns + 1);
    for (int i = 0; i < Ns; ++i) {
        exch[i] = (int)lat->exchange[i] - 1;
        mult[i] = (int)lat->mult[i];
        if (exch[i] < 0 || exch[i] >= Ns) return bail("exchange table out of range");
    }
    for (int i = 0; i <= Ns; ++i) off[i] = (int)lat->overlap_offsets[i];
    const int64_t R = off[Ns];
    std::vector<unsigned> rows(R > 0 ? R : 1);
    for (int64_t j = 0; j < R; ++j) {
        const int64_t a = lat->overlap_rows[3 * j] - 1, b = lat->overlap_rows[3 * j + 1] - 1;
        const int64_t mm = lat->overlap_rows[3 * j + 2];
        if (a < 0 || a >= Ns || b < 0 || b >= Ns) return bail("overlap table out of range");
        if (mm < 0 || mm >= 65536) return bail("overlap multiplicity out of range");
        rows[j] = (unsigned)a | ((unsigned)b << 8) | ((unsigned)mm << 16);
    }
    for (int i = 0; i < Ns; ++i)
        if (off[i] > off[i + 1] || off[i] < 0) return bail("overlap offsets not increasing");
    ctx->lat.Ns = Ns;
    ctx->lat.rows = R;
    auto dalloc = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes > 0 ? bytes : 8) == cudaSuccess; };
    bool ok = dalloc((void**)&ctx->lat.exch, sizeof(int) * Ns) && dalloc((void**)&ctx->lat.mult, sizeof(int) * Ns) &&
              dalloc((void**)&ctx->lat.ov_off, sizeof(int) * (Ns + 1)) &&
              dalloc((void**)&ctx->lat.ov_rows, sizeof(unsigned) * rows.size()) &&
              dalloc((void**)&ctx->mesh, 2 * sizeof(double) * (L.Nsig + 2 * L.NO + 2 * L.Nn)) &&
              dalloc((void**)&ctx->mesh_ff, sizeof(float) * (3 * (L.Nsig + 2 * L.NO + 2 * L.Nn) + kMeshGuess)) &&
              dalloc((void**)&ctx->mesh_new, sizeof(double) * (L.Nsig + 2 * L.NO + 2 * L.Nn)) &&
              dalloc((void**)&ctx->scan_arg, sizeof(long long) * 3 * L.C) &&
              dalloc((void**)&ctx->scan_cuts, sizeof(double) * 3 * L.C * (L.NO + 3 * L.Nn));
    for (int k = 0; k < PFFRG_NUM_SLOTS && ok; ++k) ok = dalloc((void**)&ctx->slot[k], sizeof(double) * L.total);
    ok = ok && dalloc((void**)&ctx->da_l, sizeof(double) * L.total) &&
         dalloc((void**)&ctx->da_c, sizeof(double) * L.total) &&
         dalloc((void**)&ctx->da_temp, sizeof(double) * L.total) &&
         dalloc((void**)&ctx->da_sig, sizeof(double) * L.total) &&
         dalloc((void**)&ctx->sig_tmp, sizeof(double) * L.Nsig) &&
         dalloc((void**)&ctx->f_a, sizeof(float) * (L.total + 2)) &&
         dalloc((void**)&ctx->f_da, sizeof(float) * (L.total + 2)) &&
         dalloc((void**)&ctx->f_dal, sizeof(float) * (L.total + 2)) &&
         dalloc((void**)&ctx->f_dtemp, sizeof(float) * (L.total + 2)) &&
         dalloc((void**)&ctx->corrs, sizeof(double) * 6 * L.NO) &&
         dalloc((void**)&ctx->corrs_sde, sizeof(double) * 6 * L.NO) &&
         dalloc((void**)&ctx->partial, sizeof(double) * kPartials) &&
         dalloc((void**)&ctx->scalars, sizeof(double) * 4) && dalloc((void**)&ctx->status, sizeof(int)) &&
         dalloc((void**)&ctx->counter, 6 * sizeof(unsigned long long));
    if (!ok) return bail("device allocation failed");
    if (cudaHostAlloc((void**)&ctx->h_scalars, sizeof(double) * 4, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc((void**)&ctx->h_wave_counters, sizeof(int) * 8, cudaHostAllocDefault) != cudaSuccess)
        return bail("pinned allocation failed");
    std::vector<int4> ts = make_tasks(L.NO, L.Nn, 0), tf = make_tasks(L.NO, L.Nn, 1), tr = make_tasks(L.NO, L.Nn, 2);
    ctx->n_sym = (int)ts.size();
    ctx->n_full = (int)tf.size();
    ctx->n_red = (int)tr.size();
    ok = dalloc((void**)&ctx->tasks_sym, sizeof(int4) * ts.size()) &&
         dalloc((void**)&ctx->tasks_full, sizeof(int4) * tf.size()) &&
         dalloc((void**)&ctx->tasks_red, sizeof(int4) * tr.size());
    if (!ok) return bail("device allocation failed");
    cudaStream_t st = ctx->st;
    bool cp = cudaMemcpyAsync(ctx->lat.exch, exch.data(), sizeof(int) * Ns, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(ctx->lat.mult, mult.data(), sizeof(int) * Ns, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(ctx->lat.ov_off, off.data(), sizeof(int) * (Ns + 1), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(ctx->lat.ov_rows, rows.data(), sizeof(unsigned) * rows.size(), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(ctx->tasks_sym, ts.data(), sizeof(int4) * ts.size(), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(ctx->tasks_full, tf.data(), sizeof(int4) * tf.size(), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(ctx->tasks_red, tr.data(), sizeof(int4) * tr.size(), cudaMemcpyHostToDevice, st) == cudaSuccess;
    for (int k = 0; k < PFFRG_NUM_SLOTS && cp; ++k)
        cp = cudaMemsetAsync(ctx->slot[k], 0, sizeof(double) * L.total, st) == cudaSuccess;
    double* scr[] = {ctx->da_l, ctx->da_c, ctx->da_temp, ctx->da_sig};
    for (double* p : scr)
        if (cp) cp = cudaMemsetAsync(p, 0, sizeof(double) * L.total, st) == cudaSuccess;
    cp = cp && cudaMemsetAsync(ctx->status, 0, sizeof(int), st) == cudaSuccess &&
         cudaMemsetAsync(ctx->corrs_sde, 0, sizeof(double) * 6 * L.NO, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
    if (!cp) return bail("device initialisation failed");
    // hand the ABI's pinned copies of the 1-based tables back: nothing else to keep
    if (upload_mesh(ctx, mesh)) return bail(ctx->err);
    // Gauss-Kronrod scratch for the largest launch of the right-hand side (dΣ or the boundary
    // corrections), so that it is not reallocated between kernels of one call
    if (ensure_gk(ctx, std::max<long long>(L.Nsig, 6ll * L.NO))) return bail(ctx->err);
    return ctx;
}

int pffrg_set_mesh(pffrg_ctx* ctx, const pffrg_mesh_view* mesh) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    return upload_mesh(ctx, mesh);
}

int pffrg_set_precision(pffrg_ctx* ctx, int precision) {
    if (!ctx) return PFFRG_E_ARGS;
    if (precision != PFFRG_FP64 && precision != PFFRG_MIXED) return ctx->fail(PFFRG_E_ARGS, "unknown precision %d", precision);
    ctx->precision = precision;
    return 0;
}

int pffrg_upload(pffrg_ctx* ctx, int slot, const pffrg_action_view* a) {
    if (!ctx || slot < 0 || slot >= PFFRG_NUM_SLOTS) return ctx ? ctx->fail(PFFRG_E_ARGS, "bad slot") : PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    if (int rc = copy_view(ctx, ctx->slot[slot], a, true)) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pffrg_download(pffrg_ctx* ctx, int slot, pffrg_action_view* a) {
    if (!ctx || slot < 0 || slot >= PFFRG_NUM_SLOTS) return ctx ? ctx->fail(PFFRG_E_ARGS, "bad slot") : PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    if (int rc = copy_view(ctx, ctx->slot[slot], a, false)) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

static int dsigma_once(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a, pffrg_action_view* da, double atol,
                 double rtol) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    if (int rc = copy_view(ctx, ctx->slot[PFFRG_SLOT_A], a, true)) return rc;
    if (int rc = copy_view(ctx, ctx->slot[PFFRG_SLOT_DA], da, true)) return rc;
    int rc = dsigma_dev(ctx, Lam, ctx->slot[PFFRG_SLOT_A], ctx->slot[PFFRG_SLOT_DA], atol, rtol);
    if (rc) return rc;
    if ((rc = check_finite(ctx, ctx->slot[PFFRG_SLOT_DA]))) return rc;
    if ((rc = check_status(ctx))) return rc;
    if ((rc = copy_view(ctx, ctx->slot[PFFRG_SLOT_DA], da, false))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pffrg_dsigma(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a, pffrg_action_view* da, double atol,
                 double rtol) {
    return gk_retry(ctx, [&] { return dsigma_once(ctx, Lam, a, da, atol, rtol); });
}

static int dgamma_once(pffrg_ctx* ctx, int loops, double Lam, const pffrg_action_view* a, pffrg_action_view* da, int eval,
                 double gatol, double grtol, int sigma_corr, double satol, double srtol) {
    if (!ctx) return PFFRG_E_ARGS;
    if (loops < 1 || eval < 1) return ctx->fail(PFFRG_E_ARGS, "loops and eval must be positive");
    CK(cudaSetDevice(ctx->device));
    if (int rc = copy_view(ctx, ctx->slot[PFFRG_SLOT_A], a, true)) return rc;
    if (int rc = copy_view(ctx, ctx->slot[PFFRG_SLOT_DA], da, true)) return rc;
    int rc = ctx->precision == PFFRG_FP64
                 ? dgamma_dev<double>(ctx, loops, Lam, ctx->slot[PFFRG_SLOT_A], ctx->slot[PFFRG_SLOT_DA], eval, gatol,
                                      grtol, sigma_corr, satol, srtol)
                 : dgamma_dev<float>(ctx, loops, Lam, ctx->slot[PFFRG_SLOT_A], ctx->slot[PFFRG_SLOT_DA], eval, gatol,
                                     grtol, sigma_corr, satol, srtol);
    if (rc) return rc;
    if ((rc = check_finite(ctx, ctx->slot[PFFRG_SLOT_DA]))) return rc;
    if ((rc = check_status(ctx))) return rc;
    if ((rc = read_evals(ctx))) return rc;
    if ((rc = copy_view(ctx, ctx->slot[PFFRG_SLOT_DA], da, false))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pffrg_dgamma(pffrg_ctx* ctx, int loops, double Lam, const pffrg_action_view* a, pffrg_action_view* da, int eval,
                 double gatol, double grtol, int sigma_corr, double satol, double srtol) {
    return gk_retry(ctx, [&] { return dgamma_once(ctx, loops, Lam, a, da, eval, gatol, grtol, sigma_corr, satol, srtol); });
}

static int rhs_once(pffrg_ctx* ctx, int loops, double Lam, int a_slot, int da_slot, int eval, double gatol,
              double grtol, double satol, double srtol, int sigma_corr) {
    if (!ctx) return PFFRG_E_ARGS;
    if (a_slot < 0 || a_slot >= PFFRG_NUM_SLOTS || da_slot < 0 || da_slot >= PFFRG_NUM_SLOTS || a_slot == da_slot)
        return ctx->fail(PFFRG_E_ARGS, "bad slots");
    if (loops < 1 || eval < 1) return ctx->fail(PFFRG_E_ARGS, "loops and eval must be positive");
    CK(cudaSetDevice(ctx->device));
    if (ctx->timing) {
        for (auto& e : ctx->rhs_ev)
            if (!e) CK(cudaEventCreate(&e));
        CK(cudaEventRecord(ctx->rhs_ev[0], ctx->st));
    }
    int rc = rhs_dev(ctx, loops, Lam, ctx->slot[a_slot], ctx->slot[da_slot], eval, gatol, grtol, satol, srtol,
                     sigma_corr);
    if (rc) return rc;
    if (ctx->timing) CK(cudaEventRecord(ctx->rhs_ev[1], ctx->st));
    if ((rc = check_status(ctx))) return rc;
    if ((rc = read_evals(ctx))) return rc;
    if (ctx->timing) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->rhs_ev[0], ctx->rhs_ev[1]));
        ctx->rhs_ms += ms;
    }
    return 0;
}

int pffrg_rhs(pffrg_ctx* ctx, int loops, double Lam, int a_slot, int da_slot, int eval, double gatol,
              double grtol, double satol, double srtol, int sigma_corr) {
    return gk_retry(ctx, [&] { return rhs_once(ctx, loops, Lam, a_slot, da_slot, eval, gatol, grtol, satol, srtol, sigma_corr); });
}

int pffrg_autotune_team_shape(pffrg_ctx* ctx, int loops, double Lam, int a_slot, int da_slot, int eval, double gatol,
                              double grtol, double satol, double srtol, int* lanes, int* sites_per_lane) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    const int Ns = ctx->L.Ns;
    static const int shapes[][2] = {{8, 1}, {16, 1}, {32, 1}, {16, 3}, {16, 4}, {32, 2}, {32, 3}, {32, 4}, {32, 8}};
    cudaEvent_t ev[2];
    CK(cudaEventCreate(&ev[0]));
    if (cudaEventCreate(&ev[1]) != cudaSuccess) {
        cudaEventDestroy(ev[0]);
        return ctx->fail(PFFRG_E_CUDA, "cudaEventCreate failed");
    }
    float best = 0.f;
    int bT = 0, bS = 0, rc = 0;
    for (const auto& sh : shapes) {
        const int cover = sh[0] * sh[1];
        if (cover < Ns || cover > std::max(2 * Ns, 8)) continue;  // shapes that leave at most half the lanes idle
        ctx->team_T = sh[0];
        ctx->team_SPL = sh[1];
        float ms = 0.f;
        for (int rep = 0; rep < 2 && !rc; ++rep) {  // the first right-hand side loads the shape's kernels
            cudaError_t e = cudaEventRecord(ev[0], ctx->st);
            if (e == cudaSuccess) rc = pffrg_rhs(ctx, loops, Lam, a_slot, da_slot, eval, gatol, grtol, satol, srtol, 0);
            if (e == cudaSuccess && !rc) e = cudaEventRecord(ev[1], ctx->st);
            if (e == cudaSuccess && !rc) e = cudaEventSynchronize(ev[1]);
            if (e == cudaSuccess && !rc) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
            if (e != cudaSuccess && !rc) rc = ctx->fail(PFFRG_E_CUDA, "timing failed: %s", cudaGetErrorString(e));
        }
        if (rc) break;
        if (!bT || ms < best) {
            best = ms;
            bT = sh[0];
            bS = sh[1];
        }
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    ctx->team_T = rc ? 0 : bT;
    ctx->team_SPL = rc ? 0 : bS;
    if (rc) return rc;
    if (!bT) return ctx->fail(PFFRG_E_ARGS, "no team shape is built for %d sites", Ns);
    if (lanes) *lanes = bT;
    if (sites_per_lane) *sites_per_lane = bS;
    return 0;
}

}  // extern "C"

namespace {

// compute_Σ! (SDE.jl:58-96) on device actions d1 -> d2: the boundary corrections (kept for the
// next BSE), the reduced s bubble (slot 1 is the bare vertex) and the SDE self energy
int sde_dev(pffrg_ctx* ctx, double Lam, double* d1, double* d2, int eval, double gatol, double grtol, double satol,
            double srtol) {
    auto run = [&](auto tag) -> int {
        using R = decltype(tag);
        const R* r1;
        if constexpr (sizeof(R) == 8) {
            r1 = (const R*)d1;
        } else {
            if (int rc = to_f(ctx, d1, ctx->f_a)) return rc;
            r1 = (const R*)ctx->f_a;
        }
        if (int rc = corrs_run<double>(ctx, PROP_PLAIN, Lam, d1, d1, gatol, grtol, ctx->corrs_sde)) return rc;
        if (int rc = upload_log_bounds(ctx, Lam, eval)) return rc;
        // reduced s bubble (SDE.jl:2-56): slot 1 is the bare vertex
        PassArgs<R> p = base_pass<R>(ctx, Lam, eval, gatol, grtol);
        p.tasks = ctx->tasks_red;
        p.ntasks = ctx->n_red;
        p.corrs = ctx->corrs_sde;
        p.nchan = 1;
        p.chan_of_y[0] = 0;
        set_slots<R>(p, r1, r1, r1, r1, kMaskReduced);
        p.reduced = 1;
        p.prop_kind = PROP_PLAIN;
        p.prop_a = r1;
        p.prop_da = r1;
        p.out = d2;
        CK_PASS(run_pass<R>(ctx, p));
        return sigma_run<double>(ctx, SIG_SDE, Lam, d1, d2, d2, satol, srtol);
    };
    int rc = ctx->precision == PFFRG_FP64 ? run(double{}) : run(float{});
    if (rc) return rc;
    return check_finite(ctx, d2);
}

// compute_Γ! (compute.jl:2-54) on device actions d1 -> d2 with the boundary corrections of the
// last SDE call
int bse_dev(pffrg_ctx* ctx, double Lam, double* d1, double* d2, int eval, double atol, double rtol) {
    auto run = [&](auto tag) -> int {
        using R = decltype(tag);
        const R* r1;
        if constexpr (sizeof(R) == 8) {
            r1 = (const R*)d1;
        } else {
            if (int rc = to_f(ctx, d1, ctx->f_a)) return rc;
            r1 = (const R*)ctx->f_a;
        }
        if (int rc = upload_log_bounds(ctx, Lam, eval)) return rc;
        // BSE kernels (BSE_su2_{s,t,u}.jl): slot 1 without the own channel
        PassArgs<R> p = base_pass<R>(ctx, Lam, eval, atol, rtol);
        set_tasks(p, ctx, false);
        p.corrs = ctx->corrs_sde;
        p.prop_kind = PROP_PLAIN;
        p.prop_a = r1;
        p.prop_da = r1;
        p.out = d2;
        set_slots<R>(p, r1, r1, r1, r1, kMaskLeft);
        CK_PASS(run_pass<R>(ctx, p));
        CK((++ctx->launches, launch_symmetrize)(ctx->L, ctx->lat.exch, d2, ctx->st));
        return 0;
    };
    int rc = ctx->precision == PFFRG_FP64 ? run(double{}) : run(float{});
    if (rc) return rc;
    return check_finite(ctx, d2);
}

// One SDE or BSE evaluation of the device parquet loop, repeated with more Gauss-Kronrod segments
// or a bigger chunk queue when it ran out of them (the inputs are unchanged by a failed evaluation)
template <class Fn>
int parquet_eval(pffrg_ctx* ctx, Fn fn) {
    for (;;) {
        int rc = fn();
        if (!rc) rc = check_status(ctx);
        if (rc != PFFRG_E_LIMIT || !(grow_gk(ctx) || grow_queue(ctx))) return rc;
    }
}

}  // namespace

extern "C" {

static int sde_once(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a1, pffrg_action_view* a2, int eval, double gatol,
              double grtol, double satol, double srtol) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    double* d1 = ctx->slot[PFFRG_SLOT_A];
    double* d2 = ctx->slot[PFFRG_SLOT_DA];
    if (int rc = copy_view(ctx, d1, a1, true)) return rc;
    if (int rc = copy_view(ctx, d2, a2, true)) return rc;
    int rc = sde_dev(ctx, Lam, d1, d2, eval, gatol, grtol, satol, srtol);
    if (rc) return rc;
    if ((rc = check_status(ctx))) return rc;
    if ((rc = copy_view(ctx, d2, a2, false))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pffrg_sde(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a1, pffrg_action_view* a2, int eval, double gatol,
              double grtol, double satol, double srtol) {
    return gk_retry(ctx, [&] { return sde_once(ctx, Lam, a1, a2, eval, gatol, grtol, satol, srtol); });
}

static int bse_once(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a1, pffrg_action_view* a2, int eval, double atol,
              double rtol) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    double* d1 = ctx->slot[PFFRG_SLOT_A];
    double* d2 = ctx->slot[PFFRG_SLOT_DA];
    if (int rc = copy_view(ctx, d1, a1, true)) return rc;
    if (int rc = copy_view(ctx, d2, a2, true)) return rc;
    int rc = bse_dev(ctx, Lam, d1, d2, eval, atol, rtol);
    if (rc) return rc;
    if ((rc = check_status(ctx))) return rc;
    if ((rc = copy_view(ctx, d2, a2, false))) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pffrg_bse(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a1, pffrg_action_view* a2, int eval, double atol,
              double rtol) {
    return gk_retry(ctx, [&] { return bse_once(ctx, Lam, a1, a2, eval, atol, rtol); });
}

int pffrg_parquet(pffrg_ctx* ctx, double Lam, int eval, double gatol, double grtol, double satol, double srtol,
                  double tol_abs, double tol_rel, double beta, int max_iter, int* iterations, double* abs_err,
                  double* rel_err, double* residuals) {
    if (!ctx) return PFFRG_E_ARGS;
    if (eval < 1 || max_iter < 0 || !(beta > 0.0) || beta > 1.0)
        return ctx->fail(PFFRG_E_ARGS, "eval >= 1, max_iter >= 0 and 0 < beta <= 1 required");
    CK(cudaSetDevice(ctx->device));
    const Layout& L = ctx->L;
    double* A = ctx->slot[PFFRG_SLOT_A];    // a: the iterate, updated in place
    double* P = ctx->slot[PFFRG_SLOT_DA];   // ap: SDE / BSE result
    double* E = ctx->slot[PFFRG_SLOT_ERR];  // a_err = ap - a on the vertex
    double* h = ctx->h_scalars;
    double ea = INFINITY, er = INFINITY;
    int count = 1;
    // parquet.jl:43-80
    while (ea >= tol_abs && er >= tol_rel && count <= max_iter) {
        double sa = INFINITY, sr = INFINITY;
        int scount = 1;
        while (sa >= tol_abs && sr >= tol_rel && scount <= max_iter) {
            if (int rc = parquet_eval(ctx, [&] { return sde_dev(ctx, Lam, A, P, eval, gatol, grtol, satol, srtol); }))
                return rc;
            // max|ap.Σ - a.Σ|, max|a.Σ|, max|ap.Σ|, then a.Σ = (1 - β) a.Σ + β ap.Σ
            ++ctx->launches;
            CK(launch_sigma_err(L.Nsig, A, P, ctx->scalars, ctx->st));
            CK((++ctx->launches, launch_axpby)(L, 1.0 - beta, P, beta, A, true, false, ctx->st));
            CK(cudaMemcpyAsync(h, ctx->scalars, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->st));
            CK(cudaStreamSynchronize(ctx->st));
            sa = h[0];
            sr = sa / std::max(h[1], h[2]);
            ++scount;
        }
        if (int rc = parquet_eval(ctx, [&] { return bse_dev(ctx, Lam, A, P, eval, gatol, grtol); })) return rc;
        // a_err = ap - a on the vertex; abs = max|a_err.q3|, rel = abs / max(max|a.q3|, max|ap.q3|)
        CK(cudaMemcpyAsync(E, P, sizeof(double) * L.total, cudaMemcpyDeviceToDevice, ctx->st));
        CK((++ctx->launches, launch_axpby)(L, 1.0, A, -1.0, E, false, true, ctx->st));
        if (int rc = absmax(ctx, E, ctx->scalars + 0)) return rc;
        if (int rc = absmax(ctx, A, ctx->scalars + 1)) return rc;
        if (int rc = absmax(ctx, P, ctx->scalars + 2)) return rc;
        // a = (1 - β) a + β ap on the vertex (bare excluded)
        CK((++ctx->launches, launch_axpby)(L, 1.0 - beta, P, beta, A, false, true, ctx->st));
        CK(cudaMemcpyAsync(h, ctx->scalars, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        ea = h[0];
        if (residuals) residuals[count - 1] = ea;
        er = ea / std::max(h[1], h[2]);
        ++count;
    }
    if (iterations) *iterations = count - 1;
    if (abs_err) *abs_err = ea;
    if (rel_err) *rel_err = er;
    return 0;
}

static int bs_step_once(pffrg_ctx* ctx, int loops, double Lam, double dLam, int eval, double gatol, double grtol,
                  double satol, double srtol, int sigma_corr, double ode_atol, double ode_rtol, double* err,
                  double* abs_max_next) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    const Layout& L = ctx->L;
    double* A = ctx->slot[PFFRG_SLOT_A];
    double* K = ctx->slot[PFFRG_SLOT_DA];
    double* I = ctx->slot[PFFRG_SLOT_INTER];
    double* E = ctx->slot[PFFRG_SLOT_ERR];
    double* N = ctx->slot[PFFRG_SLOT_NEXT];
    const size_t bytes = sizeof(double) * L.total;
    auto rhs = [&](double lam, const double* src) {
        return rhs_dev(ctx, loops, lam, src, K, eval, gatol, grtol, satol, srtol, sigma_corr);
    };
    // the stage derivative has zero bare couplings, as the reference's a_stage (the 2-loop left
    // kernels read them); the host-buffer entry points may have staged other values in this slot
    for (int c = 0; c < L.C; ++c) CK(cudaMemsetAsync(K + L.bare(c), 0, sizeof(double) * L.Ns, ctx->st));
    // launcher_1l.jl:83-116
    CK(cudaMemcpyAsync(N, A, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    CK(cudaMemcpyAsync(E, A, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    int64_t evals = 0;
    if (int rc = rhs(Lam, A)) return rc;
    if (int rc = read_evals(ctx)) return rc;
    evals += ctx->last_evals;
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -2.0 * dLam / 9.0, N, true, true, ctx->st));
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -7.0 * dLam / 24.0, E, true, true, ctx->st));
    CK(cudaMemcpyAsync(I, A, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -0.5 * dLam, I, true, true, ctx->st));
    if (int rc = rhs(Lam - 0.5 * dLam, I)) return rc;
    if (int rc = read_evals(ctx)) return rc;
    evals += ctx->last_evals;
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -1.0 * dLam / 3.0, N, true, true, ctx->st));
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -1.0 * dLam / 4.0, E, true, true, ctx->st));
    CK(cudaMemcpyAsync(I, A, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -0.75 * dLam, I, true, true, ctx->st));
    if (int rc = rhs(Lam - 0.75 * dLam, I)) return rc;
    if (int rc = read_evals(ctx)) return rc;
    evals += ctx->last_evals;
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -4.0 * dLam / 9.0, N, true, true, ctx->st));
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -1.0 * dLam / 3.0, E, true, true, ctx->st));
    CK(cudaMemcpyAsync(I, N, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    if (int rc = rhs(Lam - dLam, I)) return rc;
    if (int rc = read_evals(ctx)) return rc;
    evals += ctx->last_evals;
    CK((++ctx->launches, launch_axpby)(L, 1.0, K, -1.0 * dLam / 8.0, E, true, true, ctx->st));
    // subtract_from!(a_inter, a_err) and the error ratio (launcher_1l.jl:112-116)
    CK((++ctx->launches, launch_axpby)(L, 1.0, I, -1.0, E, true, true, ctx->st));
    if (int rc = absmax(ctx, E, ctx->scalars + 0)) return rc;
    if (int rc = absmax(ctx, I, ctx->scalars + 1)) return rc;
    if (int rc = absmax(ctx, A, ctx->scalars + 2)) return rc;
    CK(cudaMemcpyAsync(ctx->h_scalars, ctx->scalars, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (int rc = check_status(ctx)) return rc;
    const double delta = ctx->h_scalars[0];
    const double scale = ode_atol + fmax(ctx->h_scalars[1], ctx->h_scalars[2]) * ode_rtol;
    if (err) *err = delta / scale;
    if (abs_max_next) *abs_max_next = ctx->h_scalars[1];
    ctx->last_evals = evals;
    return 0;
}

int pffrg_bs_step(pffrg_ctx* ctx, int loops, double Lam, double dLam, int eval, double gatol, double grtol,
                  double satol, double srtol, int sigma_corr, double ode_atol, double ode_rtol, double* err,
                  double* abs_max_next) {
    return gk_retry(ctx, [&] { return bs_step_once(ctx, loops, Lam, dLam, eval, gatol, grtol, satol, srtol, sigma_corr, ode_atol, ode_rtol, err, abs_max_next); });
}

int pffrg_accept(pffrg_ctx* ctx) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(ctx->slot[PFFRG_SLOT_A], ctx->slot[PFFRG_SLOT_NEXT], sizeof(double) * ctx->L.total,
                       cudaMemcpyDeviceToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pffrg_chi(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a, const double* chi_mesh, int num_chi,
              double atol, double rtol, double* chi) {
    if (!ctx) return PFFRG_E_ARGS;
    CK(cudaSetDevice(ctx->device));
    if (int rc = copy_view(ctx, ctx->slot[PFFRG_SLOT_A], a, true)) return rc;
    return chi_dev(ctx, Lam, ctx->slot[PFFRG_SLOT_A], chi_mesh, num_chi, atol, rtol, chi);
}

int pffrg_chi_slot(pffrg_ctx* ctx, double Lam, int slot, const double* chi_mesh, int num_chi, double atol,
                   double rtol, double* chi) {
    if (!ctx) return PFFRG_E_ARGS;
    if (slot < 0 || slot >= PFFRG_NUM_SLOTS) return ctx->fail(PFFRG_E_ARGS, "bad slot");
    CK(cudaSetDevice(ctx->device));
    return chi_dev(ctx, Lam, ctx->slot[slot], chi_mesh, num_chi, atol, rtol, chi);
}

int pffrg_scan_cuts(pffrg_ctx* ctx, int slot, double* sigma, int64_t* argmax, double* cuts) {
    if (!ctx || !sigma || !argmax || !cuts) return ctx ? ctx->fail(PFFRG_E_ARGS, "null output") : PFFRG_E_ARGS;
    if (slot < 0 || slot >= PFFRG_NUM_SLOTS) return ctx->fail(PFFRG_E_ARGS, "bad slot");
    CK(cudaSetDevice(ctx->device));
    const Layout& L = ctx->L;
    ++ctx->launches;
    CK(launch_scan_cuts(L, ctx->slot[slot], ctx->scan_arg, ctx->scan_cuts, ctx->st));
    CK(cudaMemcpyAsync(sigma, ctx->slot[slot], sizeof(double) * L.Nsig, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(argmax, ctx->scan_arg, sizeof(long long) * 3 * L.C, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(cuts, ctx->scan_cuts, sizeof(double) * 3 * L.C * (L.NO + 3 * L.Nn), cudaMemcpyDeviceToHost,
                       ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return 0;
}

int pffrg_resample(pffrg_ctx* ctx, int src_slot, int dst_slot, const pffrg_mesh_view* mesh) {
    if (!ctx) return PFFRG_E_ARGS;
    if (src_slot < 0 || src_slot >= PFFRG_NUM_SLOTS || dst_slot < 0 || dst_slot >= PFFRG_NUM_SLOTS ||
        src_slot == dst_slot)
        return ctx->fail(PFFRG_E_ARGS, "bad slots");
    if (int rc = check_mesh(ctx, mesh)) return rc;
    const Layout& L = ctx->L;
    if (mesh->num_sigma != L.Nsig || mesh->num_omega != L.NO || mesh->num_nu != L.Nn)
        return ctx->fail(PFFRG_E_ARGS, "mesh sizes differ from the context's");
    CK(cudaSetDevice(ctx->device));
    std::vector<double> h;
    h.insert(h.end(), mesh->sigma, mesh->sigma + mesh->num_sigma);
    h.insert(h.end(), mesh->omega_s, mesh->omega_s + mesh->num_omega);
    h.insert(h.end(), mesh->nu_s, mesh->nu_s + mesh->num_nu);
    h.insert(h.end(), mesh->omega_t, mesh->omega_t + mesh->num_omega);
    h.insert(h.end(), mesh->nu_t, mesh->nu_t + mesh->num_nu);
    CK(cudaMemcpyAsync(ctx->mesh_new, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, ctx->st));
    ++ctx->launches;
    CK(launch_resample(L, ctx->mesh, ctx->mesh_new, ctx->slot[src_slot], ctx->slot[dst_slot], ctx->st));
    // the new meshes become the context's
    return upload_mesh(ctx, mesh);
}

int pffrg_set_async_waves(pffrg_ctx* ctx, int on) {
    if (!ctx) return PFFRG_E_ARGS;
    ctx->async_waves = on ? 1 : 0;
    return 0;
}

int pffrg_set_fp64_handoff(pffrg_ctx* ctx, double eps) {
    if (!ctx) return PFFRG_E_ARGS;
    if (!(eps >= 0.0) || eps >= 1.0) return ctx->fail(PFFRG_E_ARGS, "hand-off margin must be in [0, 1)");
    ctx->esc_eps = eps;
    return 0;
}

int pffrg_set_chi_cluster(pffrg_ctx* ctx, int64_t min_regions, int blocks) {
    if (!ctx) return PFFRG_E_ARGS;
    if (min_regions < 0) return ctx->fail(PFFRG_E_ARGS, "negative region count");
    if (blocks != 8 && blocks != 16) return ctx->fail(PFFRG_E_ARGS, "cluster of %d blocks is not built", blocks);
    ctx->chi_cluster_min = min_regions;
    ctx->chi_cluster_blocks = blocks;
    return 0;
}

int pffrg_set_chi_integrand(pffrg_ctx* ctx, int precision) {
    if (!ctx) return PFFRG_E_ARGS;
    if (precision != PFFRG_FP64 && precision != PFFRG_MIXED) return ctx->fail(PFFRG_E_ARGS, "bad precision");
    ctx->chi_fp64 = precision == PFFRG_FP64 ? 1 : 0;
    return 0;
}

int pffrg_set_team_shape(pffrg_ctx* ctx, int lanes, int sites_per_lane) {
    if (!ctx) return PFFRG_E_ARGS;
    static const int shapes[][2] = {{0, 0}, {8, 1}, {16, 1}, {16, 3}, {16, 4}, {32, 1}, {32, 2}, {32, 3}, {32, 4},
                                    {32, 8}};
    for (const auto& sh : shapes)
        if (sh[0] == lanes && sh[1] == sites_per_lane) {
            ctx->team_T = lanes;
            ctx->team_SPL = sites_per_lane;
            return 0;
        }
    return ctx->fail(PFFRG_E_ARGS, "team shape %dx%d is not built", lanes, sites_per_lane);
}

int pffrg_set_capacities(pffrg_ctx* ctx, int64_t queue_chunks, int64_t gk_segments) {
    if (!ctx) return PFFRG_E_ARGS;
    if (queue_chunks < 0 || queue_chunks > (1ll << 30)) return ctx->fail(PFFRG_E_ARGS, "queue capacity out of range");
    if (gk_segments != 0 && (gk_segments < 16 || gk_segments > kGkCapMax))
        return ctx->fail(PFFRG_E_ARGS, "Gauss-Kronrod capacity must be 0 or in [16, %lld]", kGkCapMax);
    CK(cudaSetDevice(ctx->device));
    ctx->queue_cap_req = queue_chunks;
    ctx->wave_nsub = 0;  // the next pass allocates the requested (or the default) queue
    ctx->gk_overflow = 0;
    ctx->gk_cap = gk_segments > 0 ? gk_segments : kGkCap0;
    CK(stream_free(ctx->st, ctx->gk_seg));
    ctx->gk_seg = nullptr;
    ctx->gk_slots = 0;
    return 0;
}

int pffrg_set_overlap_staging(pffrg_ctx* ctx, int mode) {
    if (!ctx) return PFFRG_E_ARGS;
    if (mode < 0 || mode > 2) return ctx->fail(PFFRG_E_ARGS, "overlap staging mode %d (0, 1 or 2)", mode);
    ctx->rows_mode = mode;
    return 0;
}

void* pffrg_host_alloc(int64_t bytes) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return p;
}

void pffrg_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"

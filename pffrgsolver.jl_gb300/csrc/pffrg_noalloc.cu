// One-loop dΓ without device allocation.
//
// Some callers cannot allocate device memory themselves: hosts whose device
// memory belongs to another framework's pool allocator (a second allocator
// fragments the pool and can fail under the first one's reservations), and
// embedders whose device-memory budget is fixed when they start.  For them
// pffrg_dgamma_1l_noalloc computes compute_dΓ_1l!'s result (boundary
// corrections, Katanin bubbles of all channel tasks, symmetrisation) with
// every piece of scratch -- lattice and mesh tables, the integration bounds,
// the boundary corrections and the adaptive-quadrature workspace -- inside
// one statically sized device array of this file.  It calls no cudaMalloc,
// cudaFree or other allocating CUDA routine.  It copies its tables from
// pageable host memory and waits for the stream before it returns.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/pffrg_gpu.h"
#include "pffrg_internal.h"

using namespace pffrg;

namespace {

// Fixed scratch of the no-allocation entry point: 128 MiB, held by every GPU
// that loads this library until the process exits.
constexpr size_t kNoAllocScratchBytes = size_t(128) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;
thread_local std::string g_noalloc_error;

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_noalloc_error = buf;
    return code;
}

// Device address of the static scratch on the current device, looked up once per device.
int scratch_address(int dev, void** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(PFFRG_E_LIMIT, "device ordinal %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(PFFRG_E_CUDA, "cudaGetSymbolAddress of the static scratch failed: %s", cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return 0;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

#define NK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return fail(PFFRG_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

extern "C" {

const char* pffrg_noalloc_last_error(void) { return g_noalloc_error.c_str(); }

int64_t pffrg_noalloc_scratch_bytes(void) { return (int64_t)kNoAllocScratchBytes; }

int pffrg_dgamma_1l_noalloc(const pffrg_lattice_view* lat, const pffrg_mesh_view* mesh, double S, double Lam,
                            const double* a_dev, double* da_dev, int eval, double atol, double rtol,
                            void* stream) {
    g_noalloc_error.clear();
    if (!lat || !mesh || !a_dev || !da_dev || !lat->exchange || !lat->mult || !lat->overlap_offsets)
        return fail(PFFRG_E_ARGS, "null argument");
    // the site count bounds every table read below, the overlap offsets included
    if (lat->num_sites < 1 || lat->num_sites > 256) return fail(PFFRG_E_LIMIT, "between 1 and 256 irreducible sites");
    if (!lat->overlap_rows && lat->overlap_offsets[lat->num_sites] > 0) return fail(PFFRG_E_ARGS, "null overlap rows");
    if (!mesh->sigma || !mesh->omega_s || !mesh->nu_s || !mesh->omega_t || !mesh->nu_t)
        return fail(PFFRG_E_ARGS, "mesh view has null arrays");
    if (mesh->num_sigma < 2 || mesh->num_omega < 2 || mesh->num_nu < 2 || mesh->num_sigma > kMaxMesh ||
        mesh->num_omega > kMaxMesh || mesh->num_nu > kMaxMesh)
        return fail(PFFRG_E_LIMIT, "mesh lengths must lie in [2, %d]", kMaxMesh);
    if (eval < 1) return fail(PFFRG_E_ARGS, "eval must be positive");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0;
    NK(cudaGetDevice(&dev));
    void* scratch = nullptr;
    if (int rc = scratch_address(dev, &scratch)) return rc;

    const int Ns = (int)lat->num_sites;
    const Layout L = make_layout(Ns, (int)mesh->num_sigma, (int)mesh->num_omega, (int)mesh->num_nu, 2);
    const int NO = L.NO, Nn = L.Nn;

    // host-side tables: 0-based exchange, packed overlap rows, mesh block, task list, log bounds
    std::vector<int> exch(Ns), off(Ns + 1);
    for (int i = 0; i < Ns; ++i) {
        exch[i] = (int)lat->exchange[i] - 1;
        if (exch[i] < 0 || exch[i] >= Ns) return fail(PFFRG_E_ARGS, "exchange table out of range");
    }
    for (int i = 0; i <= Ns; ++i) off[i] = (int)lat->overlap_offsets[i];
    const int64_t R = off[Ns];
    std::vector<unsigned> rows(R > 0 ? R : 1);
    for (int64_t j = 0; j < R; ++j) {
        const int64_t a = lat->overlap_rows[3 * j] - 1, b = lat->overlap_rows[3 * j + 1] - 1;
        const int64_t mm = lat->overlap_rows[3 * j + 2];
        if (a < 0 || a >= Ns || b < 0 || b >= Ns || mm < 0 || mm >= 65536)
            return fail(PFFRG_E_ARGS, "overlap table out of range");
        rows[j] = (unsigned)a | ((unsigned)b << 8) | ((unsigned)mm << 16);
    }
    std::vector<double> hmesh;
    hmesh.insert(hmesh.end(), mesh->sigma, mesh->sigma + L.Nsig);
    hmesh.insert(hmesh.end(), mesh->omega_s, mesh->omega_s + NO);
    hmesh.insert(hmesh.end(), mesh->nu_s, mesh->nu_s + Nn);
    hmesh.insert(hmesh.end(), mesh->omega_t, mesh->omega_t + NO);
    hmesh.insert(hmesh.end(), mesh->nu_t, mesh->nu_t + Nn);
    append_inverse_spacings(hmesh, L.Nsig, NO, Nn);
    // channel tasks with w2 >= w3 (compute.jl:73-107), 0-based
    std::vector<int4> tasks;
    for (int w1 = 0; w1 < NO; ++w1) {
        tasks.push_back(make_int4(1, w1, -1, -1));
        for (int w3 = 0; w3 < Nn; ++w3) {
            tasks.push_back(make_int4(2, w1, w3, -1));
            tasks.push_back(make_int4(3, w1, -1, w3));
            for (int w2 = w3; w2 < Nn; ++w2) tasks.push_back(make_int4(4, w1, w2, w3));
        }
    }
    // ξ^k a of integrate_log! with libm's pow, as the reference rounds them
    std::vector<double> bounds((size_t)2 * NO * (eval + 1), 0.0);
    for (int m = 0; m < 2; ++m) {
        const double* Om = m ? mesh->omega_t : mesh->omega_s;
        const double* nu = m ? mesh->nu_t : mesh->nu_s;
        const double val = Om[NO - 1] + nu[Nn - 1];
        for (int w1 = 0; w1 < NO; ++w1) {
            const double a = 2.0 * (Lam + 0.5 * Om[w1]), b = 1.0 * val;
            if (!(b > a)) continue;
            const double xi = std::pow(b / a, 1.0 / eval);
            for (int k = 0; k <= eval; ++k) bounds[(size_t)(m * NO + w1) * (eval + 1) + k] = std::pow(xi, (double)k) * a;
        }
    }

    // carve the static scratch
    const long long ntasks = (long long)tasks.size();
    const long long nsub = ntasks * 3 * (4 * eval + 1);
    // chunk queue of one level: a quarter of the regular path's 8 nsub + 65536, so that square L = 3
    // with 50/15/10 meshes at eval 10 fits the array; a level that needs more returns PFFRG_E_LIMIT
    const long long qcap = 2 * nsub + 4096;
    size_t o = 0;
    const size_t o_exch = o;
    o = align_up(o + sizeof(int) * Ns);
    const size_t o_off = o;
    o = align_up(o + sizeof(int) * (Ns + 1));
    const size_t o_rows = o;
    o = align_up(o + sizeof(unsigned) * rows.size());
    const size_t o_mesh = o;
    o = align_up(o + sizeof(double) * hmesh.size());
    const size_t o_bounds = o;
    o = align_up(o + sizeof(double) * bounds.size());
    const size_t o_tasks = o;
    o = align_up(o + sizeof(int4) * tasks.size());
    const size_t o_corrs = o;
    o = align_up(o + sizeof(double) * 6 * NO);
    const size_t o_gk = o;  // Gauss-Kronrod segments of the 6 NO boundary integrals
    o = align_up(o + sizeof(double) * 4 * (size_t)kGkCap0 * 6 * NO);
    const size_t o_gk_status = o;  // segment-capacity flag of those integrals (the passes clear their counters)
    o = align_up(o + sizeof(int));
    const size_t o_wave = o;
    o += wave_space_bytes(nsub, Ns, qcap, 2);
    if (o > kNoAllocScratchBytes)
        return fail(PFFRG_E_LIMIT,
                    "problem needs %zu bytes of scratch, the no-allocation entry point holds %zu "
                    "(fewer sites, frequencies or eval)",
                    o, kNoAllocScratchBytes);
    char* base = static_cast<char*>(scratch);
    NK(cudaMemcpyAsync(base + o_exch, exch.data(), sizeof(int) * Ns, cudaMemcpyHostToDevice, st));
    NK(cudaMemcpyAsync(base + o_off, off.data(), sizeof(int) * (Ns + 1), cudaMemcpyHostToDevice, st));
    NK(cudaMemcpyAsync(base + o_rows, rows.data(), sizeof(unsigned) * rows.size(), cudaMemcpyHostToDevice, st));
    NK(cudaMemcpyAsync(base + o_mesh, hmesh.data(), sizeof(double) * hmesh.size(), cudaMemcpyHostToDevice, st));
    NK(cudaMemcpyAsync(base + o_bounds, bounds.data(), sizeof(double) * bounds.size(), cudaMemcpyHostToDevice, st));
    NK(cudaMemcpyAsync(base + o_tasks, tasks.data(), sizeof(int4) * tasks.size(), cudaMemcpyHostToDevice, st));
    WaveSpace W;
    wave_space_carve(W, base + o_wave, nsub, Ns, qcap, 2);
    // the wave counters and the Gauss-Kronrod flag are the only scratch read before this call writes it
    NK(cudaMemsetAsync(W.counters, 0, sizeof(int) * 8, st));
    int* gk_status = reinterpret_cast<int*>(base + o_gk_status);
    NK(cudaMemsetAsync(gk_status, 0, sizeof(int), st));

    // boundary corrections of the Katanin bubbles (bubbles.jl:99-159)
    CorrsArgs<double> c;
    c.NO = NO;
    c.Nn = Nn;
    c.Nsig = L.Nsig;
    c.kind = PROP_KAT;
    c.a = a_dev;
    c.da = da_dev;
    c.mesh = reinterpret_cast<const double*>(base + o_mesh);
    c.Lam = Lam;
    c.atol = atol;
    c.rtol = rtol;
    c.corrs = reinterpret_cast<double*>(base + o_corrs);
    c.seg = reinterpret_cast<double*>(base + o_gk);
    c.seg_cap = kGkCap0;
    c.status = gk_status;
    NK(launch_corrs<double>(c, st));
    // the passes weight their boundary nodes with these corrections: stop here if any integral ran
    // out of segments (the regular entry points grow the segment buffer and repeat instead)
    int status = 0;
    NK(cudaMemcpyAsync(&status, gk_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    NK(cudaStreamSynchronize(st));
    if (status)
        return fail(PFFRG_E_LIMIT, "adaptive Gauss-Kronrod segment capacity (%lld per boundary integral) exceeded",
                    (long long)kGkCap0);

    // Katanin bubbles of all channel tasks (flow_su2_{s,t,u}.jl:2-55)
    PassArgs<double> p;
    std::memset(&p, 0, sizeof(p));
    p.L = L;
    for (int k = 0; k < 4; ++k) p.src[k] = a_dev;
    for (int X = 0; X < 3; ++X)
        for (int k = 0; k < 4; ++k) p.mask[X][k] = CH_ALL;
    p.prop_kind = PROP_KAT;
    p.prop_a = a_dev;
    p.prop_da = da_dev;
    p.prop_a64 = a_dev;
    p.prop_da64 = da_dev;
    p.out = da_dev;
    p.exch = reinterpret_cast<const int*>(base + o_exch);
    p.ov_off = reinterpret_cast<const int*>(base + o_off);
    p.ov_rows = reinterpret_cast<const unsigned*>(base + o_rows);
    p.rows_total = R;
    p.mesh = reinterpret_cast<const double*>(base + o_mesh);
    p.log_bounds = reinterpret_cast<const double*>(base + o_bounds);
    p.corrs = reinterpret_cast<const double*>(base + o_corrs);
    p.tasks = reinterpret_cast<const int4*>(base + o_tasks);
    p.ntasks = (int)ntasks;
    p.nchan = 3;
    p.chan_of_y[0] = 1;
    p.chan_of_y[1] = 0;
    p.chan_of_y[2] = 2;
    p.Lam = Lam;
    p.atol = atol;
    p.rtol = rtol;
    p.eval = eval;
    p.twoS = 2.0 * S;
    p.node_counter = nullptr;
    static thread_local int h_counters[8];
    cudaError_t e = launch_pass<double>(p, W, h_counters, st);
    if (e == cudaErrorLaunchOutOfResources && h_counters[4])
        return fail(PFFRG_E_LIMIT, "quadrature chunk queue of the static scratch exceeded");
    NK(e);
    NK(launch_symmetrize(L, p.exch, da_dev, st));
    NK(cudaStreamSynchronize(st));
    return 0;
}

}  // extern "C"

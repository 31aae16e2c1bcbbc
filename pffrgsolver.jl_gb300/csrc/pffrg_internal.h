// Host-side interface between the translation units of libpffrg_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "pffrg_device.cuh"

namespace pffrg {

enum PropKind { PROP_KAT = 0, PROP_PLAIN = 1 };
enum ChannelMask { CH_S = 1, CH_T = 2, CH_U = 4, CH_ALL = 7 };

// Lattice tables on the device (0-based site indices).
struct DevLattice {
    int Ns = 0;
    int64_t rows = 0;
    int* exch = nullptr;     // [Ns]
    int* mult = nullptr;     // [Ns]
    int* ov_off = nullptr;   // [Ns+1]
    unsigned* ov_rows = nullptr;  // [R] site a | site b << 8 | multiplicity << 16
};

// One pass of channel tasks (Katanin / left / central / BSE / reduced-s).
template <typename R>
struct PassArgs {
    Layout L;
    const R* src[4];   // vertex slot sources
    int mask[3][4];    // [channel X][slot]: channels read (CH_*), 0 = bare only
    int prop_kind;
    const R* prop_a;   // Σ of the propagators
    const R* prop_da;  // dΣ of the Katanin propagator
    const double* prop_a64;   // the same in FP64 (propagators of the FP64 path and of the mixed
    const double* prop_da64;  // path's FP64 hand-off pass)
    double* out;       // FP64 output action
    const int* exch;
    const int* ov_off;       // [Ns+1]
    const unsigned* ov_rows; // [R] site a | site b << 8 | multiplicity << 16
    long long rows_total;
    int rows_in_smem;        // stage the rows in shared memory
    int rows_mode;           // 0: staging chosen by size, 1: rows read through L1/L2, 2: staged when they fit
    const double* mesh;   // [σ | Ωs | νs | Ωt | νt] then their inverse spacings (FP64)
    const float* mesh_ff; // the same as float pairs h, l and FP32 inverse spacings (mixed path)
    const double* corrs;  // [2,3,NO]
    const double* log_bounds;  // [mesh s/u = 0, t = 1][w1][k = 0..eval]: ξ^k a of integrate_log!
    const int4* tasks;    // (kernel 1..4, w1, w2, w3), 0-based frequency indices
    int ntasks;
    int nchan;            // channels launched (3, or 1 for the reduced s bubble)
    int chan_of_y[3];     // blockIdx.y -> channel
    double Lam, atol, rtol;
    int eval;
    double twoS;
    int reduced;          // reduced s bubble of the SDE (U(1)-DM keeps xx, zz, dd only)
    int async_waves;      // levels without host round trips; overflow reported in *status (bit 3)
    int team_T, team_SPL; // team shape (lanes per node batch, sites per lane); 0: chosen by Ns
    // FP64 hand-off of the mixed path: 1 = FP32 pass that hands every subdomain whose Simpson test
    // is closer to its bounds than esc_eps (relative rounding of the FP32 node values) allows to
    // an FP64 pass, 2 = that FP64 pass over the handed subdomains (then the reduction), 0 = off
    int esc_mode;
    double esc_eps;
    int* status;
    unsigned long long* node_counter;  // optional: [0] integrand evaluations, [1] algorithmic values read
};

// Scratch of one pass of the level-synchronous quadrature: one record and two state
// vectors per Simpson subdomain, the chunk queues of the current and next level, and one
// partial node sum per chunk.  Carved out of one device block.
struct SubRec {
    double lo, hi, sgn;
    long long n;  // new nodes of the pending level (0: finished)
    int chunk0;   // first chunk of the pending level in the wave queue
    int nchunk;
    double sa;    // FP32 pass: bound of |weights| x |node values| of the last Simpson sum (norm)
    double fab;   // and of the last level's new nodes
};

struct WaveSpace {
    SubRec* subs;    // [nsub]
    double* stA;     // [nsub][C Ns]: Simpson sum of the last level, then the result
    double* stB;     // [nsub][C Ns]: node sum of the last level's new nodes
    int4* queue[2];  // chunk records (sub, first node, count, -) of the current / next level
    int* active[2];  // subdomains with chunks in the current / next level
    double* part;    // [qcap][C Ns] chunk partial node sums
    double* part_abs;  // [qcap] FP32 pass: norm of the chunk's sums of |node values|
    int* esc;        // [nsub] subdomains handed from the FP32 pass to the FP64 pass
    int* counters;   // [0..1] chunks, [2..3] active subdomains per parity, [4] queue overflow, [5] handed
    int nsub, qcap;
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// float-float form of a mesh block [σ | Ωs | νs | Ωt | νt] (without inverses): the high floats,
// the low floats (x - h) and the FP32 inverse spacings, then per mesh the placement parameters of
// MeshFF::g (the lin-log form of get_mesh read off the mesh itself; any increasing mesh is
// searched correctly, a mesh of that form in a step or two)
inline std::vector<float> mesh_block_ff(const std::vector<double>& x, int Nsig, int NO, int Nn) {
    const int len[5] = {Nsig, NO, Nn, NO, Nn};
    const size_t n = (size_t)Nsig + 2 * NO + 2 * Nn;
    std::vector<float> f(3 * n + kMeshGuess, 0.f);
    size_t o = 0;
    for (int a = 0; a < 5; ++a) {
        for (int k = 0; k < len[a]; ++k) {
            const double v = x[o + k];
            const float h = (float)v;
            f[o + k] = h;
            f[n + o + k] = (float)(v - (double)h);
            f[2 * n + o + k] = k + 1 < len[a] ? (float)(1.0 / (x[o + k + 1] - v)) : 0.f;
        }
        const double* m = x.data() + o;
        const int N = len[a];
        const double step = m[1] - m[0];
        if (m[0] == 0.0 && step > 0.0) {
            int nlin = 1;
            while (nlin + 1 < N && std::fabs(m[nlin + 1] - (nlin + 1) * step) <= 1e-6 * m[nlin + 1]) ++nlin;
            float* g = f.data() + 3 * n + 4 * a;
            g[0] = (float)(1.0 / step);
            g[1] = (float)nlin;
            g[2] = (float)m[nlin];
            if (nlin < N - 1 && m[N - 1] > m[nlin]) g[3] = (float)((N - 1 - nlin) / std::log(m[N - 1] / m[nlin]));
        }
        o += len[a];
    }
    return f;
}

// append the inverse spacings 1 / (x[k+1] - x[k]) (0 at the last entry) of the five meshes of a
// device mesh block [σ | Ωs | νs | Ωt | νt] to the block
inline void append_inverse_spacings(std::vector<double>& h, int Nsig, int NO, int Nn) {
    const int len[5] = {Nsig, NO, Nn, NO, Nn};
    size_t o = 0;
    for (int a = 0; a < 5; ++a) {
        for (int k = 0; k < len[a]; ++k) h.push_back(k + 1 < len[a] ? 1.0 / (h[o + k + 1] - h[o + k]) : 0.0);
        o += len[a];
    }
}

// bytes of the wave workspace for nsub subdomains, C components on Ns sites and qcap chunks
inline size_t wave_space_bytes(long long nsub, int Ns, long long qcap, int C) {
    const size_t vec = sizeof(double) * C * (size_t)Ns;
    return align256(sizeof(SubRec) * nsub) + 2 * align256(vec * nsub) + 2 * align256(sizeof(int4) * qcap) +
           2 * align256(sizeof(int) * nsub) + align256(vec * qcap) + align256(sizeof(double) * qcap) +
           align256(sizeof(int) * nsub) + align256(sizeof(int) * 8);
}

inline void wave_space_carve(WaveSpace& W, void* base, long long nsub, int Ns, long long qcap, int C) {
    char* p = static_cast<char*>(base);
    const size_t vec = sizeof(double) * C * (size_t)Ns;
    W.subs = reinterpret_cast<SubRec*>(p);
    p += align256(sizeof(SubRec) * nsub);
    W.stA = reinterpret_cast<double*>(p);
    p += align256(vec * nsub);
    W.stB = reinterpret_cast<double*>(p);
    p += align256(vec * nsub);
    for (int k = 0; k < 2; ++k) {
        W.queue[k] = reinterpret_cast<int4*>(p);
        p += align256(sizeof(int4) * qcap);
    }
    for (int k = 0; k < 2; ++k) {
        W.active[k] = reinterpret_cast<int*>(p);
        p += align256(sizeof(int) * nsub);
    }
    W.part = reinterpret_cast<double*>(p);
    p += align256(vec * qcap);
    W.part_abs = reinterpret_cast<double*>(p);
    p += align256(sizeof(double) * qcap);
    W.esc = reinterpret_cast<int*>(p);
    p += align256(sizeof(int) * nsub);
    W.counters = reinterpret_cast<int*>(p);
    W.nsub = (int)nsub;
    W.qcap = (int)qcap;
}

// one pass of channel tasks (SU(2) or U(1)-DM by a.L.C)
template <typename R>
cudaError_t launch_pass(const PassArgs<R>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st);

// GK integrals of the self energy / corrections (QuadGK-equivalent)
enum SigmaKind { SIG_FLOW = 0, SIG_CORR1 = 1, SIG_CORR2 = 2, SIG_SDE = 3 };

template <typename R>
struct SigmaArgs {
    Layout L;
    int kind;
    const R* a;    // propagator action (Σ) and, for SIG_FLOW/SIG_CORR2, the vertex
    const R* aux;  // vertex of SIG_CORR1/SIG_SDE; Σ of SIG_CORR2
    double* out;   // FP64 [Nsig] (index 0 untouched)
    const int* exch;
    const int* mult;
    const double* mesh;
    double Lam, atol, rtol, twoS;
    double* seg;        // Gauss-Kronrod segments: [Nsig - 1][4][seg_cap]
    long long seg_cap;
    int* status;   // nonzero: segment capacity exceeded
};

// Gauss-Kronrod segments per integral: the first launch's capacity and the most a
// 10^7-evaluation integral can use (QuadGK's maxevals, 30 evaluations per bisection)
constexpr long long kGkCap0 = 2048;
constexpr long long kGkCapMax = 10000000 / 30 + 8;

template <typename R>
cudaError_t launch_sigma(const SigmaArgs<R>& a, cudaStream_t st);

template <typename R>
struct CorrsArgs {
    int NO, Nn, Nsig, kind;
    const R* a;
    const R* da;
    const double* mesh;
    double Lam, atol, rtol;
    double* corrs;  // [2,3,NO]
    double* seg;          // Gauss-Kronrod segments: [6 NO][4][seg_cap]
    long long seg_cap;
    int* status;
};

template <typename R>
cudaError_t launch_corrs(const CorrsArgs<R>& a, cudaStream_t st);

// mesh scanning and resampling between flow steps
cudaError_t launch_scan_cuts(const Layout& L, const double* a, long long* argmax, double* cuts, cudaStream_t st);
cudaError_t launch_resample(const Layout& L, const double* mesh_old, const double* mesh_new, const double* a,
                            double* b, cudaStream_t st);

// correlations χ (FP64)
struct ChiArgs {
    Layout L;
    const double* a;         // the state (FP64)
    const float* af;         // its FP32 copy: integrand in FP32 (mixed path), or null
    const double* mesh;
    const double* chi_mesh;  // [num_chi]
    const float* mesh_ff;    // float-float meshes of the mixed integrand
    int num_chi;
    int ncomp;               // 1 (SU(2)) or 3 (U(1)-DM: xx, zz, xy)
    const int* exch;
    double Lam, atol, rtol, twoS;
    double* reg;             // [job slot][10][cap] region records (7) and the keys of three region lists
    int* reg_split;          // [job slot][4][cap] split dimensions and the entries of three region lists
    long long cap;           // regions per integral
    int* ctl;                // [job slot][4] a round's orders from a cluster's block 0 to the others
    double* box_out;         // [ncomp][num_chi][Ns][9]
    double* chi;             // [ncomp][Ns][num_chi], each column-major
    unsigned long long* evals;  // [0] cubature points, [1] largest region count, [2] rounds, [3] most rounds
    double* seg;             // Gauss-Kronrod segments of the local term: [num_chi][4][seg_cap]
    long long seg_cap;
    int* status;             // bit 1: GK segments exhausted
};
// the box integrals of the listed jobs (overflow[slot] = 1: region capacity exhausted), one block
// per integral, or a cluster of 8 (cluster 2..15) or 16 (cluster >= 16) blocks per integral
cudaError_t launch_chi_boxes(const ChiArgs& a, const int* jobs, int njobs, int* overflow, int cluster,
                             cudaStream_t st);
// the local term and the sums of the boxes into χ
cudaError_t launch_chi_sum(const ChiArgs& a, cudaStream_t st);

// elementwise action kernels (FP64)
cudaError_t launch_symmetrize(const Layout& L, const int* exch, double* a, cudaStream_t st);
cudaError_t launch_symmetrize_add_to(const Layout& L, const int* exch, const double* al, double* a,
                                     cudaStream_t st);
// y[gamma part] = alpha * y + beta * x over the vertex part (bare excluded); sigma_too adds Σ
cudaError_t launch_axpby(const Layout& L, double alpha, const double* x, double beta, double* y, bool sigma_too,
                         bool gamma_too, cudaStream_t st);
cudaError_t launch_to_float(const double* x, float* y, int64_t n, cudaStream_t st);
// the FP32 copy of an SU(2) action (C = 2) in the pair layout of the mixed passes (Layout::pq)
cudaError_t launch_to_float_pairs(const Layout& L, const double* x, float* y, cudaStream_t st);
// out = [max|ap.Σ - a.Σ|, max|a.Σ|, max|ap.Σ|] over the Nsig self-energy values
cudaError_t launch_sigma_err(int Nsig, const double* a, const double* ap, double* out, cudaStream_t st);
// *status |= 16 when any of a[0..n) is NaN or infinite
cudaError_t launch_check_finite(const double* a, int64_t n, int* status, cudaStream_t st);
// max |q3| over all components/channels -> out[0] (double, via block partials)
cudaError_t launch_absmax_q3(const Layout& L, const double* a, double* partial, int npartial, double* out,
                             cudaStream_t st);
// max over i of |x_i| for the vertex q3 part of (x - y) etc. are composed from the above

}  // namespace pffrg

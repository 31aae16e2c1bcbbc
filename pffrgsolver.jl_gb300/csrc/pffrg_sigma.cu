// Adaptive Gauss-Kronrod integrals of the flow right-hand side (sm_103a):
// the self-energy derivative compute_dΣ! (src/Flow/flow_self.jl:2-20), its
// multiloop corrections compute_dΣ_corr! (flow_self.jl:23-51), the SDE
// self energy of compute_Σ! (src/Flow/SDE.jl:58-96) and the boundary
// corrections compute_corrs_kat!/compute_corrs! (src/Flow/bubbles.jl:99-221).
//
// The reference integrates these with QuadGK.jl (compat 2.4, not part of the
// reference tree).  Its published algorithm is restated here: a 7-point
// Gauss / 15-point Kronrod rule per segment, error |K - G|, repeated
// bisection of the segment with the largest error until the total error is
// below max(atol, rtol |I|), infinite end points mapped by x = t / (1 - t^2)
// (both ends) or x = s0 +- t / (1 - t) (one end).  One warp owns one
// integral; the 30 nodes of a bisection are evaluated by 30 lanes.
#include <type_traits>

#include "pffrg_internal.h"

namespace pffrg {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kSigWarps = 2;

__constant__ double c_gkx[8] = {-0.991455371120812639206854697526329, -0.949107912342758524526189684047851,
                                -0.864864423359769072789712788640926, -0.741531185599394439863864773280788,
                                -0.586087235467691130294144845693013, -0.405845151377397166906606412076961,
                                -0.207784955007898467600689403773245, 0.0};
__constant__ double c_gkw[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                                0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                                0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                                0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
__constant__ double c_gw[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                               0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

// segments of one adaptive integral: [a | b | I | E] arrays of `cap` entries in
// device scratch (the integral's slot of the launch), node values in shared memory
struct SegStore {
    double* a;
    double* b;
    double* I;
    double* E;
    long long cap;
    double* f;  // [32] shared
};

__device__ __forceinline__ SegStore seg_store(double* base, long long cap, long long slot, double* fsmem) {
    double* s = base + (size_t)slot * 4 * (size_t)cap;
    return SegStore{s, s + cap, s + 2 * cap, s + 3 * cap, cap, fsmem};
}

// node j of the 15-point rule on [a, b] (j < 7: a + (1 + x_j) s, j < 14: a + (1 - x_{j-7}) s, else a + s)
__device__ __forceinline__ double gk_node(int j, double a, double b) {
    const double s = 0.5 * (b - a);
    if (j < 7) return __dadd_rn(a, __dmul_rn(1 + c_gkx[j], s));
    if (j < 14) return __dadd_rn(a, __dmul_rn(1 - c_gkx[j - 7], s));
    return a + s;
}

// evalrule (QuadGK): Kronrod and Gauss sums in QuadGK's term order
__device__ __forceinline__ void gk_combine(const double* f, double a, double b, double& I, double& E) {
    const double s = 0.5 * (b - a);
    auto pair = [&](int k) { return f[k] + f[7 + k]; };
    double fg = pair(1), fk = pair(0);
    double Ig = fg * c_gw[0];
    double Ik = fg * c_gkw[1] + fk * c_gkw[0];
    for (int i = 2; i <= 3; ++i) {
        fg = pair(2 * i - 1);
        fk = pair(2 * i - 2);
        Ig += fg * c_gw[i - 1];
        Ik += fg * c_gkw[2 * i - 1] + fk * c_gkw[2 * i - 2];
    }
    const double f0 = f[14];
    Ig += f0 * c_gw[3];
    Ik += f0 * c_gkw[7] + pair(6) * c_gkw[6];
    const double Iks = Ik * s, Igs = Ig * s;
    I = Iks;
    E = fabs(Iks - Igs);
}

// coordinate map of the integration variable: mode 0 identity, 1 both ends
// infinite, 2 x = s0 - t/(1-t), 3 x = s0 + t/(1-t); returns f(x(t)) * dx/dt
template <class F>
__device__ __forceinline__ double mapped(const F& f, int mode, double s0, double t) {
    if (mode == 0) return f(t);
    if (mode == 1) {
        const double t2 = t * t;
        const double den = 1.0 / (1.0 - t2);
        return f(t * den) * (1.0 + t2) * den * den;
    }
    const double den = 1.0 / (1.0 - t);
    return (mode == 2 ? f(s0 - t * den) : f(s0 + t * den)) * den * den;
}

// One adaptive GK integral per warp.  pts are already mapped to t.
template <class F>
__device__ double warp_quadgk(const F& f, int mode, double s0, const double* pts, int npts, double atol,
                              double rtol, SegStore S, int* status) {
    const int lane = threadIdx.x & 31;
    const long long maxevals = 10000000;
    int nseg = npts - 1;
    // initial segments, two per pass
    for (int s = 0; s < nseg; s += 2) {
        const int seg = s + lane / 15;
        const int j = lane % 15;
        if (lane < 30 && seg < nseg) S.f[lane] = mapped(f, mode, s0, gk_node(j, pts[seg], pts[seg + 1]));
        __syncwarp();
        if (lane < 2 && s + lane < nseg) {
            const int sg = s + lane;
            S.a[sg] = pts[sg];
            S.b[sg] = pts[sg + 1];
            gk_combine(S.f + 15 * lane, pts[sg], pts[sg + 1], S.I[sg], S.E[sg]);
        }
        __syncwarp();
    }
    double I = S.I[0], E = S.E[0];
    for (int k = 1; k < nseg; ++k) {
        I += S.I[k];
        E += S.E[k];
    }
    long long numevals = 15ll * nseg;
    if (E <= atol || E <= rtol * fabs(I) || numevals >= maxevals) return I;
    while (E > atol && E > rtol * fabs(I) && numevals < maxevals) {
        // segment with the largest error (QuadGK pops the max of its heap)
        double best = -1.0;
        int bi = 0;
        for (int k = lane; k < nseg; k += 32) {
            if (S.E[k] > best) {
                best = S.E[k];
                bi = k;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(kFullMask, best, o);
            const int oi = __shfl_xor_sync(kFullMask, bi, o);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (nseg >= S.cap) {
            if (lane == 0) atomicOr(status, 1);
            break;
        }
        const double a = S.a[bi], b = S.b[bi], Iold = S.I[bi], Eold = S.E[bi];
        const double mid = 0.5 * (a + b);
        if (lane < 30) {
            const double lo = lane < 15 ? a : mid, hi = lane < 15 ? mid : b;
            S.f[lane] = mapped(f, mode, s0, gk_node(lane % 15, lo, hi));
        }
        __syncwarp();
        double I1, E1, I2, E2;
        gk_combine(S.f, a, mid, I1, E1);
        gk_combine(S.f + 15, mid, b, I2, E2);
        __syncwarp();
        if (lane == 0) {
            S.a[bi] = a;
            S.b[bi] = mid;
            S.I[bi] = I1;
            S.E[bi] = E1;
            S.a[nseg] = mid;
            S.b[nseg] = b;
            S.I[nseg] = I2;
            S.E[nseg] = E2;
        }
        __syncwarp();
        ++nseg;
        I = (I - Iold) + I1 + I2;
        E = (E - Eold) + E1 + E2;
        numevals += 30;
    }
    double Ir = S.I[0];
    for (int k = 1; k < nseg; ++k) Ir += S.I[k];
    return Ir;
}

// map the user points for the coordinate transformation (QuadGK handle_infinities)
__device__ inline int map_points(const double* x, int n, double* t, double& s0) {
    const bool inf1 = isinf(x[0]), inf2 = isinf(x[n - 1]);
    s0 = 0.0;
    if (inf1 && inf2) {
        for (int k = 0; k < n; ++k) t[k] = isinf(x[k]) ? copysign(1.0, x[k]) : 2.0 * x[k] / (1.0 + hypot(1.0, 2.0 * x[k]));
        return 1;
    }
    if (inf1 || inf2) {
        s0 = inf1 ? x[n - 1] : x[0];
        const double si = inf1 ? x[0] : x[n - 1];
        if (si < 0.0) {
            for (int k = 0; k < n; ++k) t[n - 1 - k] = 1.0 / (1.0 + 1.0 / (s0 - x[k]));
            return 2;
        }
        for (int k = 0; k < n; ++k) t[k] = 1.0 / (1.0 + 1.0 / (x[k] - s0));
        return 3;
    }
    for (int k = 0; k < n; ++k) t[k] = x[k];
    return 0;
}

// one component of the vertex at one site from the three channel plans
template <typename R>
__device__ __forceinline__ R site_value(const Layout& L, const R* __restrict__ src, const Plan<R>* pl, int mask,
                                        int c, int i, int ei) {
    R val = ldg(src + L.bare(c) + i);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const Plan<R>& P = pl[ch];
        if ((mask & (1 << ch)) && P.kernel) {
            R sgn;
            const int cs = comp_read(P, L.C, c, sgn);
            const R* q = src + L.qbase(cs, P.src_ch, P.kernel - 1);
            val += sgn * plan_read(P, q, P.exch ? ei : i);
        }
    }
    return val;
}

// self-energy kernels (flow_su2_self.jl:2-102, SDE_su2.jl:45-77; U(1)-DM:
// flow_u1_dm_self.jl:2-108, SDE_u1_dm.jl:59-91)
template <typename R>
struct SigmaKernel {
    const SigmaArgs<R>& A;
    const SMesh<R>& M;
    double w;
    __device__ double operator()(double xv) const {
        const Layout& L = A.L;
        const R v = (R)xv, w_ = (R)w, h = (R)0.5;
        const int kind = A.kind;
        Plan<R> p1[3], p2[3];
        int m_loc = CH_ALL, m_non = CH_ALL;
        const R* src = A.a;
        if (kind == SIG_SDE) {
            const R inf = (R)INFINITY;
            make_plan<R>(p1[0], 0, v + w_, inf, h * (v - w_), M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p2[0], 0, v + w_, inf, h * (-v + w_), M, L.Ns, L.NO, L.Nn);
            p1[1].kernel = p1[2].kernel = p2[1].kernel = p2[2].kernel = 0;
            m_loc = m_non = CH_S;
            src = A.aux;
        } else {
            make_plan<R>(p1[0], 0, v + w_, h * (-v + w_), h * (v - w_), M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p1[1], 1, (R)0, w_, v, M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p1[2], 2, -v + w_, h * (v + w_), h * (v + w_), M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p2[0], 0, v + w_, h * (-v + w_), h * (-v + w_), M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p2[1], 1, v - w_, h * (v + w_), h * (v + w_), M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p2[2], 2, (R)0, w_, v, M, L.Ns, L.NO, L.Nn);
            if (kind == SIG_CORR1) {
                src = A.aux;
                m_loc = CH_S | CH_T;
                m_non = CH_S | CH_U;
            }
        }
        const int e0 = ldg(A.exch);
        R val;
        if (L.C == 2) {
            val = (R)3 * site_value(L, src, p2, m_loc, 0, 0, e0) + site_value(L, src, p2, m_loc, 1, 0, e0);
            const R twoS = (R)A.twoS;
            for (int j = 0; j < L.Ns; ++j) {
                const int ej = ldg(A.exch + j);
                val -= (R)2 * (R)ldg(A.mult + j) * twoS * site_value(L, src, p1, m_non, 1, j, ej);
            }
        } else {
            // 2 Γxx + Γzz + Γdd on site 1, Γdd over the lattice
            val = (R)2 * site_value(L, src, p2, m_loc, 0, 0, e0) + site_value(L, src, p2, m_loc, 1, 0, e0) +
                  site_value(L, src, p2, m_loc, 3, 0, e0);
            for (int j = 0; j < L.Ns; ++j) {
                const int ej = ldg(A.exch + j);
                val -= (R)2 * (R)ldg(A.mult + j) * site_value(L, src, p1, m_non, 3, j, ej);
            }
        }
        const R Lam = (R)A.Lam;
        switch (kind) {
            case SIG_FLOW: val *= S_single(M, L.Nsig, A.a, Lam, v) / two_pi<R>(); break;
            case SIG_CORR1: val *= -G_full(M, L.Nsig, A.a, Lam, v) / two_pi<R>(); break;
            case SIG_CORR2: {
                const R g = G_full(M, L.Nsig, A.a, Lam, v);
                val *= g * g * get_sigma(M, L.Nsig, A.aux, v) / two_pi<R>();
                break;
            }
            default: val *= -G_full(M, L.Nsig, A.a, Lam, v) / two_pi<R>(); break;
        }
        return (double)val;
    }
};

template <typename R>
__global__ void __launch_bounds__(kSigWarps * 32) sigma_kernel(SigmaArgs<R> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SMesh<R>& M = *reinterpret_cast<SMesh<R>*>(smem_raw);
    double* fs = reinterpret_cast<double*>(smem_raw + sizeof(SMesh<R>));
    load_mesh(M, A.mesh, A.L.Nsig, A.L.NO, A.L.Nn);
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    const int i = 1 + blockIdx.x * kSigWarps + warp;  // σ index (index 0 is not computed)
    if (i >= A.L.Nsig) return;
    const SegStore S = seg_store(A.seg, A.seg_cap, i - 1, fs + 32 * warp);
    SigmaKernel<R> f{A, M, A.mesh[i]};
    const double L2 = 2.0 * A.Lam, inf = INFINITY;
    const double pts[5] = {-inf, -L2, 0.0, L2, inf};
    double t[5], s0;
    const int mode = map_points(pts, 5, t, s0);
    const double I = warp_quadgk(f, mode, s0, t, 5, A.atol, A.rtol, S, A.status);
    if ((threadIdx.x & 31) == 0) A.out[i] = I;
}

template <typename R>
cudaError_t launch_sigma(const SigmaArgs<R>& a, cudaStream_t st) {
    const int n = a.L.Nsig - 1;
    if (n <= 0) return cudaSuccess;
    const size_t smem = sizeof(SMesh<R>) + sizeof(double) * 32 * kSigWarps;
    cudaError_t e = cudaFuncSetAttribute(sigma_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    sigma_kernel<R><<<(n + kSigWarps - 1) / kSigWarps, kSigWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

// boundary corrections: one warp per (Ω index, channel, side)
template <typename R>
struct CorrKernel {
    const CorrsArgs<R>& A;
    const SMesh<R>& M;
    int ch;
    R Om;
    __device__ double operator()(double xv) const {
        const R v = (R)xv;
        R r = prop_half<R>(A.kind, 0, ch, M, A.Nsig, A.a, A.da, (R)A.Lam, v, Om);
        if (A.kind == 0) r += prop_half<R>(A.kind, 1, ch, M, A.Nsig, A.a, A.da, (R)A.Lam, v, Om);
        return (double)r;
    }
};

template <typename R>
__global__ void __launch_bounds__(kSigWarps * 32) corrs_kernel(CorrsArgs<R> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SMesh<R>& M = *reinterpret_cast<SMesh<R>*>(smem_raw);
    double* fs = reinterpret_cast<double*>(smem_raw + sizeof(SMesh<R>));
    load_mesh(M, A.mesh, A.Nsig, A.NO, A.Nn);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int job = blockIdx.x * kSigWarps + warp;
    if (job >= 6 * A.NO) return;
    const SegStore S = seg_store(A.seg, A.seg_cap, job, fs + 32 * warp);
    const int side = job & 1, ch = (job >> 1) % 3, i = (job >> 1) / 3;
    const double* Os = A.mesh + A.Nsig;
    const double* ns = Os + A.NO;
    const double* Ot = ns + A.Nn;
    const double* nt = Ot + A.NO;
    const double val = (ch == 1) ? Ot[A.NO - 1] + nt[A.Nn - 1] : Os[A.NO - 1] + ns[A.Nn - 1];
    const double Om = (ch == 1) ? Ot[i] : Os[i];
    CorrKernel<R> f{A, M, ch, (R)Om};
    const double bound = f(side == 0 ? -val : val);
    double res = 0.0;
    if (fabs(bound) > 1e-8) {
        const double inf = INFINITY;
        const double pts[2] = {side == 0 ? -inf : val, side == 0 ? -val : inf};
        double t[2], s0;
        const int mode = map_points(pts, 2, t, s0);
        res = warp_quadgk(f, mode, s0, t, 2, A.atol, A.rtol, S, A.status) / bound;
    }
    if (lane == 0) A.corrs[side + 2 * (ch + 3 * i)] = res;
}

template <typename R>
cudaError_t launch_corrs(const CorrsArgs<R>& a, cudaStream_t st) {
    const int n = 6 * a.NO;
    const size_t smem = sizeof(SMesh<R>) + sizeof(double) * 32 * kSigWarps;
    cudaError_t e = cudaFuncSetAttribute(corrs_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    corrs_kernel<R><<<(n + kSigWarps - 1) / kSigWarps, kSigWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// correlations χ (src/Observable/correlation_lib/correlation_lib.jl:2-30,
// correlation_su2.jl:14-87).  The reference integrates the vertex part over
// nine boxes of the compactified (v, v') plane with Cubature.jl's hcubature_v
// (compat 1.5, wrapping S. G. Johnson's cubature library, not in the
// reference tree); its published algorithm is restated: Genz-Malik
// degree-7/5 rule for dim = 2 (17 points, error |R7 - R5|), split along the
// dimension with the largest fourth difference, and per round the bisection
// of every largest-error region needed to bring the remaining error under
// max(atol, rtol |I|).  One block per (ω, site, component, box) integral;
// the regions live in device scratch (capacity per integral: ChiArgs::cap),
// the coordinates, rules and sums in FP64.
// ---------------------------------------------------------------------------
constexpr double kGL2 = 0.3585685828003180919906451539079374954541;  // sqrt(9/70)
constexpr double kGL4 = 0.9486832980505137995996680633298155601160;  // sqrt(9/10)
constexpr double kGL5 = 0.6882472016116852977216287342936235251269;  // sqrt(9/19)

// Regions of one integral.  The geometry, rule values and errors are indexed by
// region; the regions waiting to be cut are kept as a list sorted by error
// (largest first; equal errors in the order they were filed), in three buffers
// that take turns as the list, the round's new entries and the sort scratch.
struct ChiRegions {
    double* c0;
    double* c1;
    double* h0;
    double* h1;
    double* vol;
    double* val;
    double* err;
    int* split;                   // split dimension given by the region's last rule
    unsigned long long* key[3];   // list keys: ~bits(err), ascending = error descending
    int* idx[3];                  // list entries: region index
};

constexpr int kChiThreads = 256;   // one block per integral
constexpr int kChiChunk = 128;     // regions whose 17 points are evaluated per pass of the block
constexpr int kChiScan = 1024;     // list entries staged per step of the sequential sums
constexpr int kChiSumBlocks = 256; // blocks of the final sum (the oracle sums the same blocks)
constexpr int kSortItems = 8;      // list entries per thread and tile of the radix sort

// shared scratch of one integral; the phases of a round use it in turn
struct ChiScratch {
    union {
        double f[kChiChunk * 17];
        struct {
            double e[kChiScan];
            double v[kChiScan];
        } scan;
        struct {
            unsigned hist[8][256];
            unsigned base[256];
            unsigned cnt[kChiThreads / 32][256];
        } sort;
    };
    // the FP64 integrand's propagator factors of a chunk's regions: [region][7 x | 7 y] coordinates
    double gfac[kChiChunk * 14];
    unsigned wsum[kChiThreads / 32];
    double tot_val, tot_err;
    long long numeval;
    int K, done, over;
};

__device__ __forceinline__ unsigned long long err_key(double e) {
    return ~(unsigned long long)__double_as_longlong(e);  // e >= 0: bits ascending with e
}

// Stable LSD radix sort (8-bit digits) of cnt >= 1 (key, index) pairs by the block (entries
// read through L2: other blocks of a cluster may have written them), from
// (k0, i0) with (k1, i1) as scratch; digits shared by every key are skipped.  Returns the
// buffer that holds the result (0: k0/i0, 1: k1/i1).
__device__ int block_radix_sort(unsigned long long* k0, int* i0, unsigned long long* k1, int* i1, int cnt,
                                ChiScratch& S) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int q = tid; q < 8 * 256; q += kChiThreads) (&S.sort.hist[0][0])[q] = 0u;
    __syncthreads();
    for (int e = tid; e < cnt; e += kChiThreads) {
        const unsigned long long k = __ldcg(k0 + e);
#pragma unroll
        for (int d = 0; d < 8; ++d) atomicAdd(&S.sort.hist[d][(unsigned)(k >> (8 * d)) & 255u], 1u);
    }
    __syncthreads();
    int cur = 0;
    for (int d = 0; d < 8; ++d) {
        unsigned long long* ks = cur ? k1 : k0;
        int* is = cur ? i1 : i0;
        unsigned long long* kd = cur ? k0 : k1;
        int* id = cur ? i0 : i1;
        if (S.sort.hist[d][(unsigned)(__ldcg(ks) >> (8 * d)) & 255u] == (unsigned)cnt) continue;
        {  // exclusive prefix of the digit counts
            const unsigned x = S.sort.hist[d][tid];
            unsigned inc = x;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            if (lane == 31) S.wsum[warp] = inc;
            __syncthreads();
            unsigned off = 0;
            for (int w = 0; w < warp; ++w) off += S.wsum[w];
            S.sort.base[tid] = off + inc - x;
        }
        __syncthreads();
        unsigned* cw = S.sort.cnt[warp];
        for (int t0 = 0; t0 < cnt; t0 += kChiThreads * kSortItems) {
            for (int q = lane; q < 256; q += 32) cw[q] = 0u;
            __syncwarp();
            unsigned long long kk[kSortItems];
            int ii[kSortItems];
            unsigned dg[kSortItems], rk[kSortItems];
            // each warp ranks its 256 consecutive entries of the tile, in order
#pragma unroll
            for (int s = 0; s < kSortItems; ++s) {
                const int e = t0 + (warp * kSortItems + s) * 32 + lane;
                const bool ok = e < cnt;
                kk[s] = ok ? __ldcg(ks + e) : 0ull;
                ii[s] = ok ? __ldcg(is + e) : 0;
                dg[s] = ok ? ((unsigned)(kk[s] >> (8 * d)) & 255u) : 256u + (unsigned)lane;
                const unsigned peers = __match_any_sync(0xffffffffu, dg[s]);
                rk[s] = ok ? cw[dg[s]] + (unsigned)__popc(peers & lt) : 0u;
                __syncwarp();
                if (ok && (peers & lt) == 0u) cw[dg[s]] += (unsigned)__popc(peers);
                __syncwarp();
            }
            __syncthreads();
            {  // each digit's destinations: earlier tiles, then the warps in order
                unsigned run = S.sort.base[tid];
                for (int w = 0; w < kChiThreads / 32; ++w) {
                    const unsigned c = S.sort.cnt[w][tid];
                    S.sort.cnt[w][tid] = run;
                    run += c;
                }
                S.sort.base[tid] = run;
            }
            __syncthreads();
#pragma unroll
            for (int s = 0; s < kSortItems; ++s) {
                const int e = t0 + (warp * kSortItems + s) * 32 + lane;
                if (e < cnt) {
                    const unsigned p = cw[dg[s]] + rk[s];
                    kd[p] = kk[s];
                    id[p] = ii[s];
                }
            }
            __syncthreads();
        }
        cur ^= 1;
    }
    return cur;
}

// merge the sorted lists a[0, na) and b[0, nb) into o; equal keys: a's first (reads through L2)
__device__ void block_merge(const unsigned long long* ak, const int* ai, int na, const unsigned long long* bk,
                            const int* bi, int nb, unsigned long long* ok, int* oi) {
    const int n = na + nb;
    const int per = (n + kChiThreads - 1) / kChiThreads;
    const int d0 = min(n, (int)threadIdx.x * per), d1 = min(n, d0 + per);
    if (d0 < d1) {
        int lo = max(0, d0 - nb), hi = min(d0, na);
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldcg(ak + mid) <= __ldcg(bk + d0 - 1 - mid)) lo = mid + 1;
            else hi = mid;
        }
        int i = lo, j = d0 - lo;
        for (int d = d0; d < d1; ++d) {
            if (j >= nb || (i < na && __ldcg(ak + i) <= __ldcg(bk + j))) {
                ok[d] = __ldcg(ak + i);
                oi[d] = __ldcg(ai + i);
                ++i;
            } else {
                ok[d] = __ldcg(bk + j);
                oi[d] = __ldcg(bi + j);
                ++j;
            }
        }
    }
    __syncthreads();
}

// coordinate j of the seven a region's Genz-Malik points take along one axis (centre c, half width
// h): c, c - λ2 h, c + λ2 h, c - λ4 h, c + λ4 h, c - λ5 h, c + λ5 h (rounded products and sums, so
// that every use of a coordinate gets the same value)
__device__ __forceinline__ double gm_coord(int j, double c, double h) {
    if (j == 0) return c;
    const double off = __dmul_rn(h, j <= 2 ? kGL2 : (j <= 4 ? kGL4 : kGL5));
    return __dadd_rn(c, (j & 1) ? -off : off);
}

// the coordinates (indices of gm_coord) of point k of the 17, the library's order: the centre, the
// four points on each axis (-λ2, +λ2, -λ4, +λ4), the corners at λ4 ((-,-), (+,-), (+,+), (-,+)) and
// at λ5 ((+,+), (-,+), (-,-), (+,-))
__device__ __forceinline__ void gm_index(int k, int& xi, int& yi) {
    xi = yi = 0;
    if (k == 0) return;
    if (k <= 8) {
        const int d = (k - 1) >> 2, j = ((k - 1) & 3) + 1;
        if (d == 0) xi = j;
        else yi = j;
        return;
    }
    if (k <= 12) {
        const int q = k - 9;
        xi = (q == 1 || q == 2) ? 4 : 3;
        yi = q >= 2 ? 4 : 3;
        return;
    }
    const int q = k - 13;
    xi = (q == 0 || q == 3) ? 6 : 5;
    yi = q <= 1 ? 6 : 5;
}

// point k of the 17 Genz-Malik points of region (c, h), the library's order
__device__ __forceinline__ void gm_point(int k, double c0, double c1, double h0, double h1, double& x, double& y) {
    int xi, yi;
    gm_index(k, xi, yi);
    x = gm_coord(xi, c0, h0);
    y = gm_coord(yi, c1, h1);
}

// rule75genzmalik_evalError for dim = 2 on the 17 values v
__device__ __forceinline__ void gm_rule(const double* v, double vol, double& val, double& err, int& split) {
    const double n = 2.0;
    const double w1 = (12824.0 - 9120.0 * n + 400.0 * n * n) / 19683.0;
    const double w2 = 980.0 / 6561.0;
    const double w3 = (1820.0 - 400.0 * n) / 19683.0;
    const double w4 = 200.0 / 19683.0;
    const double w5 = 6859.0 / 19683.0 / 4.0;
    const double e1 = (729.0 - 950.0 * n + 50.0 * n * n) / 729.0;
    const double e2 = 245.0 / 486.0;
    const double e3 = (265.0 - 100.0 * n) / 1458.0;
    const double e4 = 25.0 / 729.0;
    const double ratio = (kGL2 * kGL2) / (kGL4 * kGL4);
    const double val0 = v[0];
    double sum2 = 0.0, sum3 = 0.0, diff[2];
    for (int d = 0; d < 2; ++d) {
        const double v0 = v[1 + 4 * d], v1 = v[2 + 4 * d], v2 = v[3 + 4 * d], v3 = v[4 + 4 * d];
        sum2 += v0 + v1;
        sum3 += v2 + v3;
        diff[d] = fabs(v0 + v1 - 2 * val0 - ratio * (v2 + v3 - 2 * val0));
    }
    double sum4 = 0.0, sum5 = 0.0;
    for (int q = 0; q < 4; ++q) sum4 += v[9 + q];
    for (int q = 0; q < 4; ++q) sum5 += v[13 + q];
    const double result = vol * (w1 * val0 + w2 * sum2 + w3 * sum3 + w4 * sum4 + w5 * sum5);
    const double res5 = vol * (e1 * val0 + e2 * sum2 + e3 * sum3 + e4 * sum4);
    val = result;
    err = fabs(res5 - result);
    split = diff[1] > diff[0] ? 1 : 0;
}

// compute_χ_kernel! (correlation_su2.jl:14-55) and compute_χ_kernel_{xx,zz,xy}!
// (correlation_u1_dm.jl:14-149, component k = 0, 1, 2) at (x, y) of [0,1]^2
// The integrand arithmetic runs in R (FP64, or FP32 on the FP32 copy of the state for
// the mixed path); the compactified coordinates and their Jacobians are formed in FP64.
template <typename R>
struct ChiKernel {
    static constexpr bool kSplit = true;  // core(x, y) * gfac(x) * gfac(y), see chi_eval_block
    const ChiArgs& A;
    const SMesh<R>& M;
    const R* a;  // the state in R
    int site;
    int k;
    double w;
    // G(v - ω/2) G(v + ω/2) dv/dx at the compactified coordinate x (and the same at y): the factors
    // that depend on one coordinate only
    __device__ R gfac(double x) const {
        const R v = (R)((2.0 * x - 1.0) / ((1.0 - x) * x));
        const R dv = (R)((2.0 * x * x - 2.0 * x + 1) / ((1.0 - x) * (1.0 - x) * x * x));
        const R wr = (R)w, h = (R)0.5;
        const R Lam = (R)A.Lam;
        return G_full(M, A.L.Nsig, a, Lam, v - h * wr) * G_full(M, A.L.Nsig, a, Lam, v + h * wr) * dv;
    }
    __device__ double operator()(double x, double y) const { return (double)(core(x, y) * gfac(x) * gfac(y)); }
    // the vertex part of the integrand; the integrand is (core * gfac(x)) * gfac(y)
    __device__ R core(double x, double y) const {
        const Layout& L = A.L;
        const R v = (R)((2.0 * x - 1.0) / ((1.0 - x) * x));
        const R vp = (R)((2.0 * y - 1.0) / ((1.0 - y) * y));
        const R wr = (R)w, h = (R)0.5;
        Plan<R> p1[3];
        make_plan<R>(p1[0], 0, v + vp, h * (v - wr - vp), h * (-v - wr + vp), M, L.Ns, L.NO, L.Nn);
        make_plan<R>(p1[1], 1, wr, v, vp, M, L.Ns, L.NO, L.Nn);
        make_plan<R>(p1[2], 2, v - vp, h * (v - wr + vp), h * (v + wr + vp), M, L.Ns, L.NO, L.Nn);
        const R twoS = (R)A.twoS;
        const R tp2 = two_pi<R>() * two_pi<R>();
        const int ei = ldg(A.exch + site);
        R val;
        if (L.C == 2) val = -(twoS * twoS) * site_value<R>(L, a, p1, CH_ALL, 0, site, ei) / tp2;
        else val = -site_value<R>(L, a, p1, CH_ALL, k, site, ei) / tp2;  // Γxx, Γzz, ΓDM
        if (site == 0) {
            Plan<R> p2[3];
            make_plan<R>(p2[0], 0, v + vp, h * (v - wr - vp), h * (v + wr - vp), M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p2[1], 1, -v + vp, h * (v - wr + vp), h * (v + wr + vp), M, L.Ns, L.NO, L.Nn);
            make_plan<R>(p2[2], 2, -wr, v, vp, M, L.Ns, L.NO, L.Nn);
            auto g = [&](int c) { return site_value<R>(L, a, p2, CH_ALL, c, 0, ei); };
            if (L.C == 2) {
                const R vs = g(0);
                const R vd = g(1);
                val -= twoS * (vs - vd) / ((R)2 * tp2);
            } else if (k == 0) {
                const R vzz = g(1), vdd = g(3);
                val -= (vzz - vdd) / ((R)2 * tp2);
            } else if (k == 1) {
                const R vxx = g(0), vzz = g(1), vdd = g(3);
                val -= ((R)2 * vxx - vzz - vdd) / ((R)2 * tp2);
            } else {
                const R vzd = g(4), vdz = g(5);
                val -= (vzd - vdz) / ((R)2 * tp2);
            }
        }
        return val;
    }
};

// The mixed path's χ integrand: FP32 vertex and propagator arithmetic on the FP32 copy of the
// state, with the node setup (plan arguments, interval searches, weights, propagator frequencies)
// in float-float arithmetic as in the quadrature passes, and plans near a buffer switch built in
// FP64 from the same FP64 arguments as the FP64 integrand.
struct ChiKernelFF {
    static constexpr bool kSplit = false;
    const ChiArgs& A;
    const MeshFF& M;
    const float* a;  // the FP32 copy of the state
    int site;
    int k;
    double w;
    __device__ void plan(Plan<float>& P, int ch, FF a0, FF a1, FF a2, double d0, double d1, double d2, FF v, FF vp,
                         FF wr) const {
        const Layout& L = A.L;
        const float scale = fabsf(v.h) + fabsf(vp.h) + fabsf(wr.h);
        if (ff_near_switch(a0, scale, M, L.NO, L.Nn) || ff_near_switch(a1, scale, M, L.NO, L.Nn) ||
            ff_near_switch(a2, scale, M, L.NO, L.Nn)) {
            const MeshG<double> M64 = mesh_view(A.mesh, L.Nsig, L.NO, L.Nn);
            make_plan<float>(P, ch, d0, d1, d2, M64, L.Ns, L.NO, L.Nn);
        } else {
            make_plan_ff(P, ch, a0, a1, a2, M, L.Ns, L.NO, L.Nn);
        }
    }
    __device__ float G(FF x, float Lam) const { return G_full_s(get_sigma_ff(M, A.L.Nsig, a, x), Lam, x.h); }
    __device__ double operator()(double x, double y) const {
        const Layout& L = A.L;
        const double vd = (2.0 * x - 1.0) / ((1.0 - x) * x);
        const double vpd = (2.0 * y - 1.0) / ((1.0 - y) * y);
        const float dv = (float)((2.0 * x * x - 2.0 * x + 1) / ((1.0 - x) * (1.0 - x) * x * x));
        const float dvp = (float)((2.0 * y * y - 2.0 * y + 1) / ((1.0 - y) * (1.0 - y) * y * y));
        const FF v(vd), vp(vpd), wr(w), h{0.5f, 0.f};
        const double hd = 0.5;
        Plan<float> p1[3];
        plan(p1[0], 0, v + vp, h * (v - wr - vp), h * (-v - wr + vp), vd + vpd, hd * (vd - w - vpd),
             hd * (-vd - w + vpd), v, vp, wr);
        plan(p1[1], 1, wr, v, vp, w, vd, vpd, v, vp, wr);
        plan(p1[2], 2, v - vp, h * (v - wr + vp), h * (v + wr + vp), vd - vpd, hd * (vd - w + vpd),
             hd * (vd + w + vpd), v, vp, wr);
        const float twoS = (float)A.twoS;
        const float tp2 = two_pi<float>() * two_pi<float>();
        const int ei = ldg(A.exch + site);
        float val;
        if (L.C == 2) val = -(twoS * twoS) * site_value<float>(L, a, p1, CH_ALL, 0, site, ei) / tp2;
        else val = -site_value<float>(L, a, p1, CH_ALL, k, site, ei) / tp2;
        if (site == 0) {
            Plan<float> p2[3];
            plan(p2[0], 0, v + vp, h * (v - wr - vp), h * (v + wr - vp), vd + vpd, hd * (vd - w - vpd),
                 hd * (vd + w - vpd), v, vp, wr);
            plan(p2[1], 1, -v + vp, h * (v - wr + vp), h * (v + wr + vp), -vd + vpd, hd * (vd - w + vpd),
                 hd * (vd + w + vpd), v, vp, wr);
            plan(p2[2], 2, -wr, v, vp, -w, vd, vpd, v, vp, wr);
            auto g = [&](int c) { return site_value<float>(L, a, p2, CH_ALL, c, 0, ei); };
            if (L.C == 2) {
                const float vs = g(0);
                const float vdd = g(1);
                val -= twoS * (vs - vdd) / (2.f * tp2);
            } else if (k == 0) {
                const float vzz = g(1), vdd = g(3);
                val -= (vzz - vdd) / (2.f * tp2);
            } else if (k == 1) {
                const float vxx = g(0), vzz = g(1), vdd = g(3);
                val -= (2.f * vxx - vzz - vdd) / (2.f * tp2);
            } else {
                const float vzd = g(4), vdz = g(5);
                val -= (vzd - vdz) / (2.f * tp2);
            }
        }
        const float Lam = (float)A.Lam;
        val *= G(v - h * wr, Lam) * G(v + h * wr, Lam) * dv;
        val *= G(vp - h * wr, Lam) * G(vp + h * wr, Lam) * dvp;
        return (double)val;
    }
};

// evaluate regions reg(e) of one integral, e in [0, count), the block taking every CL-th
// chunk of kChiChunk regions from chunk `first`: the 17 points of a chunk over all threads,
// then each region's rule; emit(e, r, err) sees every result.  Region records are read
// through L2 (other blocks of the cluster write them).
template <class F, class Reg, class Emit>
__device__ void chi_eval_block(const F& f, const ChiRegions& R, const Reg& reg, int count, int first, int stride,
                               ChiScratch& S, const Emit& emit) {
    const int tid = threadIdx.x;
    for (int cb = first * kChiChunk; cb < count; cb += stride * kChiChunk) {
        const int cnt = min(kChiChunk, count - cb);
        if constexpr (F::kSplit) {
            // the propagator factors depend on one coordinate: seven per axis and region instead of
            // four per point (the integrand is (core(x, y) gfac(x)) gfac(y) either way)
            for (int p = tid; p < cnt * 14; p += kChiThreads) {
                const int r = reg(cb + p / 14), j = p % 14;
                S.gfac[p] = j < 7 ? f.gfac(gm_coord(j, __ldcg(R.c0 + r), __ldcg(R.h0 + r)))
                                  : f.gfac(gm_coord(j - 7, __ldcg(R.c1 + r), __ldcg(R.h1 + r)));
            }
            __syncthreads();
            for (int p = tid; p < cnt * 17; p += kChiThreads) {
                const int q = p / 17, r = reg(cb + q);
                int xi, yi;
                gm_index(p % 17, xi, yi);
                const double x = gm_coord(xi, __ldcg(R.c0 + r), __ldcg(R.h0 + r));
                const double y = gm_coord(yi, __ldcg(R.c1 + r), __ldcg(R.h1 + r));
                S.f[p] = (double)(f.core(x, y) * S.gfac[14 * q + xi] * S.gfac[14 * q + 7 + yi]);
            }
        } else {
            for (int p = tid; p < cnt * 17; p += kChiThreads) {
                const int r = reg(cb + p / 17);
                double x, y;
                gm_point(p % 17, __ldcg(R.c0 + r), __ldcg(R.c1 + r), __ldcg(R.h0 + r), __ldcg(R.h1 + r), x, y);
                S.f[p] = f(x, y);
            }
        }
        __syncthreads();
        for (int q = tid; q < cnt; q += kChiThreads) {
            const int r = reg(cb + q);
            double val, err;
            int sp;
            gm_rule(S.f + 17 * q, __ldcg(R.vol + r), val, err, sp);
            R.val[r] = val;
            R.err[r] = err;
            R.split[r] = sp;
            emit(cb + q, r, err);
        }
        __syncthreads();
    }
}

// all threads of the cluster; writes before it are seen by every block of the cluster after it
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

// One integral of the job list per cluster of CL blocks (CL = 1: a single block).  A round
// takes the head of the sorted list (the library's pop order) while the remaining error is
// above the bound, cuts those regions, evaluates the halves with all blocks of the cluster,
// adds them in cut order, sorts them and merges them into the rest of the list.  Block 0 of
// the cluster keeps the list and the totals; the others only evaluate.  A job that runs out
// of region capacity raises its overflow flag and is run again with a larger capacity.
template <typename RT, int CL>
__global__ void __launch_bounds__(kChiThreads, 1) chi_box_kernel(ChiArgs A, const int* __restrict__ jobs,
                                                                   int njobs, int* overflow) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // the meshes: FP64 SMesh (FP64 integrand) or the float-float block (mixed integrand)
    ChiScratch& S = *reinterpret_cast<ChiScratch*>(smem_raw + sizeof(SMesh<double>));
    const int nm = A.L.Nsig + 2 * A.L.NO + 2 * A.L.Nn;
    if constexpr (sizeof(RT) == 8) {
        load_mesh(*reinterpret_cast<SMesh<double>*>(smem_raw), A.mesh, A.L.Nsig, A.L.NO, A.L.Nn);
    } else {
        float* mf = reinterpret_cast<float*>(smem_raw);
        for (int q = threadIdx.x; q < 3 * nm + kMeshGuess; q += blockDim.x) mf[q] = ldg(A.mesh_ff + q);
    }
    const int tid = threadIdx.x;
    const long long slot = blockIdx.x / CL;
    const int rank = (int)(blockIdx.x % CL);  // the cluster's blocks are consecutive in x
    const bool lead = rank == 0;
    const long long job = jobs[slot];
    // job = ((ω index * Ns + site) * ncomp + component) * 9 + box
    const int box = (int)(job % 9);
    const long long rj = job / 9;
    const int k = (int)(rj % A.ncomp);
    const int site = (int)((rj / A.ncomp) % A.L.Ns), wi = (int)(rj / ((long long)A.ncomp * A.L.Ns));
    const double wv = A.chi_mesh[wi];
    // integrate_χ_boxes: the nine boxes around the image of ±width = ±4 (Λ + ω / 2)
    const double width = 4.0 * (A.Lam + 0.5 * wv);
    const double wp = (width - 2.0 + sqrt(width * width + 4.0)) / (2.0 * width);
    const double s = fabs(wp - 0.5);
    const double lo[3] = {0.0, 0.5 - s, 0.5 + s}, hi[3] = {0.5 - s, 0.5 + s, 1.0};
    const int row = 2 - box / 3, col = box % 3;  // the reference's order: top line first
    ChiRegions R;
    const long long cap = A.cap;
    {
        double* d = A.reg + (size_t)slot * cap * 10;
        int* i = A.reg_split + (size_t)slot * cap * 4;
        R.c0 = d;
        R.c1 = d + cap;
        R.h0 = d + 2 * cap;
        R.h1 = d + 3 * cap;
        R.vol = d + 4 * cap;
        R.val = d + 5 * cap;
        R.err = d + 6 * cap;
        R.split = i;
        for (int b = 0; b < 3; ++b) {
            R.key[b] = reinterpret_cast<unsigned long long*>(d + (7 + b) * cap);
            R.idx[b] = i + (1 + b) * cap;
        }
    }
    int* ctl = A.ctl + slot * 4;  // the round's orders to the cluster: stop, K, first new region, list
    const MeshFF MF = mesh_view_ff(reinterpret_cast<const float*>(smem_raw), A.L.Nsig, A.L.NO, A.L.Nn);
    using Kern = typename std::conditional<sizeof(RT) == 8, ChiKernel<double>, ChiKernelFF>::type;
    const Kern f = [&]() {
        if constexpr (sizeof(RT) == 8)
            return ChiKernel<double>{A, *reinterpret_cast<const SMesh<double>*>(smem_raw), A.a, site, k, wv};
        else
            return ChiKernelFF{A, MF, A.af, site, k, wv};
    }();
    if (lead && tid == 0) {
        R.c0[0] = 0.5 * (lo[col] + hi[col]);
        R.c1[0] = 0.5 * (lo[row] + hi[row]);
        R.h0[0] = 0.5 * (hi[col] - lo[col]);
        R.h1[0] = 0.5 * (hi[row] - lo[row]);
        R.vol[0] = (2.0 * R.h0[0]) * (2.0 * R.h1[0]);
    }
    __syncthreads();  // the mesh and region 0
    int cur = 0;
    int n = 1, m = 1;  // regions; list length (every region is on the list between rounds)
    long long rounds = 0;
    const long long maxevals = 10000000;
    auto converged = [&](double err, double val) { return !(err > A.atol && err > fabs(val) * A.rtol); };
    if (lead) {
        chi_eval_block(f, R, [](int) { return 0; }, 1, 0, 1, S, [&](int, int r, double e) {
            R.key[cur][0] = err_key(e);
            R.idx[cur][0] = r;
        });
        if (tid == 0) {
            S.tot_val = __ldcg(R.val);
            S.tot_err = __ldcg(R.err);
            S.numeval = 17;
            S.over = 0;
        }
        __syncthreads();
    }
    for (;;) {
        int stop = 0, K = 0, n0 = n;
        if (lead) {
            stop = S.numeval >= maxevals || converged(S.tot_err, S.tot_val);
            if (!stop) {
                ++rounds;
                // 1. the pops: list head while the remaining error is above the bound
                double ee_err = S.tot_err;
                const double ee_val = S.tot_val;
                for (int b0 = 0;; b0 += kChiScan) {
                    const int nb = min(kChiScan, m - b0);
                    for (int t = tid; t < nb; t += kChiThreads) {
                        const int q = R.idx[cur][b0 + t];
                        S.scan.e[t] = __ldcg(R.err + q);
                        S.scan.v[t] = __ldcg(R.val + q);
                    }
                    __syncthreads();
                    if (tid == 0) {
                        int done = 0;
                        double tv = S.tot_val, te = S.tot_err;
                        long long ne = S.numeval;
                        for (int t = 0; t < nb; ++t) {
                            if (n0 + K + 1 > cap) {
                                S.over = 1;
                                done = 1;
                                break;
                            }
                            tv -= S.scan.v[t];
                            te -= S.scan.e[t];
                            ee_err -= S.scan.e[t];
                            ++K;
                            ne += 34;
                            if (converged(ee_err, ee_val) || K >= m || ne >= maxevals) {
                                done = 1;
                                break;
                            }
                        }
                        S.tot_val = tv;
                        S.tot_err = te;
                        S.numeval = ne;
                        S.K = K;
                        S.done = done;
                    }
                    __syncthreads();
                    if (S.done) break;
                }
                K = S.K;
                stop = S.over;
            }
            if (!stop) {
                // 2. cut: the first half keeps the index, the second half is region n0 + j
                for (int j = tid; j < K; j += kChiThreads) {
                    const int bi = R.idx[cur][j], q = n0 + j;
                    const int d = __ldcg(R.split + bi);
                    double c0 = R.c0[bi], c1 = R.c1[bi], h0 = R.h0[bi], h1 = R.h1[bi];
                    double cq0 = c0, cq1 = c1;
                    if (d == 0) {
                        h0 *= 0.5;
                        c0 -= h0;
                        cq0 += h0;
                    } else {
                        h1 *= 0.5;
                        c1 -= h1;
                        cq1 += h1;
                    }
                    R.c0[bi] = c0;
                    R.c1[bi] = c1;
                    R.h0[bi] = h0;
                    R.h1[bi] = h1;
                    R.vol[bi] *= 0.5;
                    R.c0[q] = cq0;
                    R.c1[q] = cq1;
                    R.h0[q] = h0;
                    R.h1[q] = h1;
                    R.vol[q] = (2.0 * h0) * (2.0 * h1);
                }
            }
            if (CL > 1 && tid == 0) {
                ctl[0] = stop;
                ctl[1] = K;
                ctl[2] = n0;
                ctl[3] = cur;
            }
        }
        if constexpr (CL > 1) {
            cluster_barrier();
            stop = __ldcg(ctl);
            K = __ldcg(ctl + 1);
            n0 = __ldcg(ctl + 2);
            cur = __ldcg(ctl + 3);
        } else {
            __syncthreads();
        }
        if (stop) break;
        // 3. evaluate the halves in cut order (j's first half, j's second half, ...) into list b1
        const int b1 = (cur + 1) % 3, b2 = (cur + 2) % 3;
        const int* head = R.idx[cur];
        auto cut = [head, n0](int e) { return (e & 1) ? n0 + (e >> 1) : __ldcg(head + (e >> 1)); };
        unsigned long long* nk = R.key[b1];
        int* ni = R.idx[b1];
        chi_eval_block(f, R, cut, 2 * K, rank, CL, S, [&](int e, int r, double err) {
            nk[e] = err_key(err);
            ni[e] = r;
        });
        if constexpr (CL > 1) cluster_barrier();
        if (!lead) continue;
        // 4. the new regions join the totals in cut order
        for (int b0 = 0; b0 < 2 * K; b0 += kChiScan) {
            const int nb = min(kChiScan, 2 * K - b0);
            for (int t = tid; t < nb; t += kChiThreads) {
                const int r = cut(b0 + t);
                S.scan.e[t] = __ldcg(R.err + r);
                S.scan.v[t] = __ldcg(R.val + r);
            }
            __syncthreads();
            if (tid == 0) {
                double tv = S.tot_val, te = S.tot_err;
                for (int t = 0; t < nb; ++t) {
                    tv += S.scan.v[t];
                    te += S.scan.e[t];
                }
                S.tot_val = tv;
                S.tot_err = te;
            }
            __syncthreads();
        }
        // 5. sort them and merge them after equal errors of the rest of the list
        const int in_b2 = block_radix_sort(nk, ni, R.key[b2], R.idx[b2], 2 * K, S);
        const int bs = in_b2 ? b2 : b1, bo = in_b2 ? b1 : b2;
        block_merge(R.key[cur] + K, R.idx[cur] + K, m - K, R.key[bs], R.idx[bs], 2 * K, R.key[bo], R.idx[bo]);
        cur = bo;
        m += K;
        n = n0 + K;
    }
    if (!lead) return;
    // the total: kChiSumBlocks consecutive blocks of regions, each summed in index order
    const int over = S.over;
    __syncthreads();
    static_assert(kChiSumBlocks == kChiThreads, "one block of the sum per thread");
    {
        const int c = (n + kChiSumBlocks - 1) / kChiSumBlocks;
        const int q0 = min(n, tid * c), q1 = min(n, q0 + c);
        double p = 0.0;
        for (int q = q0; q < q1; ++q) p += __ldcg(R.val + q);
        S.f[tid] = p;
    }
    __syncthreads();
    if (tid == 0) {
        double I = 0.0;
        for (int t = 0; t < kChiSumBlocks; ++t) I += S.f[t];
        A.box_out[job] = I;
        overflow[slot] = over ? 1 : -n;  // the regions the integral needed, when it fitted
        if (A.evals && !over) {
            atomicAdd(A.evals, (unsigned long long)S.numeval);
            atomicMax(A.evals + 1, (unsigned long long)n);
            atomicAdd(A.evals + 2, (unsigned long long)rounds);
            atomicMax(A.evals + 3, (unsigned long long)rounds);
        }
    }
}

// local term (correlation_su2.jl:77-81) and the sum of the nine boxes
__global__ void __launch_bounds__(kSigWarps * 32) chi_local_kernel(ChiArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SMesh<double>& M = *reinterpret_cast<SMesh<double>*>(smem_raw);
    double* fs = reinterpret_cast<double*>(smem_raw + sizeof(SMesh<double>));
    load_mesh(M, A.mesh, A.L.Nsig, A.L.NO, A.L.Nn);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wi = blockIdx.x * kSigWarps + warp;
    if (wi >= A.num_chi) return;
    const SegStore S = seg_store(A.seg, A.seg_cap, wi, fs + 32 * warp);
    const double wv = A.chi_mesh[wi];
    const double ref = A.Lam + 0.5 * wv;
    struct G2 {
        const ChiArgs& A;
        const SMesh<double>& M;
        double w;
        __device__ double operator()(double v) const {
            const double pref = A.L.C == 2 ? A.twoS : 1.0;
            return pref * G_full(M, A.L.Nsig, A.a, A.Lam, v - 0.5 * w) * G_full(M, A.L.Nsig, A.a, A.Lam, v + 0.5 * w) /
                   (2.0 * two_pi<double>());
        }
    } g{A, M, wv};
    const double inf = INFINITY;
    const double pts[5] = {-inf, -2.0 * ref, 0.0, 2.0 * ref, inf};
    double t[5], s0;
    const int mode = map_points(pts, 5, t, s0);
    const double loc = warp_quadgk(g, mode, s0, t, 5, A.atol, A.rtol, S, A.status);
    if (lane == 0) {
        const size_t plane = (size_t)A.L.Ns * A.num_chi;
        for (int i = 0; i < A.L.Ns; ++i) {
            for (int k = 0; k < A.ncomp; ++k) {
                const double* b = A.box_out + (((size_t)wi * A.L.Ns + i) * A.ncomp + k) * 9;
                double c = b[0];
                for (int q = 1; q < 9; ++q) c += b[q];
                if (i == 0 && k < 2) c += loc;  // χ (SU(2)) or χxx and χzz (U(1)-DM)
                A.chi[k * plane + i + (size_t)A.L.Ns * wi] = c;
            }
        }
    }
}

template <typename R, int CL>
static cudaError_t launch_chi_boxes_r(const ChiArgs& a, const int* jobs, int njobs, int* overflow, cudaStream_t st) {
    static_assert(sizeof(SMesh<double>) >= 3 * sizeof(float) * 5 * kMaxMesh, "float-float meshes fit");
    const size_t smem = sizeof(SMesh<double>) + sizeof(ChiScratch);
    auto kern = chi_box_kernel<R, CL>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (CL > 8) {  // clusters beyond the portable size of 8 blocks
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)njobs * CL);
    cfg.blockDim = dim3(kChiThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a, jobs, njobs, overflow);
}

cudaError_t launch_chi_boxes(const ChiArgs& a, const int* jobs, int njobs, int* overflow, int cluster,
                             cudaStream_t st) {
    if (cluster >= 16)
        return a.af ? launch_chi_boxes_r<float, 16>(a, jobs, njobs, overflow, st)
                    : launch_chi_boxes_r<double, 16>(a, jobs, njobs, overflow, st);
    if (cluster > 1)
        return a.af ? launch_chi_boxes_r<float, 8>(a, jobs, njobs, overflow, st)
                    : launch_chi_boxes_r<double, 8>(a, jobs, njobs, overflow, st);
    return a.af ? launch_chi_boxes_r<float, 1>(a, jobs, njobs, overflow, st)
                : launch_chi_boxes_r<double, 1>(a, jobs, njobs, overflow, st);
}

cudaError_t launch_chi_sum(const ChiArgs& a, cudaStream_t st) {
    const size_t smem2 = sizeof(SMesh<double>) + sizeof(double) * 32 * kSigWarps;
    cudaError_t e = cudaFuncSetAttribute(chi_local_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
    if (e != cudaSuccess) return e;
    chi_local_kernel<<<(a.num_chi + kSigWarps - 1) / kSigWarps, kSigWarps * 32, smem2, st>>>(a);
    return cudaGetLastError();
}

template cudaError_t launch_sigma<double>(const SigmaArgs<double>&, cudaStream_t);
template cudaError_t launch_corrs<double>(const CorrsArgs<double>&, cudaStream_t);

}  // namespace pffrg

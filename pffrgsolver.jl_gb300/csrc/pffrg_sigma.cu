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
// max(atol, rtol |I|).  One warp per (ω, site, box) integral, FP64; the
// regions live in device scratch (capacity per integral: chi_cap).
// ---------------------------------------------------------------------------
constexpr double kGL2 = 0.3585685828003180919906451539079374954541;  // sqrt(9/70)
constexpr double kGL4 = 0.9486832980505137995996680633298155601160;  // sqrt(9/10)
constexpr double kGL5 = 0.6882472016116852977216287342936235251269;  // sqrt(9/19)

struct ChiRegions {
    double* c0;
    double* c1;
    double* h0;
    double* h1;
    double* vol;
    double* val;
    double* err;
    int* split;    // bit 0: split dimension; bits 1+: the region the second half of a cut was cut from
    double* hkey;  // max-heap of region indices keyed by error
    int* hidx;
};

// region heap of one integral: 32 children per node, the oracle's sift rules.  push runs on
// lane 0; pop is warp-collective, one lane per child of the node being sifted.
constexpr int kHeapD = 32;

__device__ __forceinline__ void heap_push(ChiRegions& R, int& hn, double k, int i) {
    int h = hn++;
    while (h > 0) {
        const int p = (h - 1) / kHeapD;
        if (R.hkey[p] >= k) break;
        R.hkey[h] = R.hkey[p];
        R.hidx[h] = R.hidx[p];
        h = p;
    }
    R.hkey[h] = k;
    R.hidx[h] = i;
}

__device__ __forceinline__ int heap_pop_warp(ChiRegions& R, int& hn) {
    const int lane = threadIdx.x & 31;
    const int top = R.hidx[0];
    const int n = --hn;
    const double k = R.hkey[n];
    const int i = R.hidx[n];
    __syncwarp();
    int h = 0;
    if (n > 0) {
        for (;;) {
            const int c0 = kHeapD * h + 1;
            if (c0 >= n) break;
            const int c = c0 + lane;
            double best = (c < n) ? R.hkey[c] : -1.0;
            int bc = (c < n) ? c : 0x7fffffff;
            // the largest child, the first of equal largest keys
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oc = __shfl_xor_sync(0xffffffffu, bc, o);
                if (ob > best || (ob == best && oc < bc)) {
                    best = ob;
                    bc = oc;
                }
            }
            if (best <= k) break;
            if (lane == 0) {
                R.hkey[h] = best;
                R.hidx[h] = R.hidx[bc];
            }
            __syncwarp();
            h = bc;
        }
        if (lane == 0) {
            R.hkey[h] = k;
            R.hidx[h] = i;
        }
    }
    __syncwarp();
    return top;
}

// point k of the 17 Genz-Malik points of region (c, h), the library's order
__device__ __forceinline__ void gm_point(int k, double c0, double c1, double h0, double h1, double& x, double& y) {
    x = c0;
    y = c1;
    if (k == 0) return;
    if (k <= 8) {
        const int d = (k - 1) >> 2, q = (k - 1) & 3;
        const double hw = d == 0 ? h0 : h1;
        const double off = (q < 2 ? hw * kGL2 : hw * kGL4) * ((q & 1) ? 1.0 : -1.0);
        if (d == 0) x = c0 + off;
        else y = c1 + off;
        return;
    }
    if (k <= 12) {
        const double a = h0 * kGL4, b = h1 * kGL4;
        const int q = k - 9;  // (-,-), (+,-), (+,+), (-,+)
        x = c0 + ((q == 1 || q == 2) ? a : -a);
        y = c1 + ((q >= 2) ? b : -b);
        return;
    }
    const double a = h0 * kGL5, b = h1 * kGL5;
    const int q = k - 13;  // (+,+), (-,+), (-,-), (+,-)
    x = c0 + ((q == 0 || q == 3) ? a : -a);
    y = c1 + ((q <= 1) ? b : -b);
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
    const ChiArgs& A;
    const SMesh<R>& M;
    const R* a;  // the state in R
    int site;
    int k;
    double w;
    __device__ double operator()(double x, double y) const {
        const Layout& L = A.L;
        const R v = (R)((2.0 * x - 1.0) / ((1.0 - x) * x));
        const R vp = (R)((2.0 * y - 1.0) / ((1.0 - y) * y));
        const R dv = (R)((2.0 * x * x - 2.0 * x + 1) / ((1.0 - x) * (1.0 - x) * x * x));
        const R dvp = (R)((2.0 * y * y - 2.0 * y + 1) / ((1.0 - y) * (1.0 - y) * y * y));
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
        const R Lam = (R)A.Lam;
        val *= G_full(M, L.Nsig, a, Lam, v - h * wr) * G_full(M, L.Nsig, a, Lam, v + h * wr) * dv;
        val *= G_full(M, L.Nsig, a, Lam, vp - h * wr) * G_full(M, L.Nsig, a, Lam, vp + h * wr) * dvp;
        return (double)val;
    }
};

// evaluate the pending regions [first, first + count) of one integral (17 points each over the lanes)
template <class F>
__device__ void chi_eval_regions(const F& f, ChiRegions R, const int* idx, int count, double* fbuf) {
    const int lane = threadIdx.x & 31;
    for (int base = 0; base < count * 17; base += 32) {
        const int e = base + lane;
        if (e < count * 17) {
            const int r = idx[e / 17], k = e % 17;
            double x, y;
            gm_point(k, R.c0[r], R.c1[r], R.h0[r], R.h1[r], x, y);
            fbuf[e] = f(x, y);
        }
    }
    __syncwarp();
    for (int q = lane; q < count; q += 32) {
        const int r = idx[q];
        double val, err;
        int sp;
        gm_rule(fbuf + 17 * q, R.vol[r], val, err, sp);
        R.val[r] = val;
        R.err[r] = err;
        R.split[r] = (R.split[r] & ~1) | sp;
    }
    __syncwarp();
}

constexpr int kChiWarps = 2;
constexpr int kChiPend = 64;  // regions evaluated per batch

// One warp per (ω, site, component, box) integral of the job list; a job that
// runs out of region capacity raises its overflow flag and is run again with a
// larger capacity.
template <typename RT>
__global__ void __launch_bounds__(kChiWarps * 32) chi_box_kernel(ChiArgs A, const int* __restrict__ jobs, int njobs,
                                                                  int* overflow) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SMesh<RT>& M = *reinterpret_cast<SMesh<RT>*>(smem_raw);
    double* fb = reinterpret_cast<double*>(smem_raw + sizeof(SMesh<RT>));
    int* pend = reinterpret_cast<int*>(fb + kChiWarps * kChiPend * 17);
    load_mesh(M, A.mesh, A.L.Nsig, A.L.NO, A.L.Nn);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long slot = (long long)blockIdx.x * kChiWarps + warp;
    if (slot >= njobs) return;
    const long long job = jobs[slot];
    double* fbuf = fb + warp * kChiPend * 17;
    int* pidx = pend + warp * kChiPend;
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
    const size_t cap = A.cap;
    const size_t off = (size_t)slot * cap;
    R.c0 = A.reg + off * 8;
    R.c1 = R.c0 + cap;
    R.h0 = R.c1 + cap;
    R.h1 = R.h0 + cap;
    R.vol = R.h1 + cap;
    R.val = R.vol + cap;
    R.err = R.val + cap;
    R.hkey = R.err + cap;
    R.split = A.reg_split + off * 2;
    R.hidx = R.split + cap;
    const RT* state;
    if constexpr (sizeof(RT) == 8) state = A.a;
    else state = A.af;
    ChiKernel<RT> f{A, M, state, site, k, wv};
    if (lane == 0) {
        R.c0[0] = 0.5 * (lo[col] + hi[col]);
        R.c1[0] = 0.5 * (lo[row] + hi[row]);
        R.h0[0] = 0.5 * (hi[col] - lo[col]);
        R.h1[0] = 0.5 * (hi[row] - lo[row]);
        R.vol[0] = (2.0 * R.h0[0]) * (2.0 * R.h1[0]);
        R.split[0] = 0;
        pidx[0] = 0;
    }
    __syncwarp();
    chi_eval_regions(f, R, pidx, 1, fbuf);
    int n = 1, hn = 0;
    if (lane == 0) heap_push(R, hn, R.err[0], 0);
    hn = __shfl_sync(0xffffffffu, hn, 0);  // the heap size is kept uniform across the warp
    __syncwarp();
    double tot_val = R.val[0], tot_err = R.err[0];
    long long numeval = 17;
    const long long maxevals = 10000000;
    bool over = false;
    long long rounds = 0;
    auto converged = [&](double err, double val) { return !(err > A.atol && err > fabs(val) * A.rtol); };
    while (numeval < maxevals) {
        if (converged(tot_err, tot_val)) break;
        ++rounds;
        double ee_err = tot_err;
        const double ee_val = tot_val;
        const int n0 = n;
        int npend = 0;
        // pop the largest-error regions (the library's parallel mode) and halve each
        do {
            if (n + 1 > (int)cap) {
                over = true;
                break;
            }
            const int bi = heap_pop_warp(R, hn);
            const double pv = R.val[bi], pe = R.err[bi];
            tot_val -= pv;
            tot_err -= pe;
            ee_err -= pe;
            if (lane == 0) {
                const int d = R.split[bi] & 1;
                R.c0[n] = R.c0[bi];
                R.c1[n] = R.c1[bi];
                R.h0[n] = R.h0[bi];
                R.h1[n] = R.h1[bi];
                if (d == 0) {
                    R.h0[bi] *= 0.5;
                    R.h0[n] = R.h0[bi];
                    R.c0[bi] -= R.h0[bi];
                    R.c0[n] += R.h0[bi];
                } else {
                    R.h1[bi] *= 0.5;
                    R.h1[n] = R.h1[bi];
                    R.c1[bi] -= R.h1[bi];
                    R.c1[n] += R.h1[bi];
                }
                R.vol[bi] *= 0.5;
                R.vol[n] = (2.0 * R.h0[n]) * (2.0 * R.h1[n]);
                R.split[bi] = 0;
                R.split[n] = bi << 1;
                pidx[npend] = bi;
                pidx[npend + 1] = n;
            }
            __syncwarp();
            npend += 2;
            ++n;
            numeval += 34;
            if (converged(ee_err, ee_val)) break;
            if (npend + 2 > kChiPend) {
                chi_eval_regions(f, R, pidx, npend, fbuf);
                npend = 0;
            }
        } while (hn > 0 && numeval < maxevals);
        if (npend) chi_eval_regions(f, R, pidx, npend, fbuf);
        // the round's regions join the heap, in the order they were cut
        for (int q = n0; q < n; ++q) {
            const int tw = R.split[q] >> 1;
            tot_val += R.val[tw];
            tot_err += R.err[tw];
            tot_val += R.val[q];
            tot_err += R.err[q];
            if (lane == 0) {
                heap_push(R, hn, R.err[tw], tw);
                heap_push(R, hn, R.err[q], q);
            }
        }
        hn = __shfl_sync(0xffffffffu, hn, 0);
        __syncwarp();
        if (over) break;
    }
    // the total in heap order, as the library sums it
    double I = 0.0;
    if (lane == 0) {
        for (int q = 0; q < hn; ++q) I += R.val[R.hidx[q]];
        A.box_out[job] = I;
        overflow[slot] = over ? 1 : 0;
        if (A.evals && !over) {
            atomicAdd(A.evals, (unsigned long long)numeval);
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

template <typename R>
static cudaError_t launch_chi_boxes_r(const ChiArgs& a, const int* jobs, int njobs, int* overflow, cudaStream_t st) {
    const size_t smem = sizeof(SMesh<R>) + sizeof(double) * kChiWarps * kChiPend * 17 + sizeof(int) * kChiWarps * kChiPend;
    cudaError_t e = cudaFuncSetAttribute(chi_box_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    chi_box_kernel<R><<<(unsigned)((njobs + kChiWarps - 1) / kChiWarps), kChiWarps * 32, smem, st>>>(a, jobs, njobs,
                                                                                                      overflow);
    return cudaGetLastError();
}

cudaError_t launch_chi_boxes(const ChiArgs& a, const int* jobs, int njobs, int* overflow, cudaStream_t st) {
    return a.af ? launch_chi_boxes_r<float>(a, jobs, njobs, overflow, st)
                : launch_chi_boxes_r<double>(a, jobs, njobs, overflow, st);
}

cudaError_t launch_chi_sum(const ChiArgs& a, cudaStream_t st) {
    const size_t smem2 = sizeof(SMesh<double>) + sizeof(double) * 32 * kSigWarps;
    cudaError_t e = cudaFuncSetAttribute(chi_local_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
    if (e != cudaSuccess) return e;
    chi_local_kernel<<<(a.num_chi + kSigWarps - 1) / kSigWarps, kSigWarps * 32, smem2, st>>>(a);
    return cudaGetLastError();
}

template cudaError_t launch_sigma<double>(const SigmaArgs<double>&, cudaStream_t);
template cudaError_t launch_sigma<float>(const SigmaArgs<float>&, cudaStream_t);
template cudaError_t launch_corrs<double>(const CorrsArgs<double>&, cudaStream_t);
template cudaError_t launch_corrs<float>(const CorrsArgs<float>&, cudaStream_t);

}  // namespace pffrg

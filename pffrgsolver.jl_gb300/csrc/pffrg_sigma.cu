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
constexpr int kMaxSeg = 384;

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

struct SegStore {
    double a[kMaxSeg], b[kMaxSeg], I[kMaxSeg], E[kMaxSeg];
    double f[32];
};

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
                              double rtol, SegStore& S, int* status) {
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
        if (nseg >= kMaxSeg) {
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
            const R* q = src + L.qbase(c, P.src_ch, P.kernel - 1);
            val += (c == 1 ? P.sgn_d : (R)1) * plan_read(P, q, P.exch ? ei : i);
        }
    }
    return val;
}

// self-energy kernels (flow_su2_self.jl:2-102, SDE_su2.jl:45-77)
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
        R val = (R)3 * site_value(L, src, p2, m_loc, 0, 0, e0) + site_value(L, src, p2, m_loc, 1, 0, e0);
        const R twoS = (R)A.twoS;
        for (int j = 0; j < L.Ns; ++j) {
            const int ej = ldg(A.exch + j);
            val -= (R)2 * (R)ldg(A.mult + j) * twoS * site_value(L, src, p1, m_non, 1, j, ej);
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
    SegStore* segs = reinterpret_cast<SegStore*>(smem_raw + sizeof(SMesh<R>));
    load_mesh(M, A.mesh, A.L.Nsig, A.L.NO, A.L.Nn);
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    const int i = 1 + blockIdx.x * kSigWarps + warp;  // σ index (index 0 is not computed)
    if (i >= A.L.Nsig) return;
    SigmaKernel<R> f{A, M, A.mesh[i]};
    const double L2 = 2.0 * A.Lam, inf = INFINITY;
    const double pts[5] = {-inf, -L2, 0.0, L2, inf};
    double t[5], s0;
    const int mode = map_points(pts, 5, t, s0);
    const double I = warp_quadgk(f, mode, s0, t, 5, A.atol, A.rtol, segs[warp], A.status);
    if ((threadIdx.x & 31) == 0) A.out[i] = I;
}

template <typename R>
cudaError_t launch_sigma(const SigmaArgs<R>& a, cudaStream_t st) {
    const int n = a.L.Nsig - 1;
    if (n <= 0) return cudaSuccess;
    const size_t smem = sizeof(SMesh<R>) + sizeof(SegStore) * kSigWarps;
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
    SegStore* segs = reinterpret_cast<SegStore*>(smem_raw + sizeof(SMesh<R>));
    load_mesh(M, A.mesh, A.Nsig, A.NO, A.Nn);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int job = blockIdx.x * kSigWarps + warp;
    if (job >= 6 * A.NO) return;
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
        res = warp_quadgk(f, mode, s0, t, 2, A.atol, A.rtol, segs[warp], A.status) / bound;
    }
    if (lane == 0) A.corrs[side + 2 * (ch + 3 * i)] = res;
}

template <typename R>
cudaError_t launch_corrs(const CorrsArgs<R>& a, cudaStream_t st) {
    const int n = 6 * a.NO;
    const size_t smem = sizeof(SMesh<R>) + sizeof(SegStore) * kSigWarps;
    cudaError_t e = cudaFuncSetAttribute(corrs_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    corrs_kernel<R><<<(n + kSigWarps - 1) / kSigWarps, kSigWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

template cudaError_t launch_sigma<double>(const SigmaArgs<double>&, cudaStream_t);
template cudaError_t launch_sigma<float>(const SigmaArgs<float>&, cudaStream_t);
template cudaError_t launch_corrs<double>(const CorrsArgs<double>&, cudaStream_t);
template cudaError_t launch_corrs<float>(const CorrsArgs<float>&, cudaStream_t);

}  // namespace pffrg

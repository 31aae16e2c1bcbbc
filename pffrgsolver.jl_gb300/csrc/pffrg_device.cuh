// Device-side building blocks of the flow right-hand side (sm_103a).
//
// Everything here is templated on the arithmetic type R of the integrand:
// double for the FP64 path, float for the mixed path (FP32 integrand, FP64
// quadrature bookkeeping).  The functions restate the reference's frequency
// lookups (src/Frequency/param.jl, buffer.jl), the self energy and propagators
// (src/Action/Action.jl:8-26, src/Flow/bubbles.jl:2-96) and the vertex
// interpolation (src/Action/channel.jl:55-305) in a form that precomputes, once
// per node, the corner weights and offsets every site then reuses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pffrg {

constexpr int kMaxMesh = 128;  // longest supported mesh (num_* + 1)

// Packed action layout: Σ[Nsig] | comp c: bare[Ns] | ch s,t,u: q1 q2_1 q2_2 q3
// (all Julia column-major, site fastest).
struct Layout {
    int Ns, Nsig, NO, Nn, C;
    int64_t K1, K2, K3, chan, comp, total;
    __host__ __device__ int64_t bare(int c) const { return Nsig + c * comp; }
    __host__ __device__ int64_t qbase(int c, int ch, int k) const {
        int64_t b = Nsig + c * comp + Ns + ch * chan;
        return b + (k == 0 ? 0 : (k == 1 ? K1 : (k == 2 ? K1 + K2 : K1 + 2 * K2)));
    }
    // The FP32 copies of the mixed path for SU(2) keep the two components of every vertex entry side
    // by side (one 8-byte read fetches spin and density): Σ[Nsig] padded to an even length, then
    // bare[Ns] and ch s, t, u: q1 q2_1 q2_2 q3 as (spin, density) pairs.  Offsets in pairs.
    __host__ __device__ int64_t pbare() const { return (Nsig + 1) / 2; }
    __host__ __device__ int64_t pq(int ch, int k) const {
        return pbare() + Ns + ch * chan + (k == 0 ? 0 : (k == 1 ? K1 : (k == 2 ? K1 + K2 : K1 + 2 * K2)));
    }
    __host__ __device__ int64_t pair_floats() const { return 2 * (pbare() + comp); }
};

inline Layout make_layout(int Ns, int Nsig, int NO, int Nn, int C) {
    Layout L;
    L.Ns = Ns;
    L.Nsig = Nsig;
    L.NO = NO;
    L.Nn = Nn;
    L.C = C;
    L.K1 = (int64_t)Ns * NO;
    L.K2 = L.K1 * Nn;
    L.K3 = L.K2 * Nn;
    L.chan = L.K1 + 2 * L.K2 + L.K3;
    L.comp = Ns + 3 * L.chan;
    L.total = Nsig + C * L.comp;
    return L;
}

// Meshes staged in shared memory: values and reciprocal spacings
// inv[k] = 1 / (x[k+1] - x[k]) (the reference's d in get_param, param.jl:73).
template <typename R>
struct SMesh {
    R sig[kMaxMesh], isig[kMaxMesh];
    R Os[kMaxMesh], iOs[kMaxMesh];
    R ns[kMaxMesh], ins[kMaxMesh];
    R Ot[kMaxMesh], iOt[kMaxMesh];
    R nt[kMaxMesh], int_[kMaxMesh];
};

// View of the FP64 device mesh block [σ | Ωs | νs | Ωt | νt] followed by the inverse spacings
// 1 / (x[k+1] - x[k]) of the same arrays (0 at the last entry): the node setup of the FP64 path
// (staged in shared memory) and the FP64 plans of the mixed path near buffer switches (read from
// global memory) use it.
template <typename R>
struct MeshG {
    const R *sig, *isig, *Os, *iOs, *ns, *ins, *Ot, *iOt, *nt, *int_;
};

__device__ __forceinline__ MeshG<double> mesh_view(const double* mesh, int Nsig, int NO, int Nn) {
    const int n = Nsig + 2 * NO + 2 * Nn;
    MeshG<double> M;
    M.sig = mesh;
    M.Os = M.sig + Nsig;
    M.ns = M.Os + NO;
    M.Ot = M.ns + Nn;
    M.nt = M.Ot + NO;
    M.isig = M.sig + n;
    M.iOs = M.Os + n;
    M.ins = M.ns + n;
    M.iOt = M.Ot + n;
    M.int_ = M.nt + n;
    return M;
}

// device mesh block written by the host: [σ | Ωs | νs | Ωt | νt] (FP64)
template <typename R>
__device__ inline void load_mesh(SMesh<R>& M, const double* mesh, int Nsig, int NO, int Nn) {
    const double* sig = mesh;
    const double* Os = sig + Nsig;
    const double* ns = Os + NO;
    const double* Ot = ns + Nn;
    const double* nt = Ot + NO;
    for (int k = threadIdx.x; k < Nsig; k += blockDim.x) {
        M.sig[k] = (R)sig[k];
        M.isig[k] = (k + 1 < Nsig) ? (R)(1.0 / (sig[k + 1] - sig[k])) : (R)0;
    }
    for (int k = threadIdx.x; k < NO; k += blockDim.x) {
        M.Os[k] = (R)Os[k];
        M.iOs[k] = (k + 1 < NO) ? (R)(1.0 / (Os[k + 1] - Os[k])) : (R)0;
        M.Ot[k] = (R)Ot[k];
        M.iOt[k] = (k + 1 < NO) ? (R)(1.0 / (Ot[k + 1] - Ot[k])) : (R)0;
    }
    for (int k = threadIdx.x; k < Nn; k += blockDim.x) {
        M.ns[k] = (R)ns[k];
        M.ins[k] = (k + 1 < Nn) ? (R)(1.0 / (ns[k + 1] - ns[k])) : (R)0;
        M.nt[k] = (R)nt[k];
        M.int_[k] = (k + 1 < Nn) ? (R)(1.0 / (nt[k + 1] - nt[k])) : (R)0;
    }
}

template <typename R>
struct Param {
    int lo, hi;
    R wl, wu;
};

// get_indices + get_param (param.jl:26-87) with a binary search that returns
// the same pair as the reference's linear scan: hi = first k with x[k] >= val.
template <typename R>
__device__ __forceinline__ Param<R> get_param(R val, const R* x, const R* ix, int n) {
    Param<R> p;
    if (val >= x[n - 1]) {
        p.lo = p.hi = n - 1;
        p.wl = (R)1;
        p.wu = (R)0;
        return p;
    }
    int lo = 0, hi = n - 1;
    if (!(val == val)) hi = 0;  // NaN: the linear scan stops at the first entry
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (x[mid] >= val) hi = mid;
        else lo = mid + 1;
    }
    p.hi = lo;
    p.lo = (val < x[lo]) ? lo - 1 : lo;
    if (p.lo < 0) p.lo = 0;
    if (p.lo < p.hi) {
        R d = ix[p.lo];
        p.wl = d * (x[p.hi] - val);
        p.wu = d * (val - x[p.lo]);
    } else {
        p.wl = (R)1;
        p.wu = (R)0;
    }
    return p;
}

// Interpolation plan of one buffer (one channel read of one vertex slot):
// the asymptotic kernel, the channel actually read (s<->u mapping), the
// site-exchange flag, the sign for the density component and the corner
// weights and offsets of the (multi)linear interpolation in the reference's
// term order (channel.jl:245-305).
template <typename R>
struct Plan {
    int kernel;  // 0 none, 1 q1, 2 q2_1, 3 q2_2, 4 q3
    int src_ch;  // 0 s, 1 t, 2 u
    int exch;
    int flags;   // bit 0: sgn_μν, bit 1: sgn_μ, bit 2: sgn_ν
    R sgn_d;
    R w[8];
    int off[8];
};

// The interval search and the weights run in the arguments' type S (FP64 for the node setup of
// both paths); the plan stores the weights in R.
template <typename R, typename S, typename MV>
__device__ __forceinline__ void make_plan(Plan<R>& P, int chan, S w, S v, S vp, const MV& M, int Ns, int NO,
                                          int Nn) {
    bool ex = false, mp = false, smn = false, sm = false, sn = false;
    if (chan == 0) {  // get_buffer_s (buffer.jl:87-124)
        if (w < (S)0) { w = -w; ex = !ex; }
        if (v < (S)0) { v = -v; ex = !ex; mp = !mp; sm = !sm; }
        if (vp < (S)0) { vp = -vp; mp = !mp; sn = !sn; }
    } else if (chan == 1) {  // get_buffer_t (buffer.jl:126-160)
        if (w < (S)0) { w = -w; smn = !smn; }
        if (v < (S)0) { v = -v; sm = !sm; }
        if (vp < (S)0) { vp = -vp; sn = !sn; }
    } else {  // get_buffer_u (buffer.jl:162-199)
        if (w < (S)0) { w = -w; ex = !ex; smn = !smn; }
        if (v < (S)0) { v = -v; ex = !ex; mp = !mp; sn = !sn; }
        if (vp < (S)0) { vp = -vp; mp = !mp; sn = !sn; }
    }
    const S* Om = chan == 1 ? M.Ot : M.Os;
    const S* iOm = chan == 1 ? M.iOt : M.iOs;
    const S* nu = chan == 1 ? M.nt : M.ns;
    const S* inu = chan == 1 ? M.int_ : M.ins;
    if (Om[NO - 1] < fabs(w)) {  // get_buffer (buffer.jl:51-84): beyond the bosonic mesh
        P.kernel = 0;
        return;
    }
    P.exch = ex ? 1 : 0;
    P.flags = (smn ? 1 : 0) | (sm ? 2 : 0) | (sn ? 4 : 0);
    P.src_ch = (chan == 1) ? 1 : ((chan == 0) == mp ? 2 : 0);
    P.sgn_d = ((sm ? -1 : 1) * (sn ? -1 : 1)) < 0 ? (R)-1 : (R)1;
    const Param<S> p1 = get_param(w, Om, iOm, NO);
    const bool vin = !(nu[Nn - 1] < fabs(v));
    const bool vpin = !(nu[Nn - 1] < fabs(vp));
    if (!vin && !vpin) {
        P.kernel = 1;
        P.w[0] = (R)(p1.wl);
        P.w[1] = (R)(p1.wu);
        P.off[0] = Ns * p1.lo;
        P.off[1] = Ns * p1.hi;
    } else if (vin != vpin) {
        P.kernel = vin ? 2 : 3;
        const Param<S> pb = get_param(vin ? v : vp, nu, inu, Nn);
        P.w[0] = (R)(p1.wl * pb.wl);
        P.w[1] = (R)(p1.wu * pb.wl);
        P.w[2] = (R)(p1.wl * pb.wu);
        P.w[3] = (R)(p1.wu * pb.wu);
        P.off[0] = Ns * (p1.lo + NO * pb.lo);
        P.off[1] = Ns * (p1.hi + NO * pb.lo);
        P.off[2] = Ns * (p1.lo + NO * pb.hi);
        P.off[3] = Ns * (p1.hi + NO * pb.hi);
    } else {
        P.kernel = 4;
        const Param<S> p2 = get_param(v, nu, inu, Nn);
        const Param<S> p3 = get_param(vp, nu, inu, Nn);
        const int NON = NO * Nn;
        P.w[0] = (R)(p1.wl * p2.wl * p3.wl);
        P.w[1] = (R)(p1.wu * p2.wl * p3.wl);
        P.w[2] = (R)(p1.wl * p2.wu * p3.wl);
        P.w[3] = (R)(p1.wu * p2.wu * p3.wl);
        P.w[4] = (R)(p1.wl * p2.wl * p3.wu);
        P.w[5] = (R)(p1.wu * p2.wl * p3.wu);
        P.w[6] = (R)(p1.wl * p2.wu * p3.wu);
        P.w[7] = (R)(p1.wu * p2.wu * p3.wu);
        P.off[0] = Ns * (p1.lo + NO * p2.lo + NON * p3.lo);
        P.off[1] = Ns * (p1.hi + NO * p2.lo + NON * p3.lo);
        P.off[2] = Ns * (p1.lo + NO * p2.hi + NON * p3.lo);
        P.off[3] = Ns * (p1.hi + NO * p2.hi + NON * p3.lo);
        P.off[4] = Ns * (p1.lo + NO * p2.lo + NON * p3.hi);
        P.off[5] = Ns * (p1.hi + NO * p2.lo + NON * p3.hi);
        P.off[6] = Ns * (p1.lo + NO * p2.hi + NON * p3.hi);
        P.off[7] = Ns * (p1.hi + NO * p2.hi + NON * p3.hi);
    }
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
    return __ldg(p);
}

// Σ_k w_k q[off_k + s] for one plan (kernel > 0), terms in the reference's order
template <typename R>
__device__ __forceinline__ R plan_read(const Plan<R>& P, const R* __restrict__ q, int s) {
    R val;
    switch (P.kernel) {
        case 1:
            val = P.w[0] * ldg(q + P.off[0] + s);
            val += P.w[1] * ldg(q + P.off[1] + s);
            return val;
        case 2:
        case 3:
            val = P.w[0] * ldg(q + P.off[0] + s);
            val += P.w[1] * ldg(q + P.off[1] + s);
            val += P.w[2] * ldg(q + P.off[2] + s);
            val += P.w[3] * ldg(q + P.off[3] + s);
            return val;
        default:
            val = P.w[0] * ldg(q + P.off[0] + s);
#pragma unroll
            for (int k = 1; k < 8; ++k) val += P.w[k] * ldg(q + P.off[k] + s);
            return val;
    }
}

// apply_flags_su2 (action_su2.jl:73-92) for C = 2 and apply_flags_u1_dm
// (action_u1_dm.jl:80-118) for C = 6: the component a plan reads for component
// c (xx, zz, DM, dd, zd, dz for u1-dm) and the sign of its contribution
template <typename R>
__device__ __forceinline__ int comp_read(const Plan<R>& P, int C, int c, R& sgn) {
    if (C == 2) {
        sgn = c == 1 ? P.sgn_d : (R)1;
        return c;
    }
    int s = 1;
    const int f = P.flags;
    if ((c == 4 || c == 5) && (f & 1)) s = -s;
    if ((c == 3 || c == 5) && (f & 2)) s = -s;
    if ((c == 3 || c == 4) && (f & 4)) s = -s;
    int src = c;
    if (P.exch) {
        if (c == 2) s = -s;
        else if (c == 4) src = 5;
        else if (c == 5) src = 4;
    }
    sgn = (R)s;
    return src;
}

__host__ __device__ constexpr int corners_of(int kernel) {
    return kernel == 0 ? 0 : (kernel == 1 ? 2 : (kernel == 4 ? 8 : 4));
}

// ---------------------------------------------------------------------------
// self energy and propagators
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R jl_sign(R x) {
    return x > (R)0 ? (R)1 : (x < (R)0 ? (R)-1 : x);
}

// get_Σ (Action.jl:8-26): Σ values of an action read from global memory
template <typename R, typename MV>
__device__ __forceinline__ R get_sigma(const MV& M, int Nsig, const R* __restrict__ Sig, R w) {
    if (fabs(w) <= M.sig[Nsig - 1]) {
        Param<R> p = get_param((R)fabs(w), M.sig, M.isig, Nsig);
        return jl_sign(w) * (p.wl * ldg(Sig + p.lo) + p.wu * ldg(Sig + p.hi));
    }
    return M.sig[Nsig - 1] * ldg(Sig + Nsig - 1) / w;
}

__device__ __forceinline__ double expm1_r(double x) { return expm1(x); }
__device__ __forceinline__ float expm1_r(float x) { return expm1f(x); }
__device__ __forceinline__ double exp_r(double x) { return exp(x); }
__device__ __forceinline__ float exp_r(float x) { return expf(x); }

template <typename R>
__device__ __forceinline__ R G_bare(R L, R w) {
    if (fabs(w) > (R)1e-8) return -expm1_r(-(w * w) / (L * L)) / w;
    return (R)0;
}

template <typename R, typename MV>
__device__ __forceinline__ R G_full(const MV& M, int Nsig, const R* Sig, R L, R w) {
    if (fabs(w) > (R)1e-8) {
        R s = get_sigma(M, Nsig, Sig, w);
        R g0 = G_bare(L, w);
        R den = (w * s >= (R)0) ? (R)1 / g0 + s : (R)1 / g0;
        return (R)1 / den;
    }
    return (R)0;
}

template <typename R, typename MV>
__device__ __forceinline__ R S_single(const MV& M, int Nsig, const R* Sig, R L, R w) {
    if (fabs(w) > (R)1e-8) {
        R g = G_full(M, Nsig, Sig, L, w);
        R g0 = G_bare(L, w);
        R r = g / g0;
        return r * r * exp_r(-(w * w) / (L * L)) * (R)2 * w / (L * L * L);
    }
    return (R)0;
}

template <typename R>
__device__ __forceinline__ R two_pi() {
    return (R)(2.0 * 3.14159265358979323846);
}

// get_propagator_kat (bubbles.jl:64-80)
template <typename R, typename MV>
__device__ __forceinline__ R prop_kat(const MV& M, int Nsig, const R* Sig, const R* dSig, R L, R w1, R w2) {
    R ds = get_sigma(M, Nsig, dSig, w1);
    R s1 = S_single(M, Nsig, Sig, L, w1);
    R g1 = G_full(M, Nsig, Sig, L, w1);
    R g2 = G_full(M, Nsig, Sig, L, w2);
    return (s1 + g1 * g1 * ds) * g2 / two_pi<R>();
}

// get_propagator (bubbles.jl:83-96)
template <typename R, typename MV>
__device__ __forceinline__ R prop_plain(const MV& M, int Nsig, const R* Sig, R L, R w1, R w2) {
    R g1 = G_full(M, Nsig, Sig, L, w1);
    R g2 = G_full(M, Nsig, Sig, L, w2);
    return g1 * g2 / two_pi<R>();
}

// one half of the bubble propagator of channel ch at node v and transfer W
// (flow_su2_{s,t,u}.jl: first lines of every kernel, bubbles.jl:99-221)
template <typename R, typename MV>
__device__ __forceinline__ R prop_half(int kind, int half, int ch, const MV& M, int Nsig, const R* Sig,
                                       const R* dSig, R L, R v, R W) {
    R w1, w2;
    const R hW = (R)0.5 * W;
    if (ch == 0) {
        w1 = v + hW;
        w2 = hW - v;
    } else if (ch == 1) {
        w1 = v + hW;
        w2 = v - hW;
    } else {
        w1 = v - hW;
        w2 = v + hW;
    }
    if (kind == 0) {
        return half == 0 ? prop_kat(M, Nsig, Sig, dSig, L, w1, w2) : prop_kat(M, Nsig, Sig, dSig, L, w2, w1);
    }
    return -prop_plain(M, Nsig, Sig, L, w1, w2);
}

// ---------------------------------------------------------------------------
// Node setup of the mixed path in float-float arithmetic.  An interpolation weight is
// (x[k+1] - arg) / (x[k+1] - x[k]); with arg and x rounded to FP32 its error is the FP32 rounding
// of |arg| divided by the mesh spacing, up to ~N ulps on a mesh of N points — the dominant error
// of an FP32 integrand (measured 2e-6 of max|dΓ|).  The mixed path therefore carries the node,
// the transfer frequencies and the meshes as unevaluated sums h + l of two floats (error-free
// two-sum additions), searches the interval on the pair and forms the weight from the pairwise
// difference: weights accurate to FP32 rounding of the weight itself, in FP32 instructions only
// (FP64 arithmetic is slow on this GPU).
// ---------------------------------------------------------------------------
struct FF {
    float h, l;
    FF() = default;
    __host__ __device__ constexpr FF(float hi, float lo) : h(hi), l(lo) {}
    // the pair nearest to x (infinities keep l = 0)
    __device__ explicit FF(double x) : h((float)x), l(isinf((float)x) ? 0.f : (float)(x - (double)(float)x)) {}
};

__device__ __forceinline__ FF ff_norm(float s, float t) {  // fast two-sum of s + t, |s| >= |t|
    const float h = __fadd_rn(s, t);
    return FF{h, __fsub_rn(t, __fsub_rn(h, s))};
}
__device__ __forceinline__ FF operator+(FF a, FF b) {
    const float s = __fadd_rn(a.h, b.h);
    if (isinf(s)) return FF{s, 0.f};
    const float bb = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    return ff_norm(s, __fadd_rn(__fadd_rn(e, a.l), b.l));
}
__device__ __forceinline__ FF operator-(FF a) { return FF{-a.h, -a.l}; }
__device__ __forceinline__ FF operator-(FF a, FF b) { return a + (-b); }
// scaling by a power of two (the 1/2 of the argument formulas): exact
__device__ __forceinline__ FF operator*(FF s, FF a) { return FF{s.h * a.h, s.h * a.l}; }
__device__ __forceinline__ bool operator<(FF a, FF b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ bool operator<(FF a, float b) { return a.h < b || (a.h == b && a.l < 0.f); }
__device__ __forceinline__ FF ff_abs(FF a) { return a < 0.f ? -a : a; }

// Per mesh of the float block, four floats that place a frequency near its interval for the lin-log
// meshes of get_mesh (mesh.jl:86-121): 1 / spacing of the linear part, its last index, its last
// point and 1 / log(ratio) of the logarithmic part (all 0 when the mesh has no such form)
constexpr int kMeshGuess = 20;

// Mesh block of the mixed path (floats): [h | l | inverse spacing], each [σ | Ωs | νs | Ωt | νt],
// then the kMeshGuess placement parameters
struct MeshFF {
    const float* h;
    const float* l;
    const float* inv;
    const float* g;
    int Nsig, NO, Nn;
    __device__ __forceinline__ int sig() const { return 0; }
    __device__ __forceinline__ int Os() const { return Nsig; }
    __device__ __forceinline__ int ns() const { return Nsig + NO; }
    __device__ __forceinline__ int Ot() const { return Nsig + NO + Nn; }
    __device__ __forceinline__ int nt() const { return Nsig + 2 * NO + Nn; }
    __device__ __forceinline__ FF at(int o, int k) const { return FF{h[o + k], l[o + k]}; }
};

__device__ __forceinline__ MeshFF mesh_view_ff(const float* block, int Nsig, int NO, int Nn) {
    const int n = Nsig + 2 * NO + 2 * Nn;
    return MeshFF{block, block + n, block + 2 * n, block + 3 * n, Nsig, NO, Nn};
}

// get_indices + get_param (param.jl:26-87) on the mesh at offset o of length n, as get_param
__device__ __forceinline__ Param<float> get_param_ff(FF val, const MeshFF& M, int o, int n) {
    Param<float> p;
    if (!(val < M.at(o, n - 1))) {
        p.lo = p.hi = n - 1;
        p.wl = 1.f;
        p.wu = 0.f;
        return p;
    }
    // first k with h[k] >= val.h (val < x[n-1] here, so one exists): a guess from the lin-log form of
    // the mesh, then steps to the exact index, which any increasing mesh reaches
    const int gi = o == 0 ? 0 : (o == M.Os() ? 1 : (o == M.ns() ? 2 : (o == M.Ot() ? 3 : 4)));
    const float* g = M.g + 4 * gi;
    const float v = val.h;
    const float kf = v <= g[2] ? ceilf(v * g[0]) : g[1] + ceilf(__logf(v / g[2]) * g[3]);
    int lo = (kf >= 0.f && kf <= (float)(n - 1)) ? (int)kf : (kf > 0.f ? n - 1 : 0);
    while (lo > 0 && M.h[o + lo - 1] >= v) --lo;
    while (lo < n - 1 && M.h[o + lo] < v) ++lo;
    // then past an equal high part whose pair is still below val (mesh points lie more than an
    // FP32 ulp apart)
    if (lo < n - 1 && M.h[o + lo] == val.h && M.l[o + lo] < val.l) ++lo;
    p.hi = lo;
    p.lo = (val < M.at(o, lo)) ? lo - 1 : lo;
    if (p.lo < 0) p.lo = 0;
    if (p.lo < p.hi) {
        const float d = M.inv[o + p.lo];
        const FF xh = M.at(o, p.hi), xl = M.at(o, p.lo);
        p.wl = d * __fadd_rn(__fsub_rn(xh.h, val.h), __fsub_rn(xh.l, val.l));
        p.wu = d * __fadd_rn(__fsub_rn(val.h, xl.h), __fsub_rn(val.l, xl.l));
    } else {
        p.wl = 1.f;
        p.wu = 0.f;
    }
    return p;
}

// make_plan with float-float arguments (same sign folding, kernel choice and corner order)
__device__ __forceinline__ void make_plan_ff(Plan<float>& P, int chan, FF w, FF v, FF vp, const MeshFF& M, int Ns,
                                             int NO, int Nn) {
    bool ex = false, mp = false, smn = false, sm = false, sn = false;
    if (chan == 0) {  // get_buffer_s (buffer.jl:87-124)
        if (w < 0.f) { w = -w; ex = !ex; }
        if (v < 0.f) { v = -v; ex = !ex; mp = !mp; sm = !sm; }
        if (vp < 0.f) { vp = -vp; mp = !mp; sn = !sn; }
    } else if (chan == 1) {  // get_buffer_t (buffer.jl:126-160)
        if (w < 0.f) { w = -w; smn = !smn; }
        if (v < 0.f) { v = -v; sm = !sm; }
        if (vp < 0.f) { vp = -vp; sn = !sn; }
    } else {  // get_buffer_u (buffer.jl:162-199)
        if (w < 0.f) { w = -w; ex = !ex; smn = !smn; }
        if (v < 0.f) { v = -v; ex = !ex; mp = !mp; sn = !sn; }
        if (vp < 0.f) { vp = -vp; mp = !mp; sn = !sn; }
    }
    const int oO = chan == 1 ? M.Ot() : M.Os();
    const int on = chan == 1 ? M.nt() : M.ns();
    if (M.at(oO, NO - 1) < w) {  // get_buffer (buffer.jl:51-84): beyond the bosonic mesh
        P.kernel = 0;
        return;
    }
    P.exch = ex ? 1 : 0;
    P.flags = (smn ? 1 : 0) | (sm ? 2 : 0) | (sn ? 4 : 0);
    P.src_ch = (chan == 1) ? 1 : ((chan == 0) == mp ? 2 : 0);
    P.sgn_d = ((sm ? -1 : 1) * (sn ? -1 : 1)) < 0 ? -1.f : 1.f;
    const Param<float> p1 = get_param_ff(w, M, oO, NO);
    const FF numax = M.at(on, Nn - 1);
    const bool vin = !(numax < v);
    const bool vpin = !(numax < vp);
    if (!vin && !vpin) {
        P.kernel = 1;
        P.w[0] = p1.wl;
        P.w[1] = p1.wu;
        P.off[0] = Ns * p1.lo;
        P.off[1] = Ns * p1.hi;
    } else if (vin != vpin) {
        P.kernel = vin ? 2 : 3;
        const Param<float> pb = get_param_ff(vin ? v : vp, M, on, Nn);
        P.w[0] = p1.wl * pb.wl;
        P.w[1] = p1.wu * pb.wl;
        P.w[2] = p1.wl * pb.wu;
        P.w[3] = p1.wu * pb.wu;
        P.off[0] = Ns * (p1.lo + NO * pb.lo);
        P.off[1] = Ns * (p1.hi + NO * pb.lo);
        P.off[2] = Ns * (p1.lo + NO * pb.hi);
        P.off[3] = Ns * (p1.hi + NO * pb.hi);
    } else {
        P.kernel = 4;
        const Param<float> p2 = get_param_ff(v, M, on, Nn);
        const Param<float> p3 = get_param_ff(vp, M, on, Nn);
        const int NON = NO * Nn;
        P.w[0] = p1.wl * p2.wl * p3.wl;
        P.w[1] = p1.wu * p2.wl * p3.wl;
        P.w[2] = p1.wl * p2.wu * p3.wl;
        P.w[3] = p1.wu * p2.wu * p3.wl;
        P.w[4] = p1.wl * p2.wl * p3.wu;
        P.w[5] = p1.wu * p2.wl * p3.wu;
        P.w[6] = p1.wl * p2.wu * p3.wu;
        P.w[7] = p1.wu * p2.wu * p3.wu;
        P.off[0] = Ns * (p1.lo + NO * p2.lo + NON * p3.lo);
        P.off[1] = Ns * (p1.hi + NO * p2.lo + NON * p3.lo);
        P.off[2] = Ns * (p1.lo + NO * p2.hi + NON * p3.lo);
        P.off[3] = Ns * (p1.hi + NO * p2.hi + NON * p3.lo);
        P.off[4] = Ns * (p1.lo + NO * p2.lo + NON * p3.hi);
        P.off[5] = Ns * (p1.hi + NO * p2.lo + NON * p3.hi);
        P.off[6] = Ns * (p1.lo + NO * p2.hi + NON * p3.hi);
        P.off[7] = Ns * (p1.hi + NO * p2.hi + NON * p3.hi);
    }
}

// True when a float-float plan argument lies within a few FP32 ulps of a point where the vertex
// buffers switch: zero (the sign folding of buffer.jl) or the last point of a bosonic or fermionic
// mesh (beyond it the kernel changes; beyond the bosonic one the vertex is zero).  The FP64
// rounding of the argument decides the side there, so such a plan is built in FP64.  (Measured:
// skipping the test for plans read at the task frequencies themselves left 2e-6 of max|dΓ| on a
// square L=3 flow state at Λ = 0.49, so every plan is tested.)
__device__ __forceinline__ bool ff_near_switch(FF a, float scale, const MeshFF& M, int NO, int Nn) {
    const float x = fabsf(a.h);
    if (isinf(x)) return false;
    if (x <= 1e-9f * scale) return true;
    const float b[4] = {M.h[M.Os() + NO - 1], M.h[M.Ot() + NO - 1], M.h[M.ns() + Nn - 1], M.h[M.nt() + Nn - 1]};
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (fabsf(x - b[q]) <= 4.8e-7f * b[q]) return true;
    return false;
}

// get_Σ of the arrays Sig (and dSig, when given) at the float-float frequency w: one interval
// search serves both
__device__ __forceinline__ float get_sigma_ff(const MeshFF& M, int Nsig, const float* __restrict__ Sig, FF w,
                                              const float* __restrict__ dSig = nullptr, float* ds = nullptr) {
    const FF aw = ff_abs(w);
    const FF smax = M.at(M.sig(), Nsig - 1);
    if (!(smax < aw)) {
        const Param<float> p = get_param_ff(aw, M, M.sig(), Nsig);
        const float sg = jl_sign(w.h);
        if (dSig) *ds = sg * (p.wl * ldg(dSig + p.lo) + p.wu * ldg(dSig + p.hi));
        return sg * (p.wl * ldg(Sig + p.lo) + p.wu * ldg(Sig + p.hi));
    }
    if (dSig) *ds = smax.h * ldg(dSig + Nsig - 1) / w.h;
    return smax.h * ldg(Sig + Nsig - 1) / w.h;
}

// G_full from Σ(w) already read
__device__ __forceinline__ float G_full_s(float s, float L, float w) {
    if (fabsf(w) > 1e-8f) {
        const float g0 = G_bare(L, w);
        const float den = (w * s >= 0.f) ? 1.f / g0 + s : 1.f / g0;
        return 1.f / den;
    }
    return 0.f;
}

// prop_half with float-float frequencies (bubbles.jl:64-96)
__device__ __forceinline__ float prop_half_ff(int kind, int half, int ch, const MeshFF& M, int Nsig, const float* Sig,
                                              const float* dSig, float L, FF v, FF W) {
    const FF hW = FF{0.5f, 0.f} * W;
    FF w1, w2;
    if (ch == 0) {
        w1 = v + hW;
        w2 = hW - v;
    } else if (ch == 1) {
        w1 = v + hW;
        w2 = v - hW;
    } else {
        w1 = v - hW;
        w2 = v + hW;
    }
    if (kind == 0) {  // get_propagator_kat: (S(a) + G(a)^2 dΣ(a)) G(b)
        const FF a = half == 0 ? w1 : w2, b = half == 0 ? w2 : w1;
        float ds = 0.f;
        const float sa = get_sigma_ff(M, Nsig, Sig, a, dSig, &ds);
        const float g1 = G_full_s(sa, L, a.h);
        const float g0 = G_bare(L, a.h);
        const float r = g1 / g0;
        const float s1 = fabsf(a.h) > 1e-8f ? r * r * expf(-(a.h * a.h) / (L * L)) * 2.f * a.h / (L * L * L) : 0.f;
        const float g2 = G_full_s(get_sigma_ff(M, Nsig, Sig, b), L, b.h);
        return (s1 + g1 * g1 * ds) * g2 / two_pi<float>();
    }
    const float g1 = G_full_s(get_sigma_ff(M, Nsig, Sig, w1), L, w1.h);
    const float g2 = G_full_s(get_sigma_ff(M, Nsig, Sig, w2), L, w2.h);
    return -(g1 * g2) / two_pi<float>();
}

}  // namespace pffrg

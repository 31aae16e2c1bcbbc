// Channel-task passes of the flow right-hand side (sm_103a): level-synchronous
// adaptive quadrature.
//
// A pass is the set of channel tasks (channel X, kernel, w1, w2, w3) that one
// call of compute_dΓ_{1l,2l,ml}!/compute_Γ!/compute_Σ! fans out
// (src/Flow/compute.jl, SDE.jl).  Each task integrates its bubble over the
// 4*eval subdomains of integrate_log!/integrate_lin! (src/Flow/quadrature.jl:
// 84-139) plus two boundary nodes (src/Flow/flow_s.jl:37-38), and every
// subdomain runs the adaptive Simpson rule with Richardson extrapolation of
// simps! (quadrature.jl:27-81), whose depth varies by orders of magnitude
// between subdomains.  Instead of one CTA per task (whose slowest member sets
// the pass time), the subdomains of all tasks advance level by level:
//
//   wave 0   every subdomain evaluates its first five nodes (the 3-point and
//            the 5-point Simpson sums) and takes the first convergence test;
//   wave k   the 2^(k+1) new nodes of every subdomain still refining are cut
//            into chunks of at most kChunk nodes; eval_kernel spreads the
//            chunks over the whole GPU and writes one partial node sum per
//            chunk; decide_kernel sums a subdomain's partials in node order,
//            forms the next Simpson sum and the Richardson value, takes the
//            reference's test (||R - S|| < atol or relative < rtol, or
//            n > 2^20) and either stores the result or queues the next level;
//   reduce   sums each task's subdomain results in a fixed order and writes
//            the output slice (flow_s.jl:41-51).
//
// The reweighted nodes of residual! (quadrature.jl:2-24) are the previous
// level's new nodes, so their sum is carried from the last level instead of
// re-evaluating the integrand there.  Results are deterministic (fixed
// summation order) and agree with the reference's arithmetic up to rounding.
//
// Node evaluation: a team of T lanes evaluates a batch of up to kBatch nodes.
// The lanes first split the batch's scalar work (propagator halves,
// bubbles.jl; 6 or 12 interpolation plans, buffer.jl + channel.jl), then each
// lane gathers and combines the vertex on its sites (flow_su2_{s,t,u}.jl,
// flow_u1_dm_{s,t,u}.jl); the t channel stages both slots in shared memory for
// the overlap sum (flow_su2_t.jl:66-75) whose rows sit packed in shared memory.
// Every kernel is templated on the vertex component count C: 2 for SU(2)
// (spin, density), 6 for U(1)-DM (xx, zz, DM, dd, zd, dz).
#pragma once

#include <algorithm>
#include <type_traits>

#include "pffrg_internal.h"

namespace pffrg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarps = 4;

template <typename R, int C>
struct NodeScratch {
    double x;      // the node (integration variable v)
    R p_half[2];
    R loc[2 * C];  // t channel: local vertices v3[C], v4[C] at site 1
    Plan<R> plan[4][3];
};

// nodes per team batch: 4 per warp in total, 2 for SU(2) when each lane holds more than four sites
// (the SU(2) t-channel staging grows with sites x nodes).  The node scratch and t-channel staging
// of a batch set the shared memory of a block, which limits the blocks per SM: on the pyrochlore
// L = 6 two-loop state 32x2 teams with 4 nodes ran 403 ms against 470 ms with 8 nodes (two blocks
// per SM instead of three), and 16x3 teams were slower with 1 node than with 2.
template <int T, int C, int SPL>
struct BatchOf {
    static constexpr int NB = (C == 2 ? (SPL <= 4 ? 4 : 2) : 4) * T / 32;
};

// SU(2) t-channel staging: per site the NB (spin, density) pairs of a batch, padded by 16 bytes so
// that the 16-byte loads of lanes reading different sites spread over the shared-memory banks
template <typename R, int NB>
__host__ __device__ constexpr int t_site_stride() {
    return NB + (sizeof(R) == 4 ? 2 : 1);  // in pairs of R
}

template <typename R, int T, int C, int SPL>
struct TeamScratch {
    NodeScratch<R, C> node[BatchOf<T, C, SPL>::NB];
};

// ---------------------------------------------------------------------------
// U(1)-DM bubbles of two vertices u, w (components xx, zz, DM, dd, zd, dz), the
// reference's term order; the same combination serves the Katanin, left,
// central, BSE and reduced kernels of a channel
// ---------------------------------------------------------------------------
// s channel (flow_u1_dm_s.jl:53-58)
template <typename R>
__device__ __forceinline__ void u1dm_s(const R* a, const R* b, R* g) {
    g[0] = a[2] * b[5] - a[2] * b[4] + a[0] * b[3] + a[3] * b[0] - a[0] * b[1] - a[5] * b[2] + a[4] * b[2] - a[1] * b[0];
    g[1] = a[1] * b[3] + a[3] * b[1] - a[5] * b[4] - (R)2 * a[0] * b[0] - (R)2 * a[2] * b[2] - a[4] * b[5];
    g[2] = a[3] * b[2] + a[2] * b[3] - a[4] * b[0] - a[0] * b[5] - a[1] * b[2] + a[0] * b[4] - a[2] * b[1] + a[5] * b[0];
    g[3] = -a[5] * b[5] + (R)2 * a[0] * b[0] + a[3] * b[3] + (R)2 * a[2] * b[2] - a[4] * b[4] + a[1] * b[1];
    g[4] = a[4] * b[3] + a[3] * b[4] - (R)2 * a[2] * b[0] + a[5] * b[1] + a[1] * b[5] + (R)2 * a[0] * b[2];
    g[5] = a[4] * b[1] + a[3] * b[5] + a[1] * b[4] + (R)2 * a[2] * b[0] + a[5] * b[3] - (R)2 * a[0] * b[2];
}
// u channel (flow_u1_dm_u.jl:52-57)
template <typename R>
__device__ __forceinline__ void u1dm_u(const R* a, const R* b, R* g) {
    g[0] = -a[2] * b[5] - a[2] * b[4] + a[0] * b[3] + a[3] * b[0] + a[0] * b[1] + a[5] * b[2] + a[4] * b[2] + a[1] * b[0];
    g[1] = a[1] * b[3] + a[3] * b[1] - a[5] * b[4] + (R)2 * a[0] * b[0] + (R)2 * a[2] * b[2] - a[4] * b[5];
    g[2] = a[3] * b[2] + a[2] * b[3] - a[4] * b[0] + a[0] * b[5] + a[1] * b[2] + a[0] * b[4] + a[2] * b[1] - a[5] * b[0];
    g[3] = -a[5] * b[5] + (R)2 * a[0] * b[0] + a[3] * b[3] + (R)2 * a[2] * b[2] - a[4] * b[4] + a[1] * b[1];
    g[4] = a[4] * b[3] + a[3] * b[4] - (R)2 * a[2] * b[0] + a[5] * b[1] + a[1] * b[5] + (R)2 * a[0] * b[2];
    g[5] = a[4] * b[1] + a[3] * b[5] + a[1] * b[4] - (R)2 * a[2] * b[0] + a[5] * b[3] + (R)2 * a[0] * b[2];
}
// t channel, local part: v1, v2 non-local at site i, v3, v4 local at site 1 (flow_u1_dm_t.jl:68-84)
template <typename R>
__device__ __forceinline__ void u1dm_t(const R* v1, const R* v2, const R* v3, const R* v4, R* g) {
    g[0] = v1[2] * v4[5] - v1[2] * v4[4] + v1[0] * v4[3] - v1[0] * v4[1] + v3[3] * v2[0] + v3[5] * v2[2] -
           v3[4] * v2[2] - v3[1] * v2[0];
    g[1] = v1[1] * v4[3] + (R)2 * v1[4] * v4[2] - v1[4] * v4[4] + v1[1] * v4[1] - (R)2 * v1[1] * v4[0] -
           v1[4] * v4[5] - (R)2 * v3[2] * v2[5] - v3[5] * v2[5] + v3[3] * v2[1] - (R)2 * v3[0] * v2[1] +
           v3[1] * v2[1] - v3[4] * v2[5];
    g[2] = v1[2] * v4[3] - v1[0] * v4[5] + v1[0] * v4[4] - v1[2] * v4[1] - v3[5] * v2[0] + v3[3] * v2[2] +
           v3[4] * v2[0] - v3[1] * v2[2];
    g[3] = -v1[5] * v4[5] + (R)2 * v1[3] * v4[0] + v1[3] * v4[1] - v1[5] * v4[4] - (R)2 * v1[5] * v4[2] +
           v1[3] * v4[3] + (R)2 * v3[2] * v2[4] + (R)2 * v3[0] * v2[3] + v3[1] * v2[3] - v3[5] * v2[4] +
           v3[3] * v2[3] - v3[4] * v2[4];
    g[4] = v1[4] * v4[1] + v1[4] * v4[3] + (R)2 * v1[4] * v4[0] + v1[1] * v4[4] + (R)2 * v1[1] * v4[2] +
           v1[1] * v4[5] + v3[4] * v2[3] + (R)2 * v3[2] * v2[3] + v3[3] * v2[4] + v3[1] * v2[4] -
           (R)2 * v3[0] * v2[4] + v3[5] * v2[3];
    g[5] = -(R)2 * v1[3] * v4[2] + v1[3] * v4[4] + v1[3] * v4[5] + v1[5] * v4[1] + v1[5] * v4[3] -
           (R)2 * v1[5] * v4[0] + v3[4] * v2[1] + (R)2 * v3[0] * v2[5] + v3[3] * v2[5] + v3[5] * v2[1] -
           (R)2 * v3[2] * v2[1] + v3[1] * v2[5];
}

// per-node argument triple (w, v, v') of buffer (slot, ch) for channel X
// (flow_su2_s.jl:21-28, flow_su2_t.jl:21-43, flow_su2_u.jl:21-28)
template <typename R>
__device__ __forceinline__ void slot_arg(int X, int slot, int ch, R v, R W, R V, R VP, R& a0, R& a1, R& a2) {
    const R h = (R)0.5;
    if (X == 0) {
        const R s = W, vs = V, vsp = VP;
        if (slot == 0) {
            if (ch == 0) { a0 = s; a1 = vs; a2 = -v; }
            else if (ch == 1) { a0 = v - vs; a1 = h * (s + v + vs); a2 = h * (s - v - vs); }
            else { a0 = v + vs; a1 = h * (s - v + vs); a2 = h * (s + v - vs); }
        } else {
            if (ch == 0) { a0 = s; a1 = v; a2 = vsp; }
            else if (ch == 1) { a0 = -v - vsp; a1 = h * (s + v - vsp); a2 = h * (s - v + vsp); }
            else { a0 = v - vsp; a1 = h * (s + v + vsp); a2 = h * (s - v - vsp); }
        }
    } else if (X == 1) {
        const R t = W, vt = V, vtp = VP;
        switch (slot) {
            case 0:
                if (ch == 0) { a0 = v + vt; a1 = h * (-t - v + vt); a2 = h * (-t + v - vt); }
                else if (ch == 1) { a0 = t; a1 = vt; a2 = v; }
                else { a0 = -v + vt; a1 = h * (-t + v + vt); a2 = h * (t + v + vt); }
                break;
            case 1:
                if (ch == 0) { a0 = v + vtp; a1 = h * (-t + v - vtp); a2 = h * (-t - v + vtp); }
                else if (ch == 1) { a0 = t; a1 = v; a2 = vtp; }
                else { a0 = v - vtp; a1 = h * (-t + v + vtp); a2 = h * (t + v + vtp); }
                break;
            case 2:
                if (ch == 0) { a0 = v + vt; a1 = h * (t + v - vt); a2 = h * (-t + v - vt); }
                else if (ch == 1) { a0 = -v + vt; a1 = h * (t + v + vt); a2 = h * (-t + v + vt); }
                else { a0 = t; a1 = v; a2 = vt; }
                break;
            default:
                if (ch == 0) { a0 = v + vtp; a1 = h * (t - v + vtp); a2 = h * (-t - v + vtp); }
                else if (ch == 1) { a0 = v - vtp; a1 = h * (t + v + vtp); a2 = h * (-t + v + vtp); }
                else { a0 = t; a1 = vtp; a2 = v; }
                break;
        }
    } else {
        const R u = W, vu = V, vup = VP;
        if (slot == 0) {
            if (ch == 0) { a0 = v + vu; a1 = h * (u - v + vu); a2 = h * (-u - v + vu); }
            else if (ch == 1) { a0 = v - vu; a1 = h * (u + v + vu); a2 = h * (-u + v + vu); }
            else { a0 = u; a1 = vu; a2 = v; }
        } else {
            if (ch == 0) { a0 = v + vup; a1 = h * (u + v - vup); a2 = h * (-u + v - vup); }
            else if (ch == 1) { a0 = -v + vup; a1 = h * (u + v + vup); a2 = h * (-u + v + vup); }
            else { a0 = u; a1 = v; a2 = vup; }
        }
    }
}

// vertex component c of one slot at one site (single value), for the t-channel local vertices
template <typename R, int C>
__device__ __forceinline__ R gather_one(const PassArgs<R>& A, const NodeScratch<R, C>& ns, int slot, int c, int i,
                                        int exch_i) {
    const R* __restrict__ src = A.src[slot];
    if constexpr (sizeof(R) == 4 && C == 2) {
        // FP32 copies of SU(2) actions hold (spin, density) pairs
        const float* __restrict__ s2 = src + c;
        R val = ldg(s2 + 2 * (A.L.pbare() + i));
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const Plan<R>& P = ns.plan[slot][ch];
            if (P.kernel) {
                const float* q = s2 + 2 * A.L.pq(P.src_ch, P.kernel - 1);
                const int s = P.exch ? exch_i : i;
                R acc = P.w[0] * ldg(q + 2 * (P.off[0] + s));
                for (int k = 1; k < corners_of(P.kernel); ++k) acc += P.w[k] * ldg(q + 2 * (P.off[k] + s));
                val += (c == 1 ? P.sgn_d : (R)1) * acc;
            }
        }
        return val;
    }
    R val = ldg(src + A.L.bare(c) + i);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const Plan<R>& P = ns.plan[slot][ch];
        if (P.kernel) {
            R sgn;
            const int cs = comp_read(P, C, c, sgn);
            const R* q = src + A.L.qbase(cs, P.src_ch, P.kernel - 1);
            R acc = plan_read(P, q, P.exch ? exch_i : i);
            val += sgn * acc;
        }
    }
    return val;
}

// all components of one slot on this lane's sites, v[c][k] = Γ_c(site tl + k T) (the U(1)-DM passes;
// SU(2) reads its pair-layout copies in Team::gather_su2): bare + Σ_ch sgn Σ_q w_q q_c'[off_q + site]
// with the read component c' and sign of apply_flags_u1_dm, channels and corners in the reference's
// order.  The loop over a channel's corners is not unrolled: one corner's reads of all components
// and sites are in flight together, and the kernel's code stays small enough for the instruction
// cache (unrolled over the eight corners, six components and the lane's sites, the reads of two
// slots made the three-loop U(1)-DM kernels wait on instruction fetch 15 cycles per issue).  Padding
// sites read site 0 and are zeroed at the end.
template <typename R, int T, int SPL, int C>
__device__ __forceinline__ void gather_slot(const PassArgs<R>& A, const NodeScratch<R, C>& ns, int slot, int tl,
                                            const int* site_ex, R v[C][SPL]) {
    const R* __restrict__ src = A.src[slot];
    const int Ns = A.L.Ns;
    int si[SPL];
#pragma unroll
    for (int k = 0; k < SPL; ++k) {
        const int i = tl + k * T;
        si[k] = i < Ns ? i : 0;
    }
#pragma unroll
    for (int k = 0; k < SPL; ++k)
#pragma unroll
        for (int c = 0; c < C; ++c) v[c][k] = ldg(src + A.L.bare(c) + si[k]);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const Plan<R>& P = ns.plan[slot][ch];
        const int kern = P.kernel;
        if (!kern) continue;
        const int nc = corners_of(kern);
        int st[SPL];
#pragma unroll
        for (int k = 0; k < SPL; ++k) st[k] = P.exch ? site_ex[k] : si[k];
        const R* q0[C];
        R sg[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int cs = comp_read(P, C, c, sg[c]);
            q0[c] = src + A.L.qbase(cs, P.src_ch, kern - 1);
        }
        R a[C][SPL];
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) a[c][k] = (R)0;
#pragma unroll 1
        for (int q = 0; q < nc; ++q) {
            const R w = P.w[q];
            const int off = P.off[q];
#pragma unroll
            for (int c = 0; c < C; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) a[c][k] += w * ldg(q0[c] + off + st[k]);
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) v[c][k] += sg[c] * a[c][k];
    }
#pragma unroll
    for (int k = 0; k < SPL; ++k)
        if (tl + k * T >= Ns)
#pragma unroll
            for (int c = 0; c < C; ++c) v[c][k] = (R)0;
}

template <typename R>
struct Acc {
    R s;
    R c;
};

template <typename R>
__device__ __forceinline__ void acc_add(Acc<R>& a, R x) {
    a.s += x;
}
// Kahan-Babuska (Neumaier) summation for the FP32 node sums
template <>
__device__ __forceinline__ void acc_add<float>(Acc<float>& a, float x) {
    float t = a.s + x;
    if (fabsf(a.s) >= fabsf(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}

template <int T>
__device__ __forceinline__ double in_team_sum(double v) {
#pragma unroll
    for (int o = 1; o < T; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// Task of a subdomain record and its frequencies (get_kernel_args, mesh.jl:30-83)
struct TaskInfo {
    int X, kernel, w1, w2, w3;
};

template <typename R>
__device__ __forceinline__ TaskInfo task_of(const PassArgs<R>& A, int sub, int jobs) {
    const int ct = sub / jobs;  // channel-task index = y * ntasks + task
    const int y = ct / A.ntasks;
    const int4 t = A.tasks[ct - y * A.ntasks];
    return TaskInfo{A.chan_of_y[y], t.x, t.y, t.z, t.w};
}

template <typename R, int T, int SPL, int C>
struct Team {
    const PassArgs<R>& A;
    // node setup: FP64 on the FP64 path, float-float on the mixed path
    using SetupT = typename std::conditional<sizeof(R) == 4, FF, double>::type;
    using SetupMesh = typename std::conditional<sizeof(R) == 4, MeshFF, MeshG<double>>::type;
    const SetupMesh& M;
    TeamScratch<R, T, C, SPL>& ts;
    R* tmp;                 // t channel: [2 C][Ns] slot values of the current node
    const unsigned* rows;   // packed overlap rows (shared or global)
    const int* row_off;     // [Ns+1]
    int tl;                 // lane in team
    int site_ex[SPL];       // exchange[site] of this lane's sites
    unsigned long long nodes, alg;

    // Evaluate the integrand of channel X at the up to NB nodes ts.node[0..count).x of one task and
    // hand each node's values to sink(j, g) in node order, g[c][k] = Γ_c(site tl + k T; x_j)
    // (zero on the padding sites k T + tl >= Ns).  Team-collective: all lanes of the warp call it
    // together (inactive teams with count = 0).
    template <class Sink>
    __device__ __forceinline__ void eval(const TaskInfo& ti, SetupT W, SetupT V, SetupT VP, int count, Sink& sink) {
        const int X = ti.X;
        const int Ns = A.L.Ns;
        const int nslots = (X == 1) ? 4 : 2;
        const int nprop = A.prop_kind == PROP_KAT ? 2 : 1;
        const int nitems = nprop + 3 * nslots;
        nodes += count;
        // teams of one warp may hold different channels and batch lengths: every lane runs
        // the same sequence of warp syncs, bounded by the warp's longest batch
        int mx = count;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
        // phase A: scalar work of all nodes of the batch, split over the team's lanes
        for (int it = tl; it < count * nitems; it += T) {
            const int j = it / nitems, item = it - j * nitems;
            NodeScratch<R, C>& ns = ts.node[j];
            const double xj = ns.x;
            const SetupT v = SetupT(xj);
            if (item < nprop) {
                if constexpr (sizeof(R) == 4)
                    ns.p_half[item] = prop_half_ff(A.prop_kind, item, X, M, A.L.Nsig, A.prop_a, A.prop_da,
                                                   (float)A.Lam, v, W);
                else
                    ns.p_half[item] = prop_half<double>(A.prop_kind, item, X, M, A.L.Nsig, A.prop_a64, A.prop_da64,
                                                        A.Lam, v, W);
            } else {
                const int k = item - nprop;
                const int slot = k / 3, ch = k - 3 * slot;
                Plan<R>& P = ns.plan[slot][ch];
                if (A.mask[X][slot] & (1 << ch)) {
                    SetupT a0, a1, a2;
                    slot_arg<SetupT>(X, slot, ch, v, W, V, VP, a0, a1, a2);
                    if constexpr (sizeof(R) == 4) {
                        const float scale = fabsf(v.h) + fabsf(W.h) + (isinf(V.h) ? 0.f : fabsf(V.h)) +
                                            (isinf(VP.h) ? 0.f : fabsf(VP.h));
                        if (ff_near_switch(a0, scale, M, A.L.NO, A.L.Nn) || ff_near_switch(a1, scale, M, A.L.NO, A.L.Nn) ||
                            ff_near_switch(a2, scale, M, A.L.NO, A.L.Nn)) {
                            // the FP64 path's rounding decides the side of a buffer switch
                            const MeshG<double> M64 = mesh_view(A.mesh, A.L.Nsig, A.L.NO, A.L.Nn);
                            double W64, V64, VP64, b0, b1, b2;
                            task_freqs(A, M64, ti, W64, V64, VP64);
                            slot_arg<double>(X, slot, ch, xj, W64, V64, VP64, b0, b1, b2);
                            make_plan<R>(P, ch, b0, b1, b2, M64, Ns, A.L.NO, A.L.Nn);
                        } else {
                            make_plan_ff(P, ch, a0, a1, a2, M, Ns, A.L.NO, A.L.Nn);
                        }
                    } else {
                        make_plan<R>(P, ch, a0, a1, a2, M, Ns, A.L.NO, A.L.Nn);
                    }
                } else {
                    P.kernel = 0;
                }
            }
        }
        __syncwarp();
        if (X == 1) {
            // local vertices at site 1 (flow_su2_t.jl:46-48, flow_u1_dm_t.jl:44-46)
            const int e0 = ldg(A.exch);
            for (int it = tl; it < count * 2 * C; it += T) {
                const int j = it / (2 * C), q = it - j * (2 * C);
                ts.node[j].loc[q] = gather_one<R, C>(A, ts.node[j], 2 + q / C, q % C, 0, e0);
            }
        }
        __syncwarp();
        if (A.node_counter && tl == 0) {
            for (int j = 0; j < count; ++j) {
                unsigned long long cs = 0, c1 = 0;
                for (int s = 0; s < nslots; ++s)
                    for (int ch = 0; ch < 3; ++ch) (s < 2 ? cs : c1) += corners_of(ts.node[j].plan[s][ch].kernel);
                unsigned long long v = cs * Ns + c1 + 3ull * Ns;
                if (X == 1) v += 2ull * row_off[Ns];
                alg += v * C;
            }
        }
        if constexpr (C == 2) {
            // every team of the warp passes the same two warp barriers, whatever its channel
            eval_su2_nodes(X, count, sink);
            __syncwarp();
            if (X == 1) eval_t_overlap(count, sink);
            __syncwarp();
            return;
        }
        // phase B of U(1)-DM: gathers and per-site combination, node by node
        for (int j = 0; j < mx; ++j) {
            const bool act = j < count;
            const NodeScratch<R, C>& ns = ts.node[act ? j : 0];
            R p = (R)0;
            R v1[C][SPL], v2[C][SPL];
            if (act) {
                p = (nprop == 2) ? ns.p_half[0] + ns.p_half[1] : ns.p_half[0];
                gather_slot<R, T, SPL, C>(A, ns, 0, tl, site_ex, v1);
                gather_slot<R, T, SPL, C>(A, ns, 1, tl, site_ex, v2);
            }
            eval_u1dm(X, j, act, p, ns, v1, v2, sink);
        }
    }

    // One non-local vertex slot of an SU(2) node on this lane's sites (get_Γ_avx!,
    // action_su2.jl:115-134): bare + Σ_ch sgn Σ_q w_q q[off_q + site], channels in the reference's
    // order.  A channel's corners are walked by a loop (smaller code and fewer live registers than
    // all eight unrolled: 113 instead of 127 for the FP32 32x2 kernel, 155 instead of 229 for the
    // FP64 one; 4-8 % faster), the FP32 loop two corners at a time (the reads of two corners for both
    // components and all of the lane's sites in flight together: a further 3-4 %; four at a time
    // was slower); the loop over the sites has no branch (padding sites read site 0 and are zeroed
    // at the end).
    __device__ __forceinline__ void gather_su2(const NodeScratch<R, C>& ns, int slot, R v[2][SPL]) {
        const int Ns = A.L.Ns;
        const R* __restrict__ src = A.src[slot];
        int si[SPL];
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const int i = tl + k * T;
            si[k] = i < Ns ? i : 0;
        }
        if constexpr (sizeof(R) == 4) {
            // FP32 copies hold (spin, density) pairs: one 8-byte read per corner and site
            const float2* __restrict__ src2 = reinterpret_cast<const float2*>(src);
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const float2 b = ldg(src2 + A.L.pbare() + si[k]);
                v[0][k] = b.x;
                v[1][k] = b.y;
            }
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                const Plan<R>& P = ns.plan[slot][ch];
                const int kern = P.kernel;
                if (!kern) continue;
                const int nc = corners_of(kern);
                const float2* q = src2 + A.L.pq(P.src_ch, kern - 1);
                const R sgn_d = P.sgn_d;
                const int ex = P.exch;
                int st[SPL];
                R a0[SPL], a1[SPL];
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    st[k] = ex ? site_ex[k] : si[k];
                    a0[k] = a1[k] = (R)0;
                }
#pragma unroll 2
                for (int c = 0; c < nc; ++c) {
                    const R w = P.w[c];
                    const int off = P.off[c];
#pragma unroll
                    for (int k = 0; k < SPL; ++k) {
                        const float2 t = ldg(q + off + st[k]);
                        a0[k] += w * t.x;
                        a1[k] += w * t.y;
                    }
                }
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    v[0][k] += a0[k];
                    v[1][k] += sgn_d * a1[k];
                }
            }
#pragma unroll
            for (int k = 0; k < SPL; ++k)
                if (tl + k * T >= Ns) v[0][k] = v[1][k] = (R)0;
            return;
        }
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            v[0][k] = ldg(src + A.L.bare(0) + si[k]);
            v[1][k] = ldg(src + A.L.bare(1) + si[k]);
        }
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const Plan<R>& P = ns.plan[slot][ch];
            const int kern = P.kernel;
            if (!kern) continue;
            const int nc = corners_of(kern);
            const R* q0 = src + A.L.qbase(0, P.src_ch, kern - 1);
            const R* q1 = src + A.L.qbase(1, P.src_ch, kern - 1);
            const R sgn_d = P.sgn_d;
            const int ex = P.exch;
            int st[SPL];
            R a0[SPL], a1[SPL];
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                st[k] = ex ? site_ex[k] : si[k];
                a0[k] = a1[k] = (R)0;
            }
#pragma unroll 1
            for (int q = 0; q < nc; ++q) {
                const R w = P.w[q];
                const int off = P.off[q];
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    a0[k] += w * ldg(q0 + off + st[k]);
                    a1[k] += w * ldg(q1 + off + st[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                v[0][k] += a0[k];
                v[1][k] += sgn_d * a1[k];
            }
        }
#pragma unroll
        for (int k = 0; k < SPL; ++k)
            if (tl + k * T >= Ns) v[0][k] = v[1][k] = (R)0;
    }

    // phase B of SU(2), node by node: the s and u bubbles (flow_su2_s.jl, flow_su2_u.jl) per site,
    // handed to the sink, or for the t channel (flow_su2_t.jl:46-81) the local part per site kept in
    // shared memory and both slots staged as [site][node] (spin, density) pairs for the overlap sums
    template <class Sink>
    __device__ __forceinline__ void eval_su2_nodes(int X, int count, Sink& sink) {
        constexpr int NB = BatchOf<T, C, SPL>::NB;
        using R2 = typename std::conditional<sizeof(R) == 4, float2, double2>::type;
        const int Ns = A.L.Ns;
        constexpr int SS = t_site_stride<R, NB>();
        R2* tb1 = reinterpret_cast<R2*>(tmp);  // [Ns][SS]
        R2* tb2 = tb1 + (size_t)Ns * SS;
        R2* tloc = tb2 + (size_t)Ns * SS + (size_t)Ns * NB;  // [Ns][NB] local parts (after the overlap sums)
        const R two = (X == 0) ? (R)-2 : (R)2;
        for (int j = 0; j < count; ++j) {
            const NodeScratch<R, C>& ns = ts.node[j];
            const R p = ns.p_half[0] + (A.prop_kind == PROP_KAT ? ns.p_half[1] : (R)0);
            R v1[2][SPL], v2[2][SPL];
            gather_su2(ns, 0, v1);
            gather_su2(ns, 1, v2);
            if (X != 1) {
                R g[2][SPL];
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    g[0][k] = -p * (two * v1[0][k] * v2[0][k] + v1[0][k] * v2[1][k] + v1[1][k] * v2[0][k]);
                    g[1][k] = -p * ((R)3 * v1[0][k] * v2[0][k] + v1[1][k] * v2[1][k]);
                }
                sink(j, g);
                continue;
            }
            const R v3s = ns.loc[0], v3d = ns.loc[1], v4s = ns.loc[2], v4d = ns.loc[3];
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                const R v1s = v1[0][k], v1d = v1[1][k], v2s = v2[0][k], v2d = v2[1][k];
                if (i < Ns) {
                    const R Gs = -p * ((R)-1 * v1s * v4s + v1s * v4d - (R)1 * v3s * v2s + v3d * v2s);
                    const R Gd = -p * ((R)3 * v1d * v4s + v1d * v4d + (R)3 * v3s * v2d + v3d * v2d);
                    tloc[(size_t)i * NB + j] = R2{Gs, Gd};
                    tb1[(size_t)i * SS + j] = R2{v1s, v1d};
                    tb2[(size_t)i * SS + j] = R2{v2s, v2d};
                }
            }
        }
    }

    // second half: the overlap sums (flow_su2_t.jl:66-75) of the whole batch.  All lanes walk the
    // sites in the same order; a lane takes every T-th row of a site, decodes it once and adds the
    // row's product for every node of the batch (the (spin, density) pairs of a site's nodes are
    // neighbours in shared memory: two 16-byte reads per vertex slot and row); the 2 NB partial sums
    // of the lanes meet by shuffles that halve the values a lane carries at every step, and one
    // lane per value stores its total.  Then the owner of a site adds -p (-2) (2S) times them to
    // its nodes' local parts and hands the nodes to the sink.  (The earlier split, NB lanes per row
    // each adding one node, decoded every row NB times: 376 against 352 ms for the pyrochlore
    // L = 6 two-loop right-hand side at 50/15/10 frequencies.)  Nodes past `count` hold stale
    // values whose sums are never used.
    template <class Sink>
    __device__ __forceinline__ void eval_t_overlap(int count, Sink& sink) {
        constexpr int NB = BatchOf<T, C, SPL>::NB;
        using R2 = typename std::conditional<sizeof(R) == 4, float2, double2>::type;
        const int Ns = A.L.Ns;
        constexpr int SS = t_site_stride<R, NB>();
        const R2* tb1 = reinterpret_cast<const R2*>(tmp);
        const R2* tb2 = tb1 + (size_t)Ns * SS;
        R2* ov = const_cast<R2*>(tb2) + (size_t)Ns * SS;  // [Ns][NB] overlap sums
        const R2* tloc = ov + (size_t)Ns * NB;
        const unsigned team_mask = (T == 32) ? kFull : (((1u << T) - 1u) << ((threadIdx.x & 31) / T * T));
        constexpr int V = 2 * NB;  // sums per site: (spin, density) of every node of the batch
        R* ovr = reinterpret_cast<R*>(ov);
        for (int i = 0; i < Ns; ++i) {
            R x[V];
#pragma unroll
            for (int v = 0; v < V; ++v) x[v] = (R)0;
            const int j1 = row_off[i + 1];
#pragma unroll 2
            for (int r = row_off[i] + tl; r < j1; r += T) {
                const unsigned row = rows[r];
                const int ia = row & 0xff, ib = (row >> 8) & 0xff;
                const R m = (R)(row >> 16);
                const R2* pa = tb1 + (size_t)ia * SS;
                const R2* pb = tb2 + (size_t)ib * SS;
                if constexpr (sizeof(R) == 4 && NB % 2 == 0) {
#pragma unroll
                    for (int j2 = 0; j2 < NB / 2; ++j2) {
                        const float4 a = reinterpret_cast<const float4*>(pa)[j2];
                        const float4 b = reinterpret_cast<const float4*>(pb)[j2];
                        x[4 * j2 + 0] += m * a.x * b.x;
                        x[4 * j2 + 1] += m * a.y * b.y;
                        x[4 * j2 + 2] += m * a.z * b.z;
                        x[4 * j2 + 3] += m * a.w * b.w;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < NB; ++j) {
                        const R2 a = pa[j], b = pb[j];
                        x[2 * j] += m * a.x * b.x;
                        x[2 * j + 1] += m * a.y * b.y;
                    }
                }
            }
            // sum over the team's lanes, halving the values each lane carries at every step
            int n = V, idx = 0;
#pragma unroll
            for (int o = T / 2; o >= 1; o >>= 1) {
                if (n > 1) {
                    n >>= 1;
                    const bool up = (tl & o) != 0;
#pragma unroll
                    for (int k = 0; k < V / 2; ++k) {
                        if (k < n) {
                            const R send = up ? x[k] : x[k + n];
                            const R keep = up ? x[k + n] : x[k];
                            x[k] = keep + __shfl_xor_sync(team_mask, send, o);
                        }
                    }
                    if (up) idx += n;
                } else {
                    x[0] += __shfl_xor_sync(team_mask, x[0], o);
                }
            }
            // every lane now holds the total of value idx; one lane per value writes it
            if ((tl & (T / V - 1)) == 0) ovr[((size_t)i * NB) * 2 + idx] = x[0];
        }
        __syncwarp(team_mask);
        const R twoS = (R)A.twoS;
#pragma unroll
        for (int jj = 0; jj < NB; ++jj) {
            if (jj >= count) continue;
            const NodeScratch<R, C>& ns = ts.node[jj];
            const R p = ns.p_half[0] + (A.prop_kind == PROP_KAT ? ns.p_half[1] : (R)0);
            const R coef = -p * (R)-2 * twoS;
            R g[2][SPL];
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                g[0][k] = g[1][k] = (R)0;
                if (i < Ns) {
                    const R2 lo = tloc[(size_t)i * NB + jj], s = ov[(size_t)i * NB + jj];
                    g[0][k] = lo.x + coef * s.x;
                    g[1][k] = lo.y + coef * s.y;
                }
            }
            sink(jj, g);
        }
    }

    // phase B of one node for U(1)-DM (flow_u1_dm_{s,t,u}.jl); team-collective like eval
    template <class Sink>
    __device__ void eval_u1dm(int X, int j, bool act, R p, const NodeScratch<R, C>& ns, const R v1[C][SPL],
                              const R v2[C][SPL], Sink& sink) {
        const int Ns = A.L.Ns;
        if (act && X != 1) {
            R g[C][SPL];
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                R a[C], b[C], h[C];
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    a[c] = v1[c][k];
                    b[c] = v2[c][k];
                }
                if (X == 0) u1dm_s(a, b, h);
                else u1dm_u(a, b, h);
#pragma unroll
                for (int c = 0; c < C; ++c) g[c][k] = -p * h[c];
                if (A.reduced) {
                    // the reduced s bubble of the SDE keeps xx, zz, dd (SDE_u1_dm.jl:38-46)
                    g[2][k] = (R)0;
                    g[4][k] = (R)0;
                    g[5][k] = (R)0;
                }
            }
            sink(j, g);
        }
        const bool tch = act && X == 1;
        if (tch) {
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                if (i < Ns) {
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        tmp[c * Ns + i] = v1[c][k];
                        tmp[(C + c) * Ns + i] = v2[c][k];
                    }
                }
            }
        }
        __syncwarp();
        if (tch) {
            const R coef = -p * (R)-2;
            R g[C][SPL];
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                R a[C], b[C], G[C];
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    a[c] = v1[c][k];
                    b[c] = v2[c][k];
                }
                u1dm_t(a, b, ns.loc, ns.loc + C, G);
#pragma unroll
                for (int c = 0; c < C; ++c) G[c] = -p * G[c];
                if (i < Ns) {
                    // overlap sum (flow_u1_dm_t.jl:86-110)
                    const int j0 = row_off[i], j1 = row_off[i + 1];
                    for (int r = j0; r < j1; ++r) {
                        const unsigned row = rows[r];
                        const int ia = row & 0xff, ib = (row >> 8) & 0xff;
                        const R mm = coef * (R)(row >> 16);
                        const R* t1 = tmp + ia;
                        const R* t2 = tmp + C * Ns + ib;
                        G[0] += mm * (t1[0] * t2[0] - t1[2 * Ns] * t2[2 * Ns]);
                        G[1] += mm * (t1[Ns] * t2[Ns] - t1[4 * Ns] * t2[5 * Ns]);
                        G[2] += mm * (t1[2 * Ns] * t2[0] + t1[0] * t2[2 * Ns]);
                        G[3] += mm * (t1[3 * Ns] * t2[3 * Ns] - t1[5 * Ns] * t2[4 * Ns]);
                        G[4] += mm * (t1[4 * Ns] * t2[3 * Ns] + t1[Ns] * t2[4 * Ns]);
                        G[5] += mm * (t1[3 * Ns] * t2[5 * Ns] + t1[5 * Ns] * t2[Ns]);
                    }
                }
#pragma unroll
                for (int c = 0; c < C; ++c) g[c][k] = G[c];
            }
            sink(j, g);
        }
        __syncwarp();
    }
};

// ---------------------------------------------------------------------------
// wave workspace (device scratch of a pass; one block carved into arrays)
// ---------------------------------------------------------------------------
constexpr int kChunk = 32;      // nodes per chunk
// chunks per subdomain and level (bigger levels use bigger chunks): the deepest subdomains set the
// length of a pass, so their levels are spread over up to 256 teams (measured on the pyrochlore
// L = 6 two-loop state: 7 % faster than 64 chunks; 1024 gave the same as 256)
constexpr int kMaxChunks = 256;

// Queue the next level (n new nodes) of subdomain sub into wave parity `par`.
__device__ __forceinline__ void enqueue(WaveSpace& Wsp, int par, int sub, long long n) {
    long long nch = (n + kChunk - 1) / kChunk;
    if (nch > kMaxChunks) nch = kMaxChunks;
    const long long per = (n + nch - 1) / nch;
    nch = (n + per - 1) / per;
    const int base = atomicAdd(&Wsp.counters[par], (int)nch);
    if (base + nch > Wsp.qcap) {
        atomicOr(&Wsp.counters[4], 1);
        Wsp.subs[sub].n = 0;
        return;
    }
    for (int k = 0; k < nch; ++k) {
        const long long f = k * per;
        const long long c = (f + per <= n) ? per : n - f;
        Wsp.queue[par][base + k] = make_int4(sub, (int)f, (int)c, 0);
    }
    Wsp.subs[sub].chunk0 = base;
    Wsp.subs[sub].nchunk = (int)nch;
    Wsp.subs[sub].n = n;
    const int a = atomicAdd(&Wsp.counters[2 + par], 1);
    Wsp.active[par][a] = sub;
}

// the meshes of the node setup (shared memory): FP64 for the FP64 path, float-float pairs for the
// mixed path
template <typename R>
__device__ __forceinline__ auto setup_mesh(const PassArgs<R>& A, const unsigned char* smem) {
    if constexpr (sizeof(R) == 4) return mesh_view_ff(reinterpret_cast<const float*>(smem), A.L.Nsig, A.L.NO, A.L.Nn);
    else return mesh_view(reinterpret_cast<const double*>(smem), A.L.Nsig, A.L.NO, A.L.Nn);
}

template <typename R>
__device__ __forceinline__ void task_freqs(const PassArgs<R>& A, const MeshFF& M, const TaskInfo& ti, FF& W, FF& V,
                                           FF& VP) {
    const int oO = (ti.X == 1) ? M.Ot() : M.Os();
    const int on = (ti.X == 1) ? M.nt() : M.ns();
    const FF inf{INFINITY, 0.f};
    W = M.at(oO, ti.w1);
    V = (ti.kernel == 2 || ti.kernel == 4) ? M.at(on, ti.w2) : inf;
    VP = (ti.kernel == 3 || ti.kernel == 4) ? M.at(on, ti.w3) : inf;
}

template <typename R>
__device__ __forceinline__ void task_freqs(const PassArgs<R>& A, const MeshG<double>& M, const TaskInfo& ti, double& W,
                                           double& V, double& VP) {
    const double* Om = (ti.X == 1) ? M.Ot : M.Os;
    const double* nu = (ti.X == 1) ? M.nt : M.ns;
    const double inf = INFINITY;
    W = Om[ti.w1];
    V = (ti.kernel == 2 || ti.kernel == 4) ? nu[ti.w2] : inf;
    VP = (ti.kernel == 3 || ti.kernel == 4) ? nu[ti.w3] : inf;
}

// shared-memory layout common to the wave kernels
template <typename R, int T, int C, int SPL>
struct SmemLayout {
    static constexpr int NPW = 32 / T;
    // t-channel staging per team: SU(2) both slots, the overlap sums and the local parts of the
    // whole batch, U(1)-DM one node
    __host__ __device__ static size_t tmp_per_team(int Ns) {
        return C == 2 ? (size_t)4 * Ns * t_site_stride<R, BatchOf<T, C, SPL>::NB>() + (size_t)4 * Ns * BatchOf<T, C, SPL>::NB
                      : (size_t)2 * C * Ns;
    }
    // the meshes of the node setup: float-float pairs and inverse spacings (mixed path) or FP64
    // values and inverse spacings, nm = Nsig + 2 NO + 2 Nn entries each (the float block ends with the
    // placement parameters of its meshes)
    __host__ __device__ static size_t mesh_bytes(int nm) {
        return sizeof(R) == 4 ? sizeof(float) * (3 * (size_t)nm + kMeshGuess) : 2 * sizeof(double) * (size_t)nm;
    }
    size_t mesh, teams, tmp, rows, total;
    __host__ __device__ SmemLayout(int Ns, int nm, long long R_rows, bool rows_in_smem) {
        mesh = 0;
        teams = (mesh_bytes(nm) + 15) & ~(size_t)15;
        tmp = (teams + sizeof(TeamScratch<R, T, C, SPL>) * kWarps * NPW + 15) & ~(size_t)15;  // 16-byte loads
        rows = tmp + ((sizeof(R) * (size_t)kWarps * NPW * tmp_per_team(Ns) + 15) & ~(size_t)15);
        total = rows + (rows_in_smem ? sizeof(unsigned) * (size_t)(R_rows + Ns + 1) : 0);
    }
};

template <typename R, int T, int SPL, int C>
__device__ __forceinline__ Team<R, T, SPL, C> make_team(const PassArgs<R>& A, unsigned char* smem,
                                                        const typename Team<R, T, SPL, C>::SetupMesh& M, int warp,
                                                        int team, int tl) {
    constexpr int NPW = 32 / T;
    const int Ns = A.L.Ns;
    SmemLayout<R, T, C, SPL> lay(Ns, A.L.Nsig + 2 * A.L.NO + 2 * A.L.Nn, A.rows_total, A.rows_in_smem);
    TeamScratch<R, T, C, SPL>* teams = reinterpret_cast<TeamScratch<R, T, C, SPL>*>(smem + lay.teams);
    R* tmp = reinterpret_cast<R*>(smem + lay.tmp) + (size_t)(warp * NPW + team) * lay.tmp_per_team(Ns);
    const unsigned* rows;
    const int* roff;
    if (A.rows_in_smem) {
        rows = reinterpret_cast<const unsigned*>(smem + lay.rows);
        roff = reinterpret_cast<const int*>(rows + A.rows_total);
    } else {
        rows = A.ov_rows;
        roff = A.ov_off;
    }
    Team<R, T, SPL, C> t{A, M, teams[warp * NPW + team], tmp, rows, roff, tl, {}, 0, 0};
#pragma unroll
    for (int k = 0; k < SPL; ++k) {
        const int i = tl + k * T;
        t.site_ex[k] = i < Ns ? ldg(A.exch + i) : 0;
    }
    return t;
}

template <typename R, int T, int C, int SPL>
__device__ __forceinline__ void load_common(const PassArgs<R>& A, unsigned char* smem) {
    const int nm = A.L.Nsig + 2 * A.L.NO + 2 * A.L.Nn;
    if constexpr (sizeof(R) == 4) {
        float* m = reinterpret_cast<float*>(smem);
        for (int k = threadIdx.x; k < 3 * nm + kMeshGuess; k += blockDim.x) m[k] = ldg(A.mesh_ff + k);
    } else {
        double* m = reinterpret_cast<double*>(smem);
        for (int k = threadIdx.x; k < 2 * nm; k += blockDim.x) m[k] = ldg(A.mesh + k);
    }
    if (A.rows_in_smem) {
        SmemLayout<R, T, C, SPL> lay(A.L.Ns, nm, A.rows_total, true);
        unsigned* rows = reinterpret_cast<unsigned*>(smem + lay.rows);
        for (long long k = threadIdx.x; k < A.rows_total; k += blockDim.x) rows[k] = ldg(A.ov_rows + k);
        int* roff = reinterpret_cast<int*>(rows + A.rows_total);
        for (int k = threadIdx.x; k <= A.L.Ns; k += blockDim.x) roff[k] = ldg(A.ov_off + k);
    }
    __syncthreads();
}

// subdomain range of job `job` of a task (flow_s.jl:29-36; quadrature.jl:84-139); false if empty
template <typename R>
__device__ __forceinline__ bool sub_range(const PassArgs<R>& A, const TaskInfo& ti, int job, double& lo, double& hi,
                                          double& sgn) {
    const double* mesh = A.mesh;
    const double* Om64 = mesh + A.L.Nsig + (ti.X == 1 ? A.L.NO + A.L.Nn : 0);
    const double* nu64 = Om64 + A.L.NO;
    const double ref = A.Lam + 0.5 * Om64[ti.w1];
    const double val = Om64[A.L.NO - 1] + nu64[A.L.Nn - 1];
    const int eval = A.eval;
    const int range = job / eval, sub = job % eval + 1;
    sgn = 1.0;
    if (range == 0 || range == 3) {
        const double a = 2.0 * ref, b = 1.0 * val;
        if (!(b > a)) return false;
        // ξ^k a with libm's pow, computed on the host: an end point at ±val sits on the jump
        // of the vertex read-out at Ω[end] + ν[end] and must round exactly like the reference
        const double* lb = A.log_bounds + (size_t)((ti.X == 1 ? A.L.NO : 0) + ti.w1) * (eval + 1);
        lo = lb[sub - 1];
        hi = lb[sub];
        sgn = range == 0 ? -1.0 : 1.0;
    } else {
        const double a = range == 1 ? -2.0 * ref : 0.0 * ref;
        const double b = range == 1 ? 0.0 * ref : 2.0 * ref;
        if (!(b > a)) return false;
        const double h = (b - a) / eval;
        lo = __dadd_rn(a, __dmul_rn((double)(sub - 1), h));
        hi = __dadd_rn(a, __dmul_rn((double)sub, h));
    }
    return true;
}

// the reference's convergence test of simps! on one team's sites; returns 1 when done
template <int T, int SPL, int C>
__device__ __forceinline__ int simps_test(const double s_old[C][SPL], const double s_new[C][SPL], long long n,
                                          double atol, double rtol, int team, bool in_team0_only) {
    double ss_r = 0.0, ss_n = 0.0, ss_d = 0.0;
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const double rich = s_old[c][k] * (-1.0 / 15.0) + (16.0 / 15.0) * s_new[c][k];
            const double dd = rich - s_new[c][k];
            ss_r += rich * rich;
            ss_n += s_new[c][k] * s_new[c][k];
            ss_d += dd * dd;
        }
    (void)team;
    (void)in_team0_only;
    ss_r = in_team_sum<T>(ss_r);
    ss_n = in_team_sum<T>(ss_n);
    ss_d = in_team_sum<T>(ss_d);
    const double adiff = sqrt(ss_d);
    const double rdiff = adiff / fmax(sqrt(ss_r), sqrt(ss_n));
    // a non-finite integrand stops refining at once (the reference would refine it to n > 2^20);
    // the result's finite check then reports it
    return (adiff < atol || rdiff < rtol || 2 * n > (1ll << 20) || !isfinite(adiff)) ? 1 : 0;
}

// The same test on the FP32 pass of the mixed path: 1 done, 0 next level, 2 hand the subdomain to
// the FP64 pass.  sa_old / sa_new bound the norms of the Simpson sums taken over |node values|
// with |weights|; with node values rounded by at most eps of their magnitude the FP64 sums lie
// within eps sa of the FP32 ones, so when the test is closer to one of its bounds than that
// margin the FP64 evaluation of the same nodes could decide the other way, and the subdomain is
// evaluated again in FP64 from its first level (all its decisions then are the FP64 path's).
template <int T, int SPL, int C>
__device__ __forceinline__ int simps_decide(const double s_old[C][SPL], const double s_new[C][SPL], long long n,
                                            double atol, double rtol, double eps, double sa_old, double sa_new) {
    double ss_r = 0.0, ss_n = 0.0, ss_d = 0.0;
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const double rich = s_old[c][k] * (-1.0 / 15.0) + (16.0 / 15.0) * s_new[c][k];
            const double dd = rich - s_new[c][k];
            ss_r += rich * rich;
            ss_n += s_new[c][k] * s_new[c][k];
            ss_d += dd * dd;
        }
    ss_r = in_team_sum<T>(ss_r);
    ss_n = in_team_sum<T>(ss_n);
    ss_d = in_team_sum<T>(ss_d);
    const double adiff = sqrt(ss_d);
    const double den = fmax(sqrt(ss_r), sqrt(ss_n));
    if (2 * n > (1ll << 20) || !isfinite(adiff)) return 1;
    const int done = (adiff < atol || adiff / den < rtol) ? 1 : 0;
    const double E = eps * (sa_new + sa_old) / 15.0;          // |Δ64 - Δ32|
    const double Es = eps * (16.0 * sa_new + sa_old) / 15.0;  // change of the norms in the bound
    const bool can_done = adiff - E < atol || adiff - E < rtol * (den + Es);
    const bool can_go = adiff + E >= atol && adiff + E >= rtol * fmax(den - Es, 0.0);
    return (can_done && can_go) ? 2 : done;
}

// norm of a team's per-site values
template <int T, int SPL, int C>
__device__ __forceinline__ double team_norm(const double v[C][SPL]) {
    double ss = 0.0;
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
        for (int k = 0; k < SPL; ++k) ss += v[c][k] * v[c][k];
    return sqrt(in_team_sum<T>(ss));
}

// hand a subdomain from the FP32 pass to the FP64 pass (team lane 0)
__device__ __forceinline__ void hand_off(WaveSpace& Wsp, int sub) {
    Wsp.subs[sub].n = 0;
    Wsp.esc[atomicAdd(&Wsp.counters[5], 1)] = sub;
}

// ---- wave 0: first five nodes of every subdomain, boundary nodes, first test ----
template <typename R, int T, int SPL, int C>
__global__ void __launch_bounds__(kWarps * 32) wave0_kernel(PassArgs<R> A, WaveSpace Wsp) {
    constexpr int NPW = 32 / T;
    extern __shared__ __align__(16) unsigned char smem[];
    load_common<R, T, C, SPL>(A, smem);
    const auto M = setup_mesh(A, smem);  // staged in shared memory by load_common
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int team = lane / T, tl = lane % T;
    Team<R, T, SPL, C> tm = make_team<R, T, SPL, C>(A, smem, M, warp, team, tl);
    const int Ns = A.L.Ns;
    const int jobs = 4 * A.eval + 1;
    const long long nwarps = (long long)gridDim.x * kWarps;
    constexpr int NB = BatchOf<T, C, SPL>::NB;
    // the FP64 pass of the mixed path starts only the subdomains the FP32 pass handed to it
    const int nwork = A.esc_mode == 2 ? Wsp.counters[5] : Wsp.nsub;
    for (long long base = ((long long)blockIdx.x * kWarps + warp) * NPW; base < nwork; base += nwarps * NPW) {
        const bool valid = base + team < nwork;
        const int sub = !valid ? 0 : (A.esc_mode == 2 ? Wsp.esc[base + team] : (int)(base + team));
        TaskInfo ti{0, 1, 0, 0, 0};
        int job = 0, cnt = 0;
        double x[8], lo = 0, hi = 0, sgn = 1;
        double c0 = 0, c1 = 0;
        bool boundary = false;
        if (valid) {
            ti = task_of(A, sub, jobs);
            job = sub % jobs;
            if (job == 4 * A.eval) {
                const double* Om64 = A.mesh + A.L.Nsig + (ti.X == 1 ? A.L.NO + A.L.Nn : 0);
                const double val = Om64[A.L.NO - 1] + Om64[A.L.NO + A.L.Nn - 1];
                x[0] = -val;
                x[1] = val;
                c0 = A.corrs[0 + 2 * (ti.X + 3 * ti.w1)];
                c1 = A.corrs[1 + 2 * (ti.X + 3 * ti.w1)];
                cnt = 2;
                boundary = true;
            } else if (sub_range(A, ti, job, lo, hi, sgn)) {
                const double mid = 0.5 * (lo + hi);
                const double h = 0.5 * (hi - lo) / 2.0;
                x[0] = sgn * lo;
                x[1] = sgn * __dadd_rn(lo, __dmul_rn(1.0, h));
                x[2] = sgn * mid;
                x[3] = sgn * __dadd_rn(lo, __dmul_rn(3.0, h));
                x[4] = sgn * hi;
                cnt = 5;
            }
        }
        typename Team<R, T, SPL, C>::SetupT W(0.0), V(0.0), VP(0.0);
        if (valid) task_freqs(A, M, ti, W, V, VP);
        // all teams of the warp evaluate together (cnt = 0 for idle teams), NB nodes at a time
        R g[5][C][SPL];
        for (int b = 0; b < 5; b += NB) {
            const int nb = max(0, min(NB, cnt - b));
            for (int j = tl; j < nb; j += T) tm.ts.node[j].x = x[b + j];
            __syncwarp();
            auto keep = [&](int j, const R (&gv)[C][SPL]) {
#pragma unroll
                for (int c = 0; c < C; ++c)
#pragma unroll
                    for (int k = 0; k < SPL; ++k) g[b + j][c][k] = gv[c][k];
            };
            tm.eval(ti, W, V, VP, nb, keep);
        }
        const bool simpson = valid && !boundary && cnt == 5;
        // simps!: 3-point sum, 5-point sum via residual! with n = 2, Richardson test
        const double we = 1.0 * (hi - lo) / 6.0, wm = 2.0 * (hi - lo) / 3.0;
        const double h = 0.5 * (hi - lo) / 2.0;
        const double wn = 4.0 * h / 3.0, wo = -2.0 * h / 3.0;
        double s_old[C][SPL], s_new[C][SPL], f_new[C][SPL];
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                s_old[c][k] = s_new[c][k] = f_new[c][k] = 0.0;
                if (!simpson) continue;
                s_old[c][k] = we * (double)g[0][c][k];
                s_old[c][k] += wm * (double)g[2][c][k];
                s_old[c][k] += we * (double)g[4][c][k];
                f_new[c][k] = (double)g[1][c][k] + (double)g[3][c][k];
                s_new[c][k] = 0.5 * s_old[c][k] + wn * f_new[c][k] + wo * (double)g[2][c][k];
            }
        // every lane takes part in the test's team reductions
        int done;
        double sa_new = 0.0, fab = 0.0;
        if (A.esc_mode == 1) {
            double a_old[C][SPL], a_new[C][SPL], a_f[C][SPL];
#pragma unroll
            for (int c = 0; c < C; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    a_old[c][k] = a_new[c][k] = a_f[c][k] = 0.0;
                    if (!simpson) continue;
                    a_old[c][k] = we * fabs((double)g[0][c][k]) + wm * fabs((double)g[2][c][k]) +
                                  we * fabs((double)g[4][c][k]);
                    a_f[c][k] = fabs((double)g[1][c][k]) + fabs((double)g[3][c][k]);
                    a_new[c][k] = 0.5 * a_old[c][k] + fabs(wn) * a_f[c][k] + fabs(wo) * fabs((double)g[2][c][k]);
                }
            const double sa_old = team_norm<T, SPL, C>(a_old);
            sa_new = team_norm<T, SPL, C>(a_new);
            fab = team_norm<T, SPL, C>(a_f);
            done = simps_decide<T, SPL, C>(s_old, s_new, 2, A.atol, A.rtol, A.esc_eps, sa_old, sa_new);
        } else {
            done = simps_test<T, SPL, C>(s_old, s_new, 2, A.atol, A.rtol, team, false);
        }
        if (!valid) continue;
        if (simpson && done == 2) {
            if (tl == 0) hand_off(Wsp, sub);
            continue;
        }
        double* sA = Wsp.stA + (size_t)sub * C * Ns;
        double* sB = Wsp.stB + (size_t)sub * C * Ns;
        if (!simpson) {
            // boundary corrections (two nodes weighted by corrs) or an empty range
#pragma unroll
            for (int c = 0; c < C; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    const int i = tl + k * T;
                    if (i < Ns) sA[c * Ns + i] = boundary ? c0 * (double)g[0][c][k] + c1 * (double)g[1][c][k] : 0.0;
                }
            if (tl == 0) Wsp.subs[sub].n = 0;
            continue;
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                if (i >= Ns) continue;
                if (done) {
                    sA[c * Ns + i] = (s_old[c][k] * (-1.0 / 15.0) + (16.0 / 15.0) * s_new[c][k] - s_new[c][k]) + s_new[c][k];
                } else {
                    sA[c * Ns + i] = s_new[c][k];
                    sB[c * Ns + i] = f_new[c][k];
                }
            }
        if (tl == 0) {
            SubRec& S = Wsp.subs[sub];
            S.lo = lo;
            S.hi = hi;
            S.sgn = sgn;
            S.sa = sa_new;
            S.fab = fab;
            if (done) S.n = 0;
            else enqueue(Wsp, 1, sub, 4);
        }
    }
    if (A.node_counter && tl == 0) {
        atomicAdd(A.node_counter, tm.nodes);
        atomicAdd(A.node_counter + 1, tm.alg);
    }
}

// ---- wave k >= 1: evaluate queued chunks, one partial node sum per chunk ----
// (FP32 kernels: SU(2) teams with at most two sites per lane held to 128 registers, four blocks of 128
// threads per SM, where their gathers do not spill (3-5 % faster than three blocks on the pyrochlore L = 6
// and square L = 5, 8 states); wider lanes and U(1)-DM entries, whose gathers spill at 128, held to 168
// registers, three blocks)
template <typename R, int T, int SPL, int C>
constexpr int eval_min_blocks() { return sizeof(R) == 4 ? (C == 2 && SPL <= 2 ? 4 : 3) : 1; }

template <typename R, int T, int SPL, int C>
__global__ void __launch_bounds__(kWarps * 32, eval_min_blocks<R, T, SPL, C>()) eval_kernel(PassArgs<R> A, WaveSpace Wsp, int par) {
    constexpr int NPW = 32 / T;
    extern __shared__ __align__(16) unsigned char smem[];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // the next level's queue starts empty (its chunks are enqueued by this wave's decide_kernel)
        Wsp.counters[par ^ 1] = 0;
        Wsp.counters[2 + (par ^ 1)] = 0;
    }
    // blocks without a chunk leave before staging the meshes and rows
    if ((long long)blockIdx.x * kWarps * NPW >= Wsp.counters[par]) return;
    load_common<R, T, C, SPL>(A, smem);
    const auto M = setup_mesh(A, smem);  // staged in shared memory by load_common
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int team = lane / T, tl = lane % T;
    Team<R, T, SPL, C> tm = make_team<R, T, SPL, C>(A, smem, M, warp, team, tl);
    const int Ns = A.L.Ns;
    const int jobs = 4 * A.eval + 1;
    // a level whose chunks overflowed the queue counted them all; only the first qcap were filed
    const int nchunks = min(Wsp.counters[par], Wsp.qcap);
    const long long nwarps = (long long)gridDim.x * kWarps;
    constexpr int NB = BatchOf<T, C, SPL>::NB;
    for (long long base = ((long long)blockIdx.x * kWarps + warp) * NPW; base < nchunks; base += nwarps * NPW) {
        const int chunk = (int)(base + team);
        const bool valid = chunk < nchunks;
        int4 cr = make_int4(0, 0, 0, 0);
        TaskInfo ti{0, 1, 0, 0, 0};
        double lo = 0, h = 0, sgn = 1;
        typename Team<R, T, SPL, C>::SetupT W(0.0), V(0.0), VP(0.0);
        if (valid) {
            cr = Wsp.queue[par][chunk];
            const SubRec S = Wsp.subs[cr.x];
            ti = task_of(A, cr.x, jobs);
            task_freqs(A, M, ti, W, V, VP);
            lo = S.lo;
            sgn = S.sgn;
            h = 0.5 * (S.hi - S.lo) / (double)S.n;
        }
        // the longest chunk of the warp's teams bounds the batch loop
        int cnt = valid ? cr.z : 0;
        int mx = cnt;
#pragma unroll
        for (int o = T; o < 32; o <<= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
        Acc<R> acc[C][SPL];
        R aab[C][SPL];  // FP32 pass of the mixed path: sums of |node values|
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                acc[c][k] = Acc<R>{(R)0, (R)0};
                aab[c][k] = (R)0;
            }
        // each node's values go straight into the chunk's compensated sums, in node order
        auto add = [&](int, const R (&gv)[C][SPL]) {
#pragma unroll
            for (int c = 0; c < C; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    acc_add(acc[c][k], gv[c][k]);
                    if constexpr (sizeof(R) == 4) aab[c][k] += fabsf(gv[c][k]);
                }
        };
        for (int b = 0; b < mx; b += NB) {
            const int nb = max(0, min(NB, cnt - b));
            if (tl < nb) {
                const long long nd = (long long)cr.y + b + tl;  // 0-based new node of the level
                tm.ts.node[tl].x = sgn * __dadd_rn(lo, __dmul_rn(2.0 * (double)(nd + 1) - 1.0, h));
            }
            __syncwarp();
            tm.eval(ti, W, V, VP, nb, add);
        }
        if constexpr (sizeof(R) == 4) {
            if (A.esc_mode == 1) {
                double ad[C][SPL];
#pragma unroll
                for (int c = 0; c < C; ++c)
#pragma unroll
                    for (int k = 0; k < SPL; ++k) ad[c][k] = (double)aab[c][k];
                const double nrm = team_norm<T, SPL, C>(ad);  // every lane of the warp takes part
                if (valid && tl == 0) Wsp.part_abs[chunk] = nrm;
            }
        }
        if (!valid) continue;
        double* P = Wsp.part + (size_t)chunk * C * Ns;
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                if (i < Ns) P[c * Ns + i] = (double)acc[c][k].s + (double)acc[c][k].c;
            }
    }
    if (A.node_counter && tl == 0) {
        atomicAdd(A.node_counter, tm.nodes);
        atomicAdd(A.node_counter + 1, tm.alg);
    }
}

// ---- wave k >= 1: per subdomain, next Simpson sum, test, result or next level ----
template <int T, int SPL, int C>
__global__ void __launch_bounds__(kWarps * 32) decide_kernel(WaveSpace Wsp, int Ns, double atol, double rtol, int par,
                                                             int esc_mode, double esc_eps) {
    constexpr int NPW = 32 / T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int team = lane / T, tl = lane % T;
    const int nact = Wsp.counters[2 + par];
    const long long nwarps = (long long)gridDim.x * kWarps;
    for (long long base = ((long long)blockIdx.x * kWarps + warp) * NPW; base < nact; base += nwarps * NPW) {
        const int a = (int)(base + team);
        const bool valid = a < nact;
        const int sub = valid ? Wsp.active[par][a] : 0;
        SubRec S;
        if (valid) S = Wsp.subs[sub];
        else S.n = 1, S.nchunk = 0, S.chunk0 = 0, S.lo = 0, S.hi = 0;
        double* sA = Wsp.stA + (size_t)sub * C * Ns;
        double* sB = Wsp.stB + (size_t)sub * C * Ns;
        double s_old[C][SPL], s_new[C][SPL], f_new[C][SPL];
        const double h = 0.5 * (S.hi - S.lo) / (double)S.n;
        const double wn = 4.0 * h / 3.0, wo = -2.0 * h / 3.0;
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                s_old[c][k] = s_new[c][k] = f_new[c][k] = 0.0;
                if (!valid || i >= Ns) continue;
                double f = 0.0;
                for (int q = 0; q < S.nchunk; ++q) f += Wsp.part[(size_t)(S.chunk0 + q) * C * Ns + c * Ns + i];
                f_new[c][k] = f;
                s_old[c][k] = sA[c * Ns + i];
                s_new[c][k] = 0.5 * s_old[c][k] + wn * f + wo * sB[c * Ns + i];
            }
        int done;
        double sa_new = 0.0, fa_new = 0.0;
        if (esc_mode == 1) {
            for (int q = 0; q < S.nchunk; ++q) fa_new += Wsp.part_abs[S.chunk0 + q];  // triangle bound
            const double sa_old = valid ? S.sa : 0.0;
            sa_new = 0.5 * sa_old + fabs(wn) * fa_new + fabs(wo) * (valid ? S.fab : 0.0);
            done = simps_decide<T, SPL, C>(s_old, s_new, S.n, atol, rtol, esc_eps, sa_old, sa_new);
        } else {
            done = simps_test<T, SPL, C>(s_old, s_new, S.n, atol, rtol, team, false);
        }
        if (!valid) continue;
        if (done == 2) {
            if (tl == 0) hand_off(Wsp, sub);
            continue;
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                if (i >= Ns) continue;
                if (done) {
                    sA[c * Ns + i] = (s_old[c][k] * (-1.0 / 15.0) + (16.0 / 15.0) * s_new[c][k] - s_new[c][k]) + s_new[c][k];
                } else {
                    sA[c * Ns + i] = s_new[c][k];
                    sB[c * Ns + i] = f_new[c][k];
                }
            }
        if (tl == 0) {
            if (done) {
                Wsp.subs[sub].n = 0;
            } else {
                Wsp.subs[sub].sa = sa_new;
                Wsp.subs[sub].fab = fa_new;
                enqueue(Wsp, par ^ 1, sub, 2 * S.n);
            }
        }
    }
}

// ---- sum each task's subdomain results (range order, boundary last) into the output ----
template <typename R, int C>
__global__ void reduce_kernel(PassArgs<R> A, WaveSpace Wsp) {
    const int ct = blockIdx.x;  // channel task
    const int jobs = 4 * A.eval + 1;
    const int Ns = A.L.Ns;
    const TaskInfo ti = task_of(A, ct * jobs, jobs);
    const Layout& L = A.L;
    int64_t off;
    switch (ti.kernel) {
        case 1: off = (int64_t)Ns * ti.w1; break;
        case 2: off = (int64_t)Ns * (ti.w1 + (int64_t)L.NO * ti.w2); break;
        case 3: off = (int64_t)Ns * (ti.w1 + (int64_t)L.NO * ti.w3); break;
        default: off = (int64_t)Ns * (ti.w1 + (int64_t)L.NO * (ti.w2 + (int64_t)L.Nn * ti.w3)); break;
    }
    for (int e = threadIdx.x; e < C * Ns; e += blockDim.x) {
        const int c = e / Ns, i = e % Ns;
        double s = 0.0;
        for (int j = 0; j < jobs; ++j) s += Wsp.stA[((size_t)ct * jobs + j) * C * Ns + c * Ns + i];
        A.out[L.qbase(c, ti.X, ti.kernel - 1) + off + i] = s;
    }
}

// a pass whose chunk queue overflowed reports it in the call's status word (bit 3)
static __global__ void wave_status_kernel(const int* counters, int* status) {
    if (threadIdx.x == 0 && counters[4]) atomicOr(status, 8);
}

// Raise a kernel's dynamic shared-memory limit to the most a block may use, once per process: the
// attribute is process-wide, and contexts of different sizes launch the same kernel from several
// host threads (coupling sweeps), so a per-launch value could be lowered under another thread's
// launch.  Each launch still asks for its own size.
template <auto K>
inline cudaError_t allow_max_dynamic_smem() {
    static const cudaError_t e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    return e;
}

// team width T = lanes per node batch, SPL = sites per lane
template <typename R, int C>
struct PassLauncher {
    template <int T, int SPL>
    static cudaError_t run(const PassArgs<R>& a0, WaveSpace& Wsp, int* h_counters, cudaStream_t st, int grid_cap) {
        // overlap rows in shared memory only while the FP32 eval kernel's register-bound number of
        // blocks (three for FP64) still fits on an SM (228 KB less 1 KB per block; a row word is read
        // once per batch of nodes, so from L1 it costs little)
        PassArgs<R> a = a0;
        const int nm = a.L.Nsig + 2 * a.L.NO + 2 * a.L.Nn;
        const size_t staged = SmemLayout<R, T, C, SPL>(a.L.Ns, nm, a.rows_total, true).total;
        constexpr int fit_kb = 228 / (sizeof(R) == 4 ? eval_min_blocks<R, T, SPL, C>() : 3) - 1;
        a.rows_in_smem = a.rows_mode == 1 ? 0 : (staged <= (size_t)(a.rows_mode == 2 ? 227 : fit_kb) * 1024);
        SmemLayout<R, T, C, SPL> lay(a.L.Ns, nm, a.rows_total, a.rows_in_smem);
        const size_t smem = lay.total;
        if (smem > (size_t)227 * 1024) return cudaErrorInvalidConfiguration;
        cudaError_t e;
        if ((e = allow_max_dynamic_smem<wave0_kernel<R, T, SPL, C>>())) return e;
        if ((e = allow_max_dynamic_smem<eval_kernel<R, T, SPL, C>>())) return e;
        constexpr int NPW = 32 / T;
        const int teams_per_block = kWarps * NPW;
        // the FP64 pass of the mixed path keeps the count of handed subdomains (counters[5])
        if ((e = cudaMemsetAsync(Wsp.counters, 0, sizeof(int) * (a.esc_mode == 2 ? 5 : 6), st))) return e;
        int g0 = (Wsp.nsub + teams_per_block - 1) / teams_per_block;
        // h_counters[7] counts the kernels this pass launches
        wave0_kernel<R, T, SPL, C><<<g0 < grid_cap ? g0 : grid_cap, kWarps * 32, smem, st>>>(a, Wsp);
        ++h_counters[7];
        if ((e = cudaGetLastError())) return e;
        if (a.async_waves) {
            // device-driven levels: every wave reads its chunk and subdomain counts from the device,
            // idle blocks leave at once, and no host round trip separates the waves (the deepest
            // level the reference allows, n > 2^20 new nodes, is reached by wave 20)
            const int gd = std::max(1, std::min(grid_cap, (Wsp.nsub + teams_per_block - 1) / teams_per_block));
            int par = 1;
            for (int wave = 1; wave <= 21; ++wave) {
                eval_kernel<R, T, SPL, C><<<grid_cap, kWarps * 32, smem, st>>>(a, Wsp, par);
                h_counters[7] += 2;
                if ((e = cudaGetLastError())) return e;
                decide_kernel<T, SPL, C><<<gd, kWarps * 32, 0, st>>>(Wsp, a.L.Ns, a.atol, a.rtol, par, a.esc_mode,
                                                                     a.esc_eps);
                if ((e = cudaGetLastError())) return e;
                par ^= 1;
            }
            wave_status_kernel<<<1, 32, 0, st>>>(Wsp.counters, a.status);
            ++h_counters[7];
            if ((e = cudaGetLastError())) return e;
            if (a.esc_mode == 1) return cudaSuccess;  // the FP64 pass finishes and reduces
            reduce_kernel<R, C><<<a.ntasks * a.nchan, 128, 0, st>>>(a, Wsp);
            ++h_counters[7];
            return cudaGetLastError();
        }
        int par = 1;
        for (int wave = 1; wave <= 21; ++wave) {
            if ((e = cudaMemcpyAsync(h_counters, Wsp.counters, sizeof(int) * 5, cudaMemcpyDeviceToHost, st))) return e;
            if ((e = cudaStreamSynchronize(st))) return e;
            if (h_counters[4]) return cudaErrorLaunchOutOfResources;  // chunk queue overflow
            const int nchunks = h_counters[par], nact = h_counters[2 + par];
            if (nact == 0) break;
            // reset the other parity's counters for the next wave's queue
            if ((e = cudaMemsetAsync(Wsp.counters + (par ^ 1), 0, sizeof(int), st))) return e;
            if ((e = cudaMemsetAsync(Wsp.counters + 2 + (par ^ 1), 0, sizeof(int), st))) return e;
            int ge = (nchunks + teams_per_block - 1) / teams_per_block;
            eval_kernel<R, T, SPL, C><<<ge < grid_cap ? ge : grid_cap, kWarps * 32, smem, st>>>(a, Wsp, par);
            h_counters[7] += 2;
            if ((e = cudaGetLastError())) return e;
            int gd = (nact + teams_per_block - 1) / teams_per_block;
            decide_kernel<T, SPL, C><<<gd < grid_cap ? gd : grid_cap, kWarps * 32, 0, st>>>(Wsp, a.L.Ns, a.atol, a.rtol,
                                                                                           par, a.esc_mode, a.esc_eps);
            if ((e = cudaGetLastError())) return e;
            par ^= 1;
        }
        if (a.esc_mode == 1) return cudaSuccess;  // the FP64 pass finishes and reduces
        reduce_kernel<R, C><<<a.ntasks * a.nchan, 128, 0, st>>>(a, Wsp);
        ++h_counters[7];
        return cudaGetLastError();
    }
};

// one team shape of one precision and component count; instantiated explicitly in
// pffrg_shapes.cu (one object per group of shapes, so the kernels compile in parallel)
template <typename R, int C, int T, int SPL>
cudaError_t run_shape(const PassArgs<R>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st, int grid_cap) {
    return PassLauncher<R, C>::template run<T, SPL>(a, Wsp, h_counters, st, grid_cap);
}

// the team shapes built: lanes per node batch x sites per lane
#define PFFRG_TEAM_SHAPES(X) X(8, 1) X(16, 1) X(32, 1) X(16, 3) X(16, 4) X(32, 2) X(32, 3) X(32, 4) X(32, 8)

// the default shape for Ns sites: the narrowest team whose lanes hold at most two sites (up to 64
// sites; measured on the pyrochlore L = 6 two-loop state, 48 sites: 32x2 403 ms, 16x3 460 ms,
// 16x4 511 ms), beyond that 32-lane teams with the fewest sites per lane that cover them (32x3 against
// 32x4: kagome L = 8 U(1)-DM three-loop state, 82 sites, mixed 1445 vs 1823 ms, FP64 4935 vs 5506 ms;
// pyrochlore L = 7 one-loop, 70 sites, mixed 455 vs 502 ms, FP64 2312 vs 2432 ms)
__host__ __device__ inline void default_team_shape(int Ns, int& T, int& SPL) {
    if (Ns <= 8) T = 8, SPL = 1;
    else if (Ns <= 16) T = 16, SPL = 1;
    else if (Ns <= 32) T = 32, SPL = 1;
    else if (Ns <= 64) T = 32, SPL = 2;
    else if (Ns <= 96) T = 32, SPL = 3;
    else if (Ns <= 128) T = 32, SPL = 4;
    else T = 32, SPL = 8;
}

template <typename R, int C>
cudaError_t launch_pass_impl(const PassArgs<R>& a, WaveSpace& Wsp, int* h_counters, cudaStream_t st) {
    const int Ns = a.L.Ns;
    if (a.ntasks == 0) return cudaSuccess;
    if (Ns > 256) return cudaErrorInvalidValue;
    const int cap = 152 * 32;
    int T, S;
    default_team_shape(Ns, T, S);
    if (a.team_T > 0 && a.team_T * a.team_SPL >= Ns) T = a.team_T, S = a.team_SPL;  // a requested shape
#define PFFRG_DISPATCH(t, s) \
    if (T == t && S == s) return run_shape<R, C, t, s>(a, Wsp, h_counters, st, cap);
    PFFRG_TEAM_SHAPES(PFFRG_DISPATCH)
#undef PFFRG_DISPATCH
    return cudaErrorInvalidValue;
}

}  // namespace pffrg

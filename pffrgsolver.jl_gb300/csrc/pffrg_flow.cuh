// Channel-task kernel of the flow right-hand side (sm_103a).
//
// One CTA integrates one channel task (channel X, kernel, w1, w2, w3) of a
// pass, i.e. one call of compute_channel_X_{kat,left,central,BSE}!
// (src/Flow/flow_s.jl:2-173, flow_t.jl, flow_u.jl, BSE_*.jl, SDE.jl:2-56):
//
//   * the 4*eval Simpson subdomains of integrate_log!/integrate_lin!
//     (src/Flow/quadrature.jl:84-139) plus the two boundary nodes are spread
//     over the CTA's warps; every warp runs the adaptive Simpson rule with
//     Richardson extrapolation of simps! (quadrature.jl:27-81) on its
//     subdomains.  The reweighted nodes of residual! (quadrature.jl:2-24) are
//     the previous level's new nodes, so instead of re-evaluating the
//     integrand there the warp keeps their running sum: one third fewer
//     integrand evaluations, identical arithmetic up to rounding order.
//   * inside a warp, a team of T lanes evaluates one node: the lanes split the
//     per-node scalar work (the two propagator halves and the 6 or 12
//     interpolation plans, bubbles.jl and buffer.jl) and then each lane
//     gathers and combines the vertex on its sites (flow_su2_{s,t,u}.jl); the
//     t channel stages both vertex slots in shared memory for the overlap sum
//     (flow_su2_t.jl:66-75).  32/T nodes are evaluated per warp at once.
//   * the per-level convergence test (Frobenius norms over all components and
//     sites) and the stage bookkeeping are FP64; the integrand runs in R
//     (double, or float with compensated summation of the node sums).
#pragma once

#include "pffrg_internal.h"

namespace pffrg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarps = 4;
constexpr int kC = 2;  // SU(2): spin and density components

template <typename R>
struct TeamScratch {
    R p_half[2];
    R loc[4];  // t channel: v3s, v3d, v4s, v4d
    Plan<R> plan[4][3];
};

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

// vertex component c of one slot at site i (get_Γ_comp_avx!, Action.jl:110-167)
template <typename R>
__device__ __forceinline__ R gather(const PassArgs<R>& A, const TeamScratch<R>& ts, int slot, int c, int i,
                                    int exch_i) {
    const R* __restrict__ src = A.src[slot];
    R val = ldg(src + A.L.bare(c) + i);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const Plan<R>& P = ts.plan[slot][ch];
        if (P.kernel) {
            const R* q = src + A.L.qbase(c, P.src_ch, P.kernel - 1);
            R acc = plan_read(P, q, P.exch ? exch_i : i);
            val += (c == 1 ? P.sgn_d : (R)1) * acc;
        }
    }
    return val;
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

template <typename R, int T>
__device__ __forceinline__ double cross_team_sum(double v) {
#pragma unroll
    for (int o = T; o < 32; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

template <int T>
__device__ __forceinline__ double in_team_sum(double v) {
#pragma unroll
    for (int o = 1; o < T; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

template <typename R, int T, int SPL>
struct Warp {
    const PassArgs<R>& A;
    const SMesh<R>& M;
    TeamScratch<R>& ts;
    R* tmp;  // t channel: [2][kC][Ns] slot values of this team's node
    int X;   // channel
    int tl;  // lane in team
    R W, V, VP;
    int nprop;
    unsigned long long nodes;  // integrand evaluations of this team
    unsigned long long alg;    // algorithmic vertex values of these evaluations (lane 0 of the team)

    // Evaluate the integrand at node x for this team's sites: g[c][k] = Γ_c(site tl + k*T).
    // Team-collective; inactive teams take part in the warp syncs only.
    __device__ __noinline__ void eval(double x, bool active, R g[kC][SPL]) {
        const R v = (R)x;
        const int Ns = A.L.Ns;
        const int nslots = (X == 1) ? 4 : 2;
        if (active) ++nodes;
        const int nitems = nprop + 3 * nslots;
        if (active) {
            for (int item = tl; item < nitems; item += T) {
                if (item < nprop) {
                    ts.p_half[item] = prop_half<R>(A.prop_kind, item, X, M, A.L.Nsig, A.prop_a, A.prop_da,
                                                   (R)A.Lam, v, W);
                } else {
                    const int k = item - nprop;
                    const int slot = k / 3, ch = k % 3;
                    Plan<R>& P = ts.plan[slot][ch];
                    if (A.mask[X][slot] & (1 << ch)) {
                        R a0, a1, a2;
                        slot_arg<R>(X, slot, ch, v, W, V, VP, a0, a1, a2);
                        make_plan<R>(P, ch, a0, a1, a2, M, Ns, A.L.NO, A.L.Nn);
                    } else {
                        P.kernel = 0;
                    }
                }
            }
        }
        __syncwarp();
        if (A.node_counter && active && tl == 0) {
            // corner reads of the two site slots on all sites and of the t-channel local
            // slots at one site, bare (2 Ns) and output (Ns) values, t-channel overlap operands
            unsigned long long cs = 0, c1 = 0;
            for (int s = 0; s < nslots; ++s)
                for (int ch = 0; ch < 3; ++ch) (s < 2 ? cs : c1) += corners_of(ts.plan[s][ch].kernel);
            unsigned long long v = cs * Ns + c1 + 3ull * Ns;
            if (X == 1) v += 2ull * ldg(A.ov_off + Ns);
            alg += v * kC;
        }
        R p = (R)0;
        if (active) p = (nprop == 2) ? ts.p_half[0] + ts.p_half[1] : ts.p_half[0];
        if (X != 1) {
            const R two = (X == 0) ? (R)-2 : (R)2;
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                g[0][k] = (R)0;
                g[1][k] = (R)0;
                if (active && i < Ns) {
                    const int ei = ldg(A.exch + i);
                    const R v1s = gather(A, ts, 0, 0, i, ei), v1d = gather(A, ts, 0, 1, i, ei);
                    const R v2s = gather(A, ts, 1, 0, i, ei), v2d = gather(A, ts, 1, 1, i, ei);
                    g[0][k] = -p * (two * v1s * v2s + v1s * v2d + v1d * v2s);
                    g[1][k] = -p * ((R)3 * v1s * v2s + v1d * v2d);
                }
            }
            __syncwarp();
            return;
        }
        // t channel: local vertices at site 1 (flow_su2_t.jl:46-48)
        if (active && tl < 4) {
            const int slot = 2 + (tl >> 1), c = tl & 1;
            ts.loc[tl] = gather(A, ts, slot, c, 0, ldg(A.exch));
        }
        // both slots on all sites into shared memory
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const int i = tl + k * T;
            if (active && i < Ns) {
                const int ei = ldg(A.exch + i);
                tmp[i] = gather(A, ts, 0, 0, i, ei);
                tmp[Ns + i] = gather(A, ts, 0, 1, i, ei);
                tmp[2 * Ns + i] = gather(A, ts, 1, 0, i, ei);
                tmp[3 * Ns + i] = gather(A, ts, 1, 1, i, ei);
            }
        }
        __syncwarp();
        const R v3s = ts.loc[0], v3d = ts.loc[1], v4s = ts.loc[2], v4d = ts.loc[3];
        const R fac = -p * (R)-2;
        const R twoS = (R)A.twoS;
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const int i = tl + k * T;
            g[0][k] = (R)0;
            g[1][k] = (R)0;
            if (active && i < Ns) {
                const R v1s = tmp[i], v1d = tmp[Ns + i], v2s = tmp[2 * Ns + i], v2d = tmp[3 * Ns + i];
                R Gs = -p * ((R)-1 * v1s * v4s + v1s * v4d - (R)1 * v3s * v2s + v3d * v2s);
                R Gd = -p * ((R)3 * v1d * v4s + v1d * v4d + (R)3 * v3s * v2d + v3d * v2d);
                const int j0 = ldg(A.ov_off + i), j1 = ldg(A.ov_off + i + 1);
                for (int j = j0; j < j1; ++j) {
                    const int ab = ldg(A.ov_ab + j);
                    const int ia = ab & 0xffff, ib = ab >> 16;
                    const R mm = fac * ldg(A.ov_m + j) * twoS;
                    Gs += mm * tmp[ia] * tmp[2 * Ns + ib];
                    Gd += mm * tmp[Ns + ia] * tmp[3 * Ns + ib];
                }
                g[0][k] = Gs;
                g[1][k] = Gd;
            }
        }
        __syncwarp();
    }
};

template <typename R, int T, int SPL>
__global__ void __launch_bounds__(kWarps * 32) pass_kernel(PassArgs<R> A) {
    constexpr int NPW = 32 / T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SMesh<R>& M = *reinterpret_cast<SMesh<R>*>(smem_raw);
    TeamScratch<R>* teams = reinterpret_cast<TeamScratch<R>*>(smem_raw + sizeof(SMesh<R>));
    const int Ns = A.L.Ns;
    R* tmp_all = reinterpret_cast<R*>(smem_raw + sizeof(SMesh<R>) + sizeof(TeamScratch<R>) * kWarps * NPW);
    double* red = reinterpret_cast<double*>(tmp_all + (size_t)kWarps * NPW * 4 * Ns);

    load_mesh(M, A.mesh, A.L.Nsig, A.L.NO, A.L.Nn);
    __syncthreads();

    const int X = A.chan_of_y[blockIdx.y];
    const int4 task = A.tasks[blockIdx.x];
    const int kernel = task.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int team = lane / T, tl = lane % T;

    // get_kernel_args (mesh.jl:30-83)
    const R* Om = (X == 1) ? M.Ot : M.Os;
    const R* nu = (X == 1) ? M.nt : M.ns;
    const double* mesh = A.mesh;
    const double* Om64 = mesh + A.L.Nsig + (X == 1 ? A.L.NO + A.L.Nn : 0);
    const double* nu64 = Om64 + A.L.NO;
    const R inf = (R)INFINITY;
    const R W = Om[task.y];
    const R V = (kernel == 2 || kernel == 4) ? nu[task.z] : inf;
    const R VP = (kernel == 3 || kernel == 4) ? nu[task.w] : inf;

    Warp<R, T, SPL> wp{A, M, teams[warp * NPW + team], tmp_all + (size_t)(warp * NPW + team) * 4 * Ns, X, tl, W, V,
                       VP, A.prop_kind == PROP_KAT ? 2 : 1, 0, 0};

    // integration ranges (flow_s.jl:29-38): ref = Λ + w/2, val = Ω[end] + ν[end], computed in FP64
    const double W64 = Om64[task.y];
    const double ref = A.Lam + 0.5 * W64;
    const double val = Om64[A.L.NO - 1] + nu64[A.L.Nn - 1];
    const int eval = A.eval;
    // subdomain end points of integrate_log! (ξ^k a, computed on the host with libm's pow
    // exactly as the reference): an end point at v = ±val sits on the jump of the vertex
    // read-out at Ω[end] + ν[end], so it must round exactly like the reference's
    const double* lb = A.log_bounds + (size_t)((X == 1 ? A.L.NO : 0) + task.y) * (eval + 1);

    double tacc[kC][SPL];
#pragma unroll
    for (int c = 0; c < kC; ++c)
#pragma unroll
        for (int k = 0; k < SPL; ++k) tacc[c][k] = 0.0;

    R g[kC][SPL];
    const int njobs = 4 * eval + 1;
    for (int job = warp; job < njobs; job += kWarps) {
        if (job == 4 * eval) {
            // boundary corrections (flow_s.jl:37-38): two single nodes weighted by corrs
            const double c0 = A.corrs[0 + 2 * (X + 3 * task.y)];
            const double c1 = A.corrs[1 + 2 * (X + 3 * task.y)];
            double bacc[kC][SPL];
#pragma unroll
            for (int c = 0; c < kC; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) bacc[c][k] = 0.0;
            for (int r = 0; r < 2; r += NPW) {
                const int nd = r + team;
                wp.eval(nd == 0 ? -val : val, nd < 2, g);
                if (nd < 2) {
                    const double wgt = nd == 0 ? c0 : c1;
#pragma unroll
                    for (int c = 0; c < kC; ++c)
#pragma unroll
                        for (int k = 0; k < SPL; ++k) bacc[c][k] += wgt * (double)g[c][k];
                }
            }
#pragma unroll
            for (int c = 0; c < kC; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) tacc[c][k] += cross_team_sum<R, T>(bacc[c][k]);
            continue;
        }
        const int range = job / eval, sub = job % eval + 1;
        double lo, hi, sgn = 1.0;
        if (range == 0 || range == 3) {
            const double a = 2.0 * ref, b = 1.0 * val;
            if (!(b > a)) continue;
            lo = lb[sub - 1];
            hi = lb[sub];
            sgn = range == 0 ? -1.0 : 1.0;
        } else {
            // integrate_lin!: a + (i-1) h and a + i h, rounded like the reference (no FMA)
            const double a = range == 1 ? -2.0 * ref : 0.0 * ref;
            const double b = range == 1 ? 0.0 * ref : 2.0 * ref;
            if (!(b > a)) continue;
            const double h = (b - a) / eval;
            lo = __dadd_rn(a, __dmul_rn((double)(sub - 1), h));
            hi = __dadd_rn(a, __dmul_rn((double)sub, h));
        }

        // ---- simps! on [lo, hi] ----
        double s_old[kC][SPL], s_new[kC][SPL], f_prev[kC][SPL];
#pragma unroll
        for (int c = 0; c < kC; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) s_old[c][k] = f_prev[c][k] = 0.0;
        const double mid = 0.5 * (lo + hi);
        const double w_end = 1.0 * (hi - lo) / 6.0, w_mid = 2.0 * (hi - lo) / 3.0;
        for (int r = 0; r < 3; r += NPW) {
            const int nd = r + team;
            const double x = nd == 0 ? lo : (nd == 1 ? mid : hi);
            wp.eval(sgn * x, nd < 3, g);
            if (nd < 3) {
                const double wgt = nd == 1 ? w_mid : w_end;
#pragma unroll
                for (int c = 0; c < kC; ++c)
#pragma unroll
                    for (int k = 0; k < SPL; ++k) {
                        s_old[c][k] += wgt * (double)g[c][k];
                        if (nd == 1) f_prev[c][k] += (double)g[c][k];
                    }
            }
        }
#pragma unroll
        for (int c = 0; c < kC; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                s_old[c][k] = cross_team_sum<R, T>(s_old[c][k]);
                f_prev[c][k] = cross_team_sum<R, T>(f_prev[c][k]);
            }
        long long n = 2;
        while (true) {
            const double h = 0.5 * (hi - lo) / (double)n;
            Acc<R> fn[kC][SPL];
#pragma unroll
            for (int c = 0; c < kC; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) fn[c][k] = Acc<R>{(R)0, (R)0};
            for (long long r = 0; r < n; r += NPW) {
                const long long nd = r + team;
                const double x = __dadd_rn(lo, __dmul_rn(2.0 * (double)(nd + 1) - 1.0, h));
                wp.eval(sgn * x, nd < n, g);
                if (nd < n) {
#pragma unroll
                    for (int c = 0; c < kC; ++c)
#pragma unroll
                        for (int k = 0; k < SPL; ++k) acc_add(fn[c][k], g[c][k]);
                }
            }
            double ss_r = 0.0, ss_n = 0.0, ss_d = 0.0;
            const double wn = 4.0 * h / 3.0, wo = -2.0 * h / 3.0;
#pragma unroll
            for (int c = 0; c < kC; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) {
                    const double fsum = cross_team_sum<R, T>((double)fn[c][k].s + (double)fn[c][k].c);
                    s_new[c][k] = 0.5 * s_old[c][k] + wn * fsum + wo * f_prev[c][k];
                    f_prev[c][k] = fsum;
                    const double rich = s_old[c][k] * (-1.0 / 15.0) + (16.0 / 15.0) * s_new[c][k];
                    const double dd = rich - s_new[c][k];
                    // a team holds a full copy: count each site once
                    if (team == 0) {
                        ss_r += rich * rich;
                        ss_n += s_new[c][k] * s_new[c][k];
                        ss_d += dd * dd;
                    }
                }
            ss_r = in_team_sum<T>(ss_r);
            ss_n = in_team_sum<T>(ss_n);
            ss_d = in_team_sum<T>(ss_d);
            const double adiff = sqrt(ss_d);
            const double rdiff = adiff / fmax(sqrt(ss_r), sqrt(ss_n));
            int done = (adiff < A.atol || rdiff < A.rtol || 2 * n > (1ll << 20)) ? 1 : 0;
            done = __shfl_sync(kFull, done, 0);
            if (done) {
#pragma unroll
                for (int c = 0; c < kC; ++c)
#pragma unroll
                    for (int k = 0; k < SPL; ++k)
                        tacc[c][k] += (s_old[c][k] * (-1.0 / 15.0) + (16.0 / 15.0) * s_new[c][k] - s_new[c][k]) +
                                      s_new[c][k];
                break;
            }
#pragma unroll
            for (int c = 0; c < kC; ++c)
#pragma unroll
                for (int k = 0; k < SPL; ++k) s_old[c][k] = s_new[c][k];
            n *= 2;
        }
    }

    if (A.node_counter && tl == 0 && wp.nodes) {
        atomicAdd(A.node_counter, wp.nodes);
        atomicAdd(A.node_counter + 1, wp.alg);
    }
    // every team holds the full per-site sums: team 0 hands them to the CTA reduction
    if (team == 0) {
#pragma unroll
        for (int c = 0; c < kC; ++c)
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const int i = tl + k * T;
                if (i < Ns) red[(warp * kC + c) * Ns + i] = tacc[c][k];
            }
    }
    __syncthreads();
    // output slice (flow_s.jl:41-51)
    const Layout& L = A.L;
    int64_t off;
    switch (kernel) {
        case 1: off = (int64_t)Ns * task.y; break;
        case 2: off = (int64_t)Ns * (task.y + (int64_t)L.NO * task.z); break;
        case 3: off = (int64_t)Ns * (task.y + (int64_t)L.NO * task.w); break;
        default: off = (int64_t)Ns * (task.y + (int64_t)L.NO * (task.z + (int64_t)L.Nn * task.w)); break;
    }
    for (int e = threadIdx.x; e < kC * Ns; e += blockDim.x) {
        const int c = e / Ns, i = e % Ns;
        double s = 0.0;
        for (int w = 0; w < kWarps; ++w) s += red[(w * kC + c) * Ns + i];
        A.out[L.qbase(c, X, kernel - 1) + off + i] = s;
    }
}

template <typename R, int T, int SPL>
static cudaError_t launch_t(const PassArgs<R>& a, cudaStream_t st) {
    constexpr int NPW = 32 / T;
    const size_t smem = sizeof(SMesh<R>) + sizeof(TeamScratch<R>) * kWarps * NPW +
                        sizeof(R) * (size_t)kWarps * NPW * 4 * a.L.Ns + sizeof(double) * kWarps * kC * a.L.Ns;
    auto kfn = pass_kernel<R, T, SPL>;
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(a.ntasks, a.nchan);
    kfn<<<grid, kWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

// team width T = lanes per node, SPL = sites per lane
template <typename R>
cudaError_t launch_pass_impl(const PassArgs<R>& a, cudaStream_t st) {
    const int Ns = a.L.Ns;
    if (a.ntasks == 0) return cudaSuccess;
    if (Ns <= 8) return launch_t<R, 8, 1>(a, st);
    if (Ns <= 16) return launch_t<R, 16, 1>(a, st);
    if (Ns <= 32) return launch_t<R, 32, 1>(a, st);
    if (Ns <= 64) return launch_t<R, 32, 2>(a, st);
    if (Ns <= 128) return launch_t<R, 32, 4>(a, st);
    if (Ns <= 256) return launch_t<R, 32, 8>(a, st);
    return cudaErrorInvalidValue;
}

}  // namespace pffrg

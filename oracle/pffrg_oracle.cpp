// CPU FP64 restatement of the PFFRGSolver.jl flow right-hand side.
//
// TEST INFRASTRUCTURE ONLY: the parity oracle and the timed CPU baseline.  It
// follows the reference's algorithms step by step (adaptive decisions
// included); every function names the reference file:line it restates.
// Third-party numerics not in the reference tree are restated from their
// published algorithms: QuadGK.jl (compat 2.4, adaptive Gauss-Kronrod 7/15
// with a max-error segment heap and the standard infinite-interval maps).
#include "pffrg_oracle.h"

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <queue>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;

thread_local oracle_stats g_stats;

// ---------------------------------------------------------------------------
// problem view
// ---------------------------------------------------------------------------
struct Dims {
    int Ns, Nsig, NO, Nn, C;
    int64_t K1, K2, K3, chan, comp, total;
};

struct Prob {
    const oracle_problem* p;
    Dims d;
    std::vector<int> exch;           // 0-based
    std::vector<double> mult;
    std::vector<int64_t> ov_off;
    std::vector<int> ov_a, ov_b;     // 0-based
    std::vector<double> ov_m;
    double S;
};

Dims make_dims(const oracle_problem* p) {
    Dims d;
    d.Ns = (int)p->num_sites;
    d.Nsig = (int)p->num_sigma;
    d.NO = (int)p->num_omega;
    d.Nn = (int)p->num_nu;
    d.C = p->symmetry == 0 ? 2 : 6;
    d.K1 = (int64_t)d.Ns * d.NO;
    d.K2 = d.K1 * d.Nn;
    d.K3 = d.K2 * d.Nn;
    d.chan = d.K1 + 2 * d.K2 + d.K3;
    d.comp = d.Ns + 3 * d.chan;
    d.total = d.Nsig + d.C * d.comp;
    return d;
}

Prob make_prob(const oracle_problem* p) {
    Prob P;
    P.p = p;
    P.d = make_dims(p);
    P.S = p->S;
    int Ns = P.d.Ns;
    P.exch.resize(Ns);
    P.mult.resize(Ns);
    for (int i = 0; i < Ns; ++i) {
        P.exch[i] = (int)p->exchange[i] - 1;
        P.mult[i] = (double)p->mult[i];
    }
    P.ov_off.assign(p->overlap_offsets, p->overlap_offsets + Ns + 1);
    int64_t R = P.ov_off[Ns];
    P.ov_a.resize(R);
    P.ov_b.resize(R);
    P.ov_m.resize(R);
    for (int64_t j = 0; j < R; ++j) {
        P.ov_a[j] = (int)p->overlap_rows[3 * j] - 1;
        P.ov_b[j] = (int)p->overlap_rows[3 * j + 1] - 1;
        P.ov_m[j] = (double)p->overlap_rows[3 * j + 2];
    }
    return P;
}

// pointers into a packed action
struct Act {
    const double* sigma;
    const double* bare[6];
    const double* q[6][3][4];  // [comp][channel s,t,u][q1,q2_1,q2_2,q3]
};

Act make_act(const Dims& d, const double* base) {
    Act a;
    a.sigma = base;
    for (int c = 0; c < d.C; ++c) {
        const double* cb = base + d.Nsig + c * d.comp;
        a.bare[c] = cb;
        for (int ch = 0; ch < 3; ++ch) {
            const double* q = cb + d.Ns + ch * d.chan;
            a.q[c][ch][0] = q;
            a.q[c][ch][1] = q + d.K1;
            a.q[c][ch][2] = q + d.K1 + d.K2;
            a.q[c][ch][3] = q + d.K1 + 2 * d.K2;
        }
    }
    return a;
}

// ---------------------------------------------------------------------------
// Param / Buffer (src/Frequency/param.jl, buffer.jl)
// ---------------------------------------------------------------------------
struct Param {
    int lo, hi;
    double wl, wu;
};

// get_indices + get_param (param.jl:26-87), 0-based indices
inline Param get_param(double val, const double* list, int n) {
    Param p;
    if (val >= list[n - 1]) {
        p.lo = p.hi = n - 1;
    } else {
        int k = 0;
        while (val > list[k]) ++k;
        p.hi = k;
        p.lo = (val < list[k]) ? k - 1 : k;
        if (p.lo < 0) p.lo = 0;
    }
    if (p.lo < p.hi) {
        double dd = 1.0 / (list[p.hi] - list[p.lo]);
        p.wl = dd * (list[p.hi] - val);
        p.wu = dd * (val - list[p.lo]);
    } else {
        p.wl = 1.0;
        p.wu = 0.0;
    }
    return p;
}

struct Buf {
    int kernel;
    bool exch, map, sgn_mn, sgn_m, sgn_n;
    Param p1, p2, p3;
};

inline Buf empty_buf() {
    Buf b;
    std::memset(&b, 0, sizeof(b));
    return b;
}

// get_buffer (buffer.jl:51-84)
inline Buf get_buffer(double w, double v, double vp, const double* Om, int nO, const double* nu,
                      int nn, bool exch, bool map, bool smn, bool sm, bool sn) {
    if (Om[nO - 1] < std::fabs(w)) return empty_buf();
    Buf b;
    b.exch = exch;
    b.map = map;
    b.sgn_mn = smn;
    b.sgn_m = sm;
    b.sgn_n = sn;
    b.p1 = get_param(w, Om, nO);
    b.p2 = Param{0, 0, 0.0, 0.0};
    b.p3 = Param{0, 0, 0.0, 0.0};
    if (nu[nn - 1] < std::fabs(v)) {
        if (nu[nn - 1] < std::fabs(vp)) {
            b.kernel = 1;
        } else {
            b.kernel = 3;
            b.p3 = get_param(vp, nu, nn);
        }
    } else {
        if (nu[nn - 1] < std::fabs(vp)) {
            b.kernel = 2;
            b.p2 = get_param(v, nu, nn);
        } else {
            b.kernel = 4;
            b.p2 = get_param(v, nu, nn);
            b.p3 = get_param(vp, nu, nn);
        }
    }
    return b;
}

// get_buffer_s (buffer.jl:87-124)
inline Buf buffer_s(const oracle_problem* m, double w, double v, double vp) {
    bool ex = false, mp = false, smn = false, sm = false, sn = false;
    if (w < 0.0) { w = -w; ex = !ex; }
    if (v < 0.0) { v = -v; ex = !ex; mp = !mp; sm = !sm; }
    if (vp < 0.0) { vp = -vp; mp = !mp; sn = !sn; }
    return get_buffer(w, v, vp, m->omega_s, (int)m->num_omega, m->nu_s, (int)m->num_nu, ex, mp, smn, sm, sn);
}

// get_buffer_t (buffer.jl:126-160)
inline Buf buffer_t(const oracle_problem* m, double w, double v, double vp) {
    bool smn = false, sm = false, sn = false;
    if (w < 0.0) { w = -w; smn = !smn; }
    if (v < 0.0) { v = -v; sm = !sm; }
    if (vp < 0.0) { vp = -vp; sn = !sn; }
    return get_buffer(w, v, vp, m->omega_t, (int)m->num_omega, m->nu_t, (int)m->num_nu, false, false, smn, sm, sn);
}

// get_buffer_u (buffer.jl:162-199); the reference flips sgn_ν (not sgn_μ) for v < 0
inline Buf buffer_u(const oracle_problem* m, double w, double v, double vp) {
    bool ex = false, mp = false, smn = false, sm = false, sn = false;
    if (w < 0.0) { w = -w; ex = !ex; smn = !smn; }
    if (v < 0.0) { v = -v; ex = !ex; mp = !mp; sn = !sn; }
    if (vp < 0.0) { vp = -vp; mp = !mp; sn = !sn; }
    return get_buffer(w, v, vp, m->omega_s, (int)m->num_omega, m->nu_s, (int)m->num_nu, ex, mp, smn, sm, sn);
}

// ---------------------------------------------------------------------------
// self energy and propagators (Action.jl:8-26, bubbles.jl:2-96)
// ---------------------------------------------------------------------------
inline double jl_sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : x); }

inline double get_sigma(const oracle_problem* m, const double* Sig, double w) {
    int n = (int)m->num_sigma;
    if (std::fabs(w) <= m->sigma[n - 1]) {
        Param p = get_param(std::fabs(w), m->sigma, n);
        return jl_sign(w) * (p.wl * Sig[p.lo] + p.wu * Sig[p.hi]);
    }
    return m->sigma[n - 1] * Sig[n - 1] / w;
}

inline double G_bare(double L, double w) {
    if (std::fabs(w) > 1e-8) return -std::expm1(-(w * w) / (L * L)) / w;
    return 0.0;
}

inline double G_full(const oracle_problem* m, const double* Sig, double L, double w) {
    if (std::fabs(w) > 1e-8) {
        double s = get_sigma(m, Sig, w);
        double g0 = G_bare(L, w);
        double den = (w * s >= 0.0) ? 1.0 / g0 + s : 1.0 / g0;
        return 1.0 / den;
    }
    return 0.0;
}

inline double S_single(const oracle_problem* m, const double* Sig, double L, double w) {
    if (std::fabs(w) > 1e-8) {
        double g = G_full(m, Sig, L, w);
        double g0 = G_bare(L, w);
        double r = g / g0;
        return r * r * std::exp(-(w * w) / (L * L)) * 2.0 * w / (L * L * L);
    }
    return 0.0;
}

inline double prop_kat(const oracle_problem* m, const double* Sig, const double* dSig, double L,
                       double w1, double w2) {
    double ds = get_sigma(m, dSig, w1);
    double s1 = S_single(m, Sig, L, w1);
    double g1 = G_full(m, Sig, L, w1);
    double g2 = G_full(m, Sig, L, w2);
    return (s1 + g1 * g1 * ds) * g2 / (2.0 * kPi);
}

inline double prop_plain(const oracle_problem* m, const double* Sig, double L, double w1, double w2) {
    double g1 = G_full(m, Sig, L, w1);
    double g2 = G_full(m, Sig, L, w2);
    return g1 * g2 / (2.0 * kPi);
}

// ---------------------------------------------------------------------------
// vertex interpolation (channel.jl:55-305, vertex.jl:63-82, Action.jl:110-167)
// ---------------------------------------------------------------------------
// add sgn * interp(q_kernel) for all sites (or site 0 only) into temp[Ns]
inline void interp_add(const Prob& P, const double* const* q, const Buf& b, double sgn,
                       double* temp, int nsites) {
    const Dims& d = P.d;
    const int Ns = d.Ns, NO = d.NO, Nn = d.Nn;
    const bool ex = b.exch;
    switch (b.kernel) {
        case 1: {
            const double* Q = q[0];
            const int64_t ol = (int64_t)Ns * b.p1.lo, ou = (int64_t)Ns * b.p1.hi;
            for (int i = 0; i < nsites; ++i) {
                int s = ex ? P.exch[i] : i;
                double val = b.p1.wl * Q[s + ol];
                val += b.p1.wu * Q[s + ou];
                temp[i] += sgn * val;
            }
            g_stats.gathered_values += 2 * nsites;
            break;
        }
        case 2:
        case 3: {
            const double* Q = (b.kernel == 2) ? q[1] : q[2];
            const Param& pa = b.p1;
            const Param& pb = (b.kernel == 2) ? b.p2 : b.p3;
            auto idx = [&](int w, int v) { return (int64_t)Ns * (w + (int64_t)NO * v); };
            const int64_t o00 = idx(pa.lo, pb.lo), o10 = idx(pa.hi, pb.lo), o01 = idx(pa.lo, pb.hi),
                          o11 = idx(pa.hi, pb.hi);
            for (int i = 0; i < nsites; ++i) {
                int s = ex ? P.exch[i] : i;
                double val = pa.wl * pb.wl * Q[s + o00];
                val += pa.wu * pb.wl * Q[s + o10];
                val += pa.wl * pb.wu * Q[s + o01];
                val += pa.wu * pb.wu * Q[s + o11];
                temp[i] += sgn * val;
            }
            g_stats.gathered_values += 4 * nsites;
            break;
        }
        case 4: {
            const double* Q = q[3];
            const Param &p1 = b.p1, &p2 = b.p2, &p3 = b.p3;
            auto idx = [&](int w, int v, int vp) {
                return (int64_t)Ns * (w + (int64_t)NO * (v + (int64_t)Nn * vp));
            };
            const int64_t o000 = idx(p1.lo, p2.lo, p3.lo), o100 = idx(p1.hi, p2.lo, p3.lo),
                          o010 = idx(p1.lo, p2.hi, p3.lo), o110 = idx(p1.hi, p2.hi, p3.lo),
                          o001 = idx(p1.lo, p2.lo, p3.hi), o101 = idx(p1.hi, p2.lo, p3.hi),
                          o011 = idx(p1.lo, p2.hi, p3.hi), o111 = idx(p1.hi, p2.hi, p3.hi);
            for (int i = 0; i < nsites; ++i) {
                int s = ex ? P.exch[i] : i;
                double val = p1.wl * p2.wl * p3.wl * Q[s + o000];
                val += p1.wu * p2.wl * p3.wl * Q[s + o100];
                val += p1.wl * p2.wu * p3.wl * Q[s + o010];
                val += p1.wu * p2.wu * p3.wl * Q[s + o110];
                val += p1.wl * p2.wl * p3.wu * Q[s + o001];
                val += p1.wu * p2.wl * p3.wu * Q[s + o101];
                val += p1.wl * p2.wu * p3.wu * Q[s + o011];
                val += p1.wu * p2.wu * p3.wu * Q[s + o111];
                temp[i] += sgn * val;
            }
            g_stats.gathered_values += 8 * nsites;
            break;
        }
        default:
            break;
    }
}

// apply_flags_su2 (action_su2.jl:73-92): sign only, component unchanged
inline double flags_su2(const Buf& b, int comp) {
    double sgn = 1.0;
    if (comp == 1 && b.sgn_m) sgn = -sgn;
    if (comp == 1 && b.sgn_n) sgn = -sgn;
    return sgn;
}

// apply_flags_u1_dm (action_u1_dm.jl:80-118), 0-based components xx, zz, DM, dd, zd, dz:
// the sign of the contribution and the component actually read
inline double flags_u1dm(const Buf& b, int comp, int& src) {
    double sgn = 1.0;
    if ((comp == 4 || comp == 5) && b.sgn_mn) sgn = -sgn;
    if ((comp == 3 || comp == 5) && b.sgn_m) sgn = -sgn;
    if ((comp == 3 || comp == 4) && b.sgn_n) sgn = -sgn;
    src = comp;
    if (b.exch) {
        if (comp == 2) sgn = -sgn;
        else if (comp == 4) src = 5;
        else if (comp == 5) src = 4;
    }
    return sgn;
}

inline double apply_flags(const Prob& P, const Buf& b, int comp, int& src) {
    if (P.p->symmetry == 0) {
        src = comp;
        return flags_su2(b, comp);
    }
    return flags_u1dm(b, comp, src);
}

enum { CH_S = 1, CH_T = 2, CH_U = 4 };

// get_Γ_comp_avx! for every component (action_su2.jl:115-134); temp[c*Ns + i]
inline void gather_slot(const Prob& P, const Act& A, const Buf& bs, const Buf& bt, const Buf& bu,
                        int mask, double* temp, int nsites) {
    const Dims& d = P.d;
    for (int c = 0; c < d.C; ++c) {
        double* t = temp + (int64_t)c * d.Ns;
        for (int i = 0; i < nsites; ++i) t[i] = A.bare[c][i];
        int src;
        if (mask & CH_S) {
            double sg = apply_flags(P, bs, c, src);
            interp_add(P, A.q[src][bs.map ? 2 : 0], bs, sg, t, nsites);
        }
        if (mask & CH_T) {
            double sg = apply_flags(P, bt, c, src);
            interp_add(P, A.q[src][1], bt, sg, t, nsites);
        }
        if (mask & CH_U) {
            double sg = apply_flags(P, bu, c, src);
            interp_add(P, A.q[src][bu.map ? 0 : 2], bu, sg, t, nsites);
        }
    }
}

// sequential get_Γ_comp for one component at one site (Action.jl:29-107)
inline double gamma_comp_site(const Prob& P, const Act& A, int comp, int site, const Buf& bs,
                              const Buf& bt, const Buf& bu, int mask) {
    // reuse the vectorised path on a single site by building the value directly
    const Dims& d = P.d;
    double val = A.bare[comp][site];
    auto one = [&](const double* const* q, const Buf& b, double sg) {
        int s = b.exch ? P.exch[site] : site;
        const int Ns = d.Ns, NO = d.NO, Nn = d.Nn;
        double v = 0.0;
        switch (b.kernel) {
            case 1:
                v = b.p1.wl * q[0][s + (int64_t)Ns * b.p1.lo];
                v += b.p1.wu * q[0][s + (int64_t)Ns * b.p1.hi];
                g_stats.gathered_values += 2;
                break;
            case 2:
            case 3: {
                const double* Q = (b.kernel == 2) ? q[1] : q[2];
                const Param& pa = b.p1;
                const Param& pb = (b.kernel == 2) ? b.p2 : b.p3;
                auto ix = [&](int w, int vv) { return s + (int64_t)Ns * (w + (int64_t)NO * vv); };
                v = pa.wl * pb.wl * Q[ix(pa.lo, pb.lo)];
                v += pa.wu * pb.wl * Q[ix(pa.hi, pb.lo)];
                v += pa.wl * pb.wu * Q[ix(pa.lo, pb.hi)];
                v += pa.wu * pb.wu * Q[ix(pa.hi, pb.hi)];
                g_stats.gathered_values += 4;
                break;
            }
            case 4: {
                const Param &p1 = b.p1, &p2 = b.p2, &p3 = b.p3;
                auto ix = [&](int w, int vv, int vp) {
                    return s + (int64_t)Ns * (w + (int64_t)NO * (vv + (int64_t)Nn * vp));
                };
                const double* Q = q[3];
                v = p1.wl * p2.wl * p3.wl * Q[ix(p1.lo, p2.lo, p3.lo)];
                v += p1.wu * p2.wl * p3.wl * Q[ix(p1.hi, p2.lo, p3.lo)];
                v += p1.wl * p2.wu * p3.wl * Q[ix(p1.lo, p2.hi, p3.lo)];
                v += p1.wu * p2.wu * p3.wl * Q[ix(p1.hi, p2.hi, p3.lo)];
                v += p1.wl * p2.wl * p3.wu * Q[ix(p1.lo, p2.lo, p3.hi)];
                v += p1.wu * p2.wl * p3.wu * Q[ix(p1.hi, p2.lo, p3.hi)];
                v += p1.wl * p2.wu * p3.wu * Q[ix(p1.lo, p2.hi, p3.hi)];
                v += p1.wu * p2.wu * p3.wu * Q[ix(p1.hi, p2.hi, p3.hi)];
                g_stats.gathered_values += 8;
                break;
            }
            default:
                break;
        }
        return sg * v;
    };
    int src;
    if (mask & CH_S) {
        const double sg = apply_flags(P, bs, comp, src);
        val += one(A.q[src][bs.map ? 2 : 0], bs, sg);
    }
    if (mask & CH_T) {
        const double sg = apply_flags(P, bt, comp, src);
        val += one(A.q[src][1], bt, sg);
    }
    if (mask & CH_U) {
        const double sg = apply_flags(P, bu, comp, src);
        val += one(A.q[src][bu.map ? 0 : 2], bu, sg);
    }
    return val;
}

// ---------------------------------------------------------------------------
// bubble integrands (flow_su2_{s,t,u}.jl, BSE_su2_*.jl, SDE_su2.jl:2-42)
// ---------------------------------------------------------------------------
enum PropKind { PROP_KAT = 0, PROP_PLAIN = 1 };

struct PassDesc {
    int ch;  // 0 s, 1 t, 2 u
    PropKind prop;
    const double* A[4];  // slot sources (packed actions)
    int mask[4];
    const double* a;   // propagator action
    const double* da;  // Katanin dΣ source
    bool reduced = false;  // reduced s bubble of the SDE: u1-dm writes xx, zz, dd only (SDE_u1_dm.jl:2-56)
};

struct Ctx {
    const Prob* P;
    const PassDesc* pd;
    Act A[4];
    double Lam;
    double W, V, VP;  // task frequencies
    std::vector<double>* temp;  // [2][C*Ns]
};

// the 12 buffer argument triples of a node (per channel, per slot)
struct Args3 {
    double w, v, vp;
};

inline void slot_args(int ch, double v, double W, double V, double VP, Args3 out[4][3]) {
    if (ch == 0) {  // s channel (flow_su2_s.jl:21-28)
        const double s = W, vs = V, vsp = VP;
        out[0][0] = {s, vs, -v};
        out[0][1] = {v - vs, 0.5 * (s + v + vs), 0.5 * (s - v - vs)};
        out[0][2] = {v + vs, 0.5 * (s - v + vs), 0.5 * (s + v - vs)};
        out[1][0] = {s, v, vsp};
        out[1][1] = {-v - vsp, 0.5 * (s + v - vsp), 0.5 * (s - v + vsp)};
        out[1][2] = {v - vsp, 0.5 * (s + v + vsp), 0.5 * (s - v - vsp)};
    } else if (ch == 1) {  // t channel (flow_su2_t.jl:21-43)
        const double t = W, vt = V, vtp = VP;
        out[0][0] = {v + vt, 0.5 * (-t - v + vt), 0.5 * (-t + v - vt)};
        out[0][1] = {t, vt, v};
        out[0][2] = {-v + vt, 0.5 * (-t + v + vt), 0.5 * (t + v + vt)};
        out[1][0] = {v + vtp, 0.5 * (-t + v - vtp), 0.5 * (-t - v + vtp)};
        out[1][1] = {t, v, vtp};
        out[1][2] = {v - vtp, 0.5 * (-t + v + vtp), 0.5 * (t + v + vtp)};
        out[2][0] = {v + vt, 0.5 * (t + v - vt), 0.5 * (-t + v - vt)};
        out[2][1] = {-v + vt, 0.5 * (t + v + vt), 0.5 * (-t + v + vt)};
        out[2][2] = {t, v, vt};
        out[3][0] = {v + vtp, 0.5 * (t - v + vtp), 0.5 * (-t - v + vtp)};
        out[3][1] = {v - vtp, 0.5 * (t + v + vtp), 0.5 * (-t + v + vtp)};
        out[3][2] = {t, vtp, v};
    } else {  // u channel (flow_su2_u.jl:21-28)
        const double u = W, vu = V, vup = VP;
        out[0][0] = {v + vu, 0.5 * (u - v + vu), 0.5 * (-u - v + vu)};
        out[0][1] = {v - vu, 0.5 * (u + v + vu), 0.5 * (-u + v + vu)};
        out[0][2] = {u, vu, v};
        out[1][0] = {v + vup, 0.5 * (u + v - vup), 0.5 * (-u + v - vup)};
        out[1][1] = {-v + vup, 0.5 * (u + v + vup), 0.5 * (-u + v + vup)};
        out[1][2] = {u, v, vup};
    }
}

inline double node_prop(const Prob& P, const PassDesc& pd, double L, double v, double W) {
    const oracle_problem* m = P.p;
    const double* Sig = pd.a;  // packed action starts with Σ
    if (pd.prop == PROP_KAT) {
        const double* dSig = pd.da;
        if (pd.ch == 0)
            return prop_kat(m, Sig, dSig, L, v + 0.5 * W, 0.5 * W - v) + prop_kat(m, Sig, dSig, L, 0.5 * W - v, v + 0.5 * W);
        if (pd.ch == 1)
            return prop_kat(m, Sig, dSig, L, v + 0.5 * W, v - 0.5 * W) + prop_kat(m, Sig, dSig, L, v - 0.5 * W, v + 0.5 * W);
        return prop_kat(m, Sig, dSig, L, v - 0.5 * W, v + 0.5 * W) + prop_kat(m, Sig, dSig, L, v + 0.5 * W, v - 0.5 * W);
    }
    if (pd.ch == 0) return -prop_plain(m, Sig, L, v + 0.5 * W, 0.5 * W - v);
    if (pd.ch == 1) return -prop_plain(m, Sig, L, v + 0.5 * W, v - 0.5 * W);
    return -prop_plain(m, Sig, L, v - 0.5 * W, v + 0.5 * W);
}

// u1-dm vertex components at one site, in the reference's order xx, zz, DM, dd, zd, dz
struct V6 {
    double xx, zz, dm, dd, zd, dz;
};

inline V6 v6_at(const double* t, int Ns, int i) {
    return V6{t[i], t[Ns + i], t[2 * Ns + i], t[3 * Ns + i], t[4 * Ns + i], t[5 * Ns + i]};
}

// s-channel bubble of two u1-dm vertices (flow_u1_dm_s.jl:53-58, the same in the left, central,
// BSE and reduced kernels)
inline void comb_s_u1dm(const V6& a, const V6& b, double g[6]) {
    g[0] = a.dm * b.dz - a.dm * b.zd + a.xx * b.dd + a.dd * b.xx - a.xx * b.zz - a.dz * b.dm + a.zd * b.dm - a.zz * b.xx;
    g[1] = a.zz * b.dd + a.dd * b.zz - a.dz * b.zd - 2.0 * a.xx * b.xx - 2.0 * a.dm * b.dm - a.zd * b.dz;
    g[2] = a.dd * b.dm + a.dm * b.dd - a.zd * b.xx - a.xx * b.dz - a.zz * b.dm + a.xx * b.zd - a.dm * b.zz + a.dz * b.xx;
    g[3] = -a.dz * b.dz + 2.0 * a.xx * b.xx + a.dd * b.dd + 2.0 * a.dm * b.dm - a.zd * b.zd + a.zz * b.zz;
    g[4] = a.zd * b.dd + a.dd * b.zd - 2.0 * a.dm * b.xx + a.dz * b.zz + a.zz * b.dz + 2.0 * a.xx * b.dm;
    g[5] = a.zd * b.zz + a.dd * b.dz + a.zz * b.zd + 2.0 * a.dm * b.xx + a.dz * b.dd - 2.0 * a.xx * b.dm;
}

// u-channel bubble (flow_u1_dm_u.jl:52-57)
inline void comb_u_u1dm(const V6& a, const V6& b, double g[6]) {
    g[0] = -a.dm * b.dz - a.dm * b.zd + a.xx * b.dd + a.dd * b.xx + a.xx * b.zz + a.dz * b.dm + a.zd * b.dm + a.zz * b.xx;
    g[1] = a.zz * b.dd + a.dd * b.zz - a.dz * b.zd + 2.0 * a.xx * b.xx + 2.0 * a.dm * b.dm - a.zd * b.dz;
    g[2] = a.dd * b.dm + a.dm * b.dd - a.zd * b.xx + a.xx * b.dz + a.zz * b.dm + a.xx * b.zd + a.dm * b.zz - a.dz * b.xx;
    g[3] = -a.dz * b.dz + 2.0 * a.xx * b.xx + a.dd * b.dd + 2.0 * a.dm * b.dm - a.zd * b.zd + a.zz * b.zz;
    g[4] = a.zd * b.dd + a.dd * b.zd - 2.0 * a.dm * b.xx + a.dz * b.zz + a.zz * b.dz + 2.0 * a.xx * b.dm;
    g[5] = a.zd * b.zz + a.dd * b.dz + a.zz * b.zd - 2.0 * a.dm * b.xx + a.dz * b.dd + 2.0 * a.xx * b.dm;
}

// t-channel local part: non-local vertices v1 (left), v2 (right) at site i with the local
// vertices v3 (left), v4 (right) at site 1 (flow_u1_dm_t.jl:68-84)
inline void comb_t_u1dm(const V6& v1, const V6& v2, const V6& v3, const V6& v4, double g[6]) {
    g[0] = v1.dm * v4.dz - v1.dm * v4.zd + v1.xx * v4.dd - v1.xx * v4.zz + v3.dd * v2.xx + v3.dz * v2.dm -
           v3.zd * v2.dm - v3.zz * v2.xx;
    g[1] = v1.zz * v4.dd + 2.0 * v1.zd * v4.dm - v1.zd * v4.zd + v1.zz * v4.zz - 2.0 * v1.zz * v4.xx - v1.zd * v4.dz -
           2.0 * v3.dm * v2.dz - v3.dz * v2.dz + v3.dd * v2.zz - 2.0 * v3.xx * v2.zz + v3.zz * v2.zz - v3.zd * v2.dz;
    g[2] = v1.dm * v4.dd - v1.xx * v4.dz + v1.xx * v4.zd - v1.dm * v4.zz - v3.dz * v2.xx + v3.dd * v2.dm +
           v3.zd * v2.xx - v3.zz * v2.dm;
    g[3] = -v1.dz * v4.dz + 2.0 * v1.dd * v4.xx + v1.dd * v4.zz - v1.dz * v4.zd - 2.0 * v1.dz * v4.dm + v1.dd * v4.dd +
           2.0 * v3.dm * v2.zd + 2.0 * v3.xx * v2.dd + v3.zz * v2.dd - v3.dz * v2.zd + v3.dd * v2.dd - v3.zd * v2.zd;
    g[4] = v1.zd * v4.zz + v1.zd * v4.dd + 2.0 * v1.zd * v4.xx + v1.zz * v4.zd + 2.0 * v1.zz * v4.dm + v1.zz * v4.dz +
           v3.zd * v2.dd + 2.0 * v3.dm * v2.dd + v3.dd * v2.zd + v3.zz * v2.zd - 2.0 * v3.xx * v2.zd + v3.dz * v2.dd;
    g[5] = -2.0 * v1.dd * v4.dm + v1.dd * v4.zd + v1.dd * v4.dz + v1.dz * v4.zz + v1.dz * v4.dd - 2.0 * v1.dz * v4.xx +
           v3.zd * v2.zz + 2.0 * v3.xx * v2.dz + v3.dd * v2.dz + v3.dz * v2.zz - 2.0 * v3.dm * v2.zz + v3.zz * v2.dz;
}

// t-channel overlap term of one (a, b) row (flow_u1_dm_t.jl:104-109), without the factor -p (-2) m
inline void comb_t_overlap_u1dm(const V6& v1, const V6& v2, double g[6]) {
    g[0] = v1.xx * v2.xx - v1.dm * v2.dm;
    g[1] = v1.zz * v2.zz - v1.zd * v2.dz;
    g[2] = v1.dm * v2.xx + v1.xx * v2.dm;
    g[3] = v1.dd * v2.dd - v1.dz * v2.zd;
    g[4] = v1.zd * v2.dd + v1.zz * v2.zd;
    g[5] = v1.dd * v2.dz + v1.dz * v2.zz;
}

struct Args3;
void integrand_u1dm(const Ctx& cx, double p, const Args3 ar[4][3], const double* t1, const double* t2, double* buff,
                    double dv);

// buff layout: buff[c*Ns + i]; adds dv * Γ(v) for all sites
void integrand(const Ctx& cx, double* buff, double v, double dv) {
    const Prob& P = *cx.P;
    const PassDesc& pd = *cx.pd;
    const Dims& d = P.d;
    const oracle_problem* m = P.p;
    const int Ns = d.Ns;
    g_stats.integrand_evals += 1;

    const double p = node_prop(P, pd, cx.Lam, v, cx.W);
    Args3 ar[4][3];
    slot_args(pd.ch, v, cx.W, cx.V, cx.VP, ar);
    double* t1 = cx.temp->data();
    double* t2 = t1 + (int64_t)d.C * Ns;
    for (int slot = 0; slot < 2; ++slot) {
        Buf bs = buffer_s(m, ar[slot][0].w, ar[slot][0].v, ar[slot][0].vp);
        Buf bt = buffer_t(m, ar[slot][1].w, ar[slot][1].v, ar[slot][1].vp);
        Buf bu = buffer_u(m, ar[slot][2].w, ar[slot][2].v, ar[slot][2].vp);
        gather_slot(P, cx.A[slot], bs, bt, bu, pd.mask[slot], slot == 0 ? t1 : t2, Ns);
    }
    if (P.p->symmetry == 1) {
        integrand_u1dm(cx, p, ar, t1, t2, buff, dv);
        return;
    }
    if (pd.ch == 0 || pd.ch == 2) {
        const double two = (pd.ch == 0) ? -2.0 : 2.0;
        for (int i = 0; i < Ns; ++i) {
            double v1s = t1[i], v1d = t1[Ns + i];
            double v2s = t2[i], v2d = t2[Ns + i];
            double Gs = -p * (two * v1s * v2s + v1s * v2d + v1d * v2s);
            double Gd = -p * (3.0 * v1s * v2s + v1d * v2d);
            buff[i] += dv * Gs;
            buff[Ns + i] += dv * Gd;
        }
        return;
    }
    // t channel: local vertices at site 1 (flow_su2_t.jl:46-48)
    double v3[2], v4[2];
    for (int slot = 2; slot < 4; ++slot) {
        Buf bs = buffer_s(m, ar[slot][0].w, ar[slot][0].v, ar[slot][0].vp);
        Buf bt = buffer_t(m, ar[slot][1].w, ar[slot][1].v, ar[slot][1].vp);
        Buf bu = buffer_u(m, ar[slot][2].w, ar[slot][2].v, ar[slot][2].vp);
        double* vv = (slot == 2) ? v3 : v4;
        for (int c = 0; c < 2; ++c) vv[c] = gamma_comp_site(P, cx.A[slot], c, 0, bs, bt, bu, pd.mask[slot]);
    }
    const double v3s = v3[0], v3d = v3[1], v4s = v4[0], v4d = v4[1];
    const double fac = -p * (-2.0);
    for (int i = 0; i < Ns; ++i) {
        double v1s = t1[i], v1d = t1[Ns + i];
        double v2s = t2[i], v2d = t2[Ns + i];
        double Gs = -p * (-1.0 * v1s * v4s + v1s * v4d - 1.0 * v3s * v2s + v3d * v2s);
        double Gd = -p * (3.0 * v1d * v4s + v1d * v4d + 3.0 * v3s * v2d + v3d * v2d);
        for (int64_t j = P.ov_off[i]; j < P.ov_off[i + 1]; ++j) {
            const int ia = P.ov_a[j], ib = P.ov_b[j];
            const double mm = fac * P.ov_m[j] * (2.0 * P.S);
            Gs += mm * t1[ia] * t2[ib];
            Gd += mm * t1[Ns + ia] * t2[Ns + ib];
        }
        g_stats.overlap_terms += P.ov_off[i + 1] - P.ov_off[i];
        buff[i] += dv * Gs;
        buff[Ns + i] += dv * Gd;
    }
}

// the u1-dm bubbles (flow_u1_dm_{s,t,u}.jl, BSE_u1_dm_*.jl, SDE_u1_dm.jl:2-56)
void integrand_u1dm(const Ctx& cx, double p, const Args3 ar[4][3], const double* t1, const double* t2, double* buff,
                    double dv) {
    const Prob& P = *cx.P;
    const PassDesc& pd = *cx.pd;
    const oracle_problem* m = P.p;
    const int Ns = P.d.Ns;
    double g[6];
    if (pd.ch == 0 || pd.ch == 2) {
        for (int i = 0; i < Ns; ++i) {
            const V6 a = v6_at(t1, Ns, i), b = v6_at(t2, Ns, i);
            if (pd.ch == 0) comb_s_u1dm(a, b, g);
            else comb_u_u1dm(a, b, g);
            for (int c = 0; c < 6; ++c) {
                if (pd.reduced && (c == 2 || c == 4 || c == 5)) continue;
                buff[c * Ns + i] += dv * (-p * g[c]);
            }
        }
        return;
    }
    double v34[2][6];
    for (int slot = 2; slot < 4; ++slot) {
        Buf bs = buffer_s(m, ar[slot][0].w, ar[slot][0].v, ar[slot][0].vp);
        Buf bt = buffer_t(m, ar[slot][1].w, ar[slot][1].v, ar[slot][1].vp);
        Buf bu = buffer_u(m, ar[slot][2].w, ar[slot][2].v, ar[slot][2].vp);
        for (int c = 0; c < 6; ++c) v34[slot - 2][c] = gamma_comp_site(P, cx.A[slot], c, 0, bs, bt, bu, pd.mask[slot]);
    }
    const V6 v3{v34[0][0], v34[0][1], v34[0][2], v34[0][3], v34[0][4], v34[0][5]};
    const V6 v4{v34[1][0], v34[1][1], v34[1][2], v34[1][3], v34[1][4], v34[1][5]};
    for (int i = 0; i < Ns; ++i) {
        const V6 v1 = v6_at(t1, Ns, i), v2 = v6_at(t2, Ns, i);
        comb_t_u1dm(v1, v2, v3, v4, g);
        double G[6];
        for (int c = 0; c < 6; ++c) G[c] = -p * g[c];
        for (int64_t j = P.ov_off[i]; j < P.ov_off[i + 1]; ++j) {
            const V6 a = v6_at(t1, Ns, P.ov_a[j]), b = v6_at(t2, Ns, P.ov_b[j]);
            double h[6];
            comb_t_overlap_u1dm(a, b, h);
            const double mm = -p * (-2.0) * P.ov_m[j];
            for (int c = 0; c < 6; ++c) G[c] += mm * h[c];
        }
        g_stats.overlap_terms += P.ov_off[i + 1] - P.ov_off[i];
        for (int c = 0; c < 6; ++c) buff[c * Ns + i] += dv * G[c];
    }
}

// ---------------------------------------------------------------------------
// adaptive Simpson (quadrature.jl:2-139)
// ---------------------------------------------------------------------------
inline double nrm2(const double* x, int n) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += x[i] * x[i];
    return std::sqrt(s);
}

template <class F>
void residual(F& f, double* buff, double a, double b, int64_t n) {
    const double h = 0.5 * (b - a) / (double)n;
    for (int64_t i = 1; i <= n; ++i) f(buff, a + (2.0 * (double)i - 1.0) * h, +4.0 * h / 3.0);
    for (int64_t i = 1; i <= n / 2; ++i) f(buff, a + (4.0 * (double)i - 2.0) * h, -2.0 * h / 3.0);
    g_stats.reevals += n / 2;
}

template <class F>
void simps(F& f, double* b1, double* b2, int len, double a, double b, double atol, double rtol) {
    std::fill(b1, b1 + len, 0.0);
    const double mid = 0.5 * (a + b);
    f(b1, a, 1.0 * (b - a) / 6.0);
    f(b1, mid, 2.0 * (b - a) / 3.0);
    f(b1, b, 1.0 * (b - a) / 6.0);
    for (int i = 0; i < len; ++i) b2[i] = 0.5 * b1[i];
    residual(f, b2, a, b, 2);
    int64_t n = 4;
    const double c1 = -1.0 / 15.0, c2 = 16.0 / 15.0;
    while (true) {
        for (int i = 0; i < len; ++i) b1[i] *= c1;
        for (int i = 0; i < len; ++i) b1[i] += c2 * b2[i];
        double n1 = nrm2(b1, len), n2 = nrm2(b2, len);
        for (int i = 0; i < len; ++i) b1[i] -= b2[i];
        double adiff = nrm2(b1, len);
        double rdiff = adiff / std::max(n1, n2);
        if (adiff < atol || rdiff < rtol || n > (int64_t(1) << 20)) {
            for (int i = 0; i < len; ++i) b1[i] += b2[i];
            int lv = 0;
            while ((int64_t(2) << lv) < n) ++lv;
            g_stats.level_hist[lv < 23 ? lv : 23] += 1;
            break;
        }
        for (int i = 0; i < len; ++i) b1[i] = b2[i];
        for (int i = 0; i < len; ++i) b2[i] = 0.5 * b1[i];
        residual(f, b2, a, b, n);
        n *= 2;
    }
}

template <class F>
void integrate_lin(F& f, double* tb1, double* tb2, double* tb3, int len, double a, double b, int eval,
                   double atol, double rtol) {
    if (b > a) {
        const double h = (b - a) / eval;
        for (int i = 1; i <= eval; ++i) {
            simps(f, tb2, tb3, len, a + (i - 1) * h, a + i * h, atol, rtol);
            for (int k = 0; k < len; ++k) tb1[k] += tb2[k];
        }
    }
}

template <class F>
void integrate_log(F& f, double* tb1, double* tb2, double* tb3, int len, double a, double b, int eval,
                   double atol, double rtol, double sgn) {
    if (b > a) {
        const double xi = std::pow(b / a, 1.0 / eval);
        auto g = [&](double* bb, double x, double dx) { f(bb, sgn * x, dx); };
        for (int i = 1; i <= eval; ++i) {
            simps(g, tb2, tb3, len, std::pow(xi, (double)(i - 1)) * a, std::pow(xi, (double)i) * a, atol, rtol);
            for (int k = 0; k < len; ++k) tb1[k] += tb2[k];
        }
    }
}

// ---------------------------------------------------------------------------
// QuadGK-equivalent adaptive Gauss-Kronrod (G7/K15)
// ---------------------------------------------------------------------------
const double kGKx[8] = {-0.991455371120812639206854697526329, -0.949107912342758524526189684047851,
                        -0.864864423359769072789712788640926, -0.741531185599394439863864773280788,
                        -0.586087235467691130294144845693013, -0.405845151377397166906606412076961,
                        -0.207784955007898467600689403773245, 0.0};
const double kGKw[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                        0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                        0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                        0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
const double kGw[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                       0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

struct Seg {
    double a, b, I, E;
    bool operator<(const Seg& o) const { return E < o.E; }
};

template <class F>
Seg evalrule(F& f, double a, double b) {
    const double s = 0.5 * (b - a);
    double fg = f(a + (1 + kGKx[1]) * s) + f(a + (1 - kGKx[1]) * s);
    double fk = f(a + (1 + kGKx[0]) * s) + f(a + (1 - kGKx[0]) * s);
    double Ig = fg * kGw[0];
    double Ik = fg * kGKw[1] + fk * kGKw[0];
    for (int i = 2; i <= 3; ++i) {
        fg = f(a + (1 + kGKx[2 * i - 1]) * s) + f(a + (1 - kGKx[2 * i - 1]) * s);
        fk = f(a + (1 + kGKx[2 * i - 2]) * s) + f(a + (1 - kGKx[2 * i - 2]) * s);
        Ig += fg * kGw[i - 1];
        Ik += fg * kGKw[2 * i - 1] + fk * kGKw[2 * i - 2];
    }
    double f0 = f(a + s);
    Ig += f0 * kGw[3];
    Ik += f0 * kGKw[7] + (f(a + (1 + kGKx[6]) * s) + f(a + (1 - kGKx[6]) * s)) * kGKw[6];
    double Iks = Ik * s, Igs = Ig * s;
    return Seg{a, b, Iks, std::fabs(Iks - Igs)};
}

template <class F>
double do_quadgk(F& f, const std::vector<double>& s, double atol, double rtol) {
    const int64_t maxevals = 10000000;
    std::vector<Seg> segs;
    for (size_t i = 0; i + 1 < s.size(); ++i) segs.push_back(evalrule(f, s[i], s[i + 1]));
    double I = segs[0].I, E = segs[0].E;
    for (size_t i = 1; i < segs.size(); ++i) {
        I += segs[i].I;
        E += segs[i].E;
    }
    int64_t numevals = 15 * (int64_t)segs.size();
    if (E <= atol || E <= rtol * std::fabs(I) || numevals >= maxevals) return I;
    std::priority_queue<Seg> heap(segs.begin(), segs.end());
    while (E > atol && E > rtol * std::fabs(I) && numevals < maxevals) {
        Seg sg = heap.top();
        heap.pop();
        double mid = 0.5 * (sg.a + sg.b);
        Seg s1 = evalrule(f, sg.a, mid);
        Seg s2 = evalrule(f, mid, sg.b);
        I = (I - sg.I) + s1.I + s2.I;
        E = (E - sg.E) + s1.E + s2.E;
        numevals += 30;
        heap.push(s1);
        heap.push(s2);
    }
    double Ir = 0.0;
    bool first = true;
    while (!heap.empty()) {
        if (first) { Ir = heap.top().I; first = false; }
        else Ir += heap.top().I;
        heap.pop();
    }
    return Ir;
}

// quadgk with the infinite-interval transformations of QuadGK.jl
template <class F>
double quadgk(F f, std::vector<double> pts, double atol, double rtol) {
    const double s1 = pts.front(), s2 = pts.back();
    const bool inf1 = std::isinf(s1), inf2 = std::isinf(s2);
    if (inf1 && inf2) {
        auto g = [&](double t) {
            double t2 = t * t;
            double den = 1.0 / (1.0 - t2);
            return f(t * den) * (1.0 + t2) * den * den;
        };
        std::vector<double> s;
        for (double x : pts) s.push_back(std::isinf(x) ? std::copysign(1.0, x) : 2.0 * x / (1.0 + std::hypot(1.0, 2.0 * x)));
        return do_quadgk(g, s, atol, rtol);
    }
    if (inf1 || inf2) {
        const double s0 = inf1 ? s2 : s1;
        const double si = inf1 ? s1 : s2;
        if (si < 0.0) {
            auto g = [&](double t) {
                double den = 1.0 / (1.0 - t);
                return f(s0 - t * den) * den * den;
            };
            std::vector<double> s;
            for (double x : pts) s.push_back(1.0 / (1.0 + 1.0 / (s0 - x)));
            std::reverse(s.begin(), s.end());
            return do_quadgk(g, s, atol, rtol);
        }
        auto g = [&](double t) {
            double den = 1.0 / (1.0 - t);
            return f(s0 + t * den) * den * den;
        };
        std::vector<double> s;
        for (double x : pts) s.push_back(1.0 / (1.0 + 1.0 / (x - s0)));
        return do_quadgk(g, s, atol, rtol);
    }
    return do_quadgk(f, pts, atol, rtol);
}

// ---------------------------------------------------------------------------
// boundary corrections (bubbles.jl:99-221)
// ---------------------------------------------------------------------------
void compute_corrs(const Prob& P, int kind, double L, const double* a, const double* da, double atol,
                   double rtol, double* corrs) {
    const oracle_problem* m = P.p;
    const int NO = P.d.NO;
    std::fill(corrs, corrs + 6 * NO, 0.0);
    const double vals[3] = {m->omega_s[NO - 1] + m->nu_s[P.d.Nn - 1], m->omega_t[NO - 1] + m->nu_t[P.d.Nn - 1],
                            m->omega_s[NO - 1] + m->nu_s[P.d.Nn - 1]};
#pragma omp parallel for schedule(dynamic) num_threads(P.p->num_threads > 0 ? P.p->num_threads : omp_get_max_threads())
    for (int job = 0; job < 3 * NO; ++job) {
        const int i = job / 3, ch = job % 3;
        const double Om = (ch == 1) ? m->omega_t[i] : m->omega_s[i];
        auto prop = [&](double v) -> double {
            if (kind == 0) {
                if (ch == 0) return prop_kat(m, a, da, L, v + 0.5 * Om, 0.5 * Om - v) + prop_kat(m, a, da, L, 0.5 * Om - v, v + 0.5 * Om);
                if (ch == 1) return prop_kat(m, a, da, L, v + 0.5 * Om, v - 0.5 * Om) + prop_kat(m, a, da, L, v - 0.5 * Om, v + 0.5 * Om);
                return prop_kat(m, a, da, L, v - 0.5 * Om, v + 0.5 * Om) + prop_kat(m, a, da, L, v + 0.5 * Om, v - 0.5 * Om);
            }
            if (ch == 0) return -prop_plain(m, a, L, v + 0.5 * Om, 0.5 * Om - v);
            if (ch == 1) return -prop_plain(m, a, L, v + 0.5 * Om, v - 0.5 * Om);
            return -prop_plain(m, a, L, v - 0.5 * Om, v + 0.5 * Om);
        };
        const double val = vals[ch];
        const double bm = prop(-val), bp = prop(val);
        const double inf = INFINITY;
        if (std::fabs(bm) > 1e-8) corrs[0 + 2 * (ch + 3 * i)] = quadgk(prop, {-inf, -val}, atol, rtol) / bm;
        if (std::fabs(bp) > 1e-8) corrs[1 + 2 * (ch + 3 * i)] = quadgk(prop, {val, inf}, atol, rtol) / bp;
    }
}

// ---------------------------------------------------------------------------
// task fan-out (flow_{s,t,u}.jl, compute.jl)
// ---------------------------------------------------------------------------
struct Task {
    int kernel, w1, w2, w3;  // 1-based frequency indices as in the reference, -1 = unused
};

std::vector<Task> make_tasks(const Dims& d, bool full) {
    std::vector<Task> T;
    for (int w1 = 1; w1 <= d.NO; ++w1) {
        T.push_back({1, w1, -1, -1});
        for (int w3 = 1; w3 <= d.Nn; ++w3) {
            T.push_back({2, w1, w3, -1});
            T.push_back({3, w1, -1, w3});
            for (int w2 = full ? 1 : w3; w2 <= d.Nn; ++w2) T.push_back({4, w1, w2, w3});
        }
    }
    return T;
}

// get_kernel_args (mesh.jl:30-83)
inline void kernel_args(const oracle_problem* m, int ch, const Task& t, double& W, double& V, double& VP) {
    const double* Om = (ch == 1) ? m->omega_t : m->omega_s;
    const double* nu = (ch == 1) ? m->nu_t : m->nu_s;
    const double inf = INFINITY;
    W = Om[t.w1 - 1];
    V = (t.kernel == 2 || t.kernel == 4) ? nu[t.w2 - 1] : inf;
    VP = (t.kernel == 3 || t.kernel == 4) ? nu[t.w3 - 1] : inf;
}

inline double* out_ptr(const Dims& d, double* act, int comp, int ch, const Task& t) {
    double* cb = act + d.Nsig + comp * d.comp + d.Ns + ch * d.chan;
    const int Ns = d.Ns, NO = d.NO, Nn = d.Nn;
    switch (t.kernel) {
        case 1: return cb + (int64_t)Ns * (t.w1 - 1);
        case 2: return cb + d.K1 + (int64_t)Ns * ((t.w1 - 1) + (int64_t)NO * (t.w2 - 1));
        case 3: return cb + d.K1 + d.K2 + (int64_t)Ns * ((t.w1 - 1) + (int64_t)NO * (t.w3 - 1));
        default:
            return cb + d.K1 + 2 * d.K2 + (int64_t)Ns * ((t.w1 - 1) + (int64_t)NO * ((t.w2 - 1) + (int64_t)Nn * (t.w3 - 1)));
    }
}

struct ThreadScratch {
    std::vector<double> tb1, tb2, tb3, temp;
};

// one channel task: compute_channel_X_{kat,left,central,BSE}! (flow_s.jl:2-56 etc.)
void run_task(const Prob& P, const PassDesc& pd, double L, const Task& t, const double* corrs, int eval,
              double atol, double rtol, double* out, ThreadScratch& ts) {
    const Dims& d = P.d;
    const oracle_problem* m = P.p;
    const int len = d.C * d.Ns;
    Ctx cx;
    cx.P = &P;
    cx.pd = &pd;
    for (int k = 0; k < 4; ++k) cx.A[k] = make_act(d, pd.A[k] ? pd.A[k] : pd.a);
    cx.Lam = L;
    kernel_args(m, pd.ch, t, cx.W, cx.V, cx.VP);
    cx.temp = &ts.temp;
    double* tb1 = ts.tb1.data();
    std::fill(tb1, tb1 + len, 0.0);
    auto f = [&](double* b, double v, double dv) { integrand(cx, b, v, dv); };
    const double ref = L + 0.5 * cx.W;
    const double val = (pd.ch == 1) ? m->omega_t[d.NO - 1] + m->nu_t[d.Nn - 1] : m->omega_s[d.NO - 1] + m->nu_s[d.Nn - 1];
    integrate_log(f, tb1, ts.tb2.data(), ts.tb3.data(), len, 2.0 * ref, 1.0 * val, eval, atol, rtol, -1.0);
    integrate_lin(f, tb1, ts.tb2.data(), ts.tb3.data(), len, -2.0 * ref, 0.0 * ref, eval, atol, rtol);
    integrate_lin(f, tb1, ts.tb2.data(), ts.tb3.data(), len, 0.0 * ref, 2.0 * ref, eval, atol, rtol);
    integrate_log(f, tb1, ts.tb2.data(), ts.tb3.data(), len, 2.0 * ref, 1.0 * val, eval, atol, rtol, 1.0);
    f(tb1, -val, corrs[0 + 2 * (pd.ch + 3 * (t.w1 - 1))]);
    f(tb1, val, corrs[1 + 2 * (pd.ch + 3 * (t.w1 - 1))]);
    for (int c = 0; c < d.C; ++c) {
        double* o = out_ptr(d, out, c, pd.ch, t);
        for (int i = 0; i < d.Ns; ++i) o[i] = tb1[(int64_t)c * d.Ns + i];
    }
}

int nthreads(const Prob& P) { return P.p->num_threads > 0 ? P.p->num_threads : omp_get_max_threads(); }

void run_pass(const Prob& P, const PassDesc base[3], double L, bool full, const double* corrs, int eval,
              double atol, double rtol, double* out) {
    const Dims& d = P.d;
    std::vector<Task> tasks = make_tasks(d, full);
    const int64_t nt = (int64_t)tasks.size() * 3;
    oracle_stats total{0, 0, 0, 0};
    const oracle_stats saved = g_stats;
#pragma omp parallel num_threads(nthreads(P))
    {
        g_stats = oracle_stats{};
        ThreadScratch ts;
        const int len = d.C * d.Ns;
        ts.tb1.resize(len);
        ts.tb2.resize(len);
        ts.tb3.resize(len);
        ts.temp.resize(2 * len);
        const int64_t stride = P.p->task_stride > 1 ? P.p->task_stride : 1;
#pragma omp for schedule(dynamic, 1)
        for (int64_t j = 0; j < nt; ++j) {
            if (j % stride) continue;
            const Task& t = tasks[j / 3];
            run_task(P, base[j % 3], L, t, corrs, eval, atol, rtol, out, ts);
        }
#pragma omp critical
        {
            total.integrand_evals += g_stats.integrand_evals;
            total.gathered_values += g_stats.gathered_values;
            total.overlap_terms += g_stats.overlap_terms;
            total.reevals += g_stats.reevals;
            for (int k = 0; k < 24; ++k) total.level_hist[k] += g_stats.level_hist[k];
        }
    }
    g_stats = saved;
    g_stats.integrand_evals += total.integrand_evals;
    g_stats.gathered_values += total.gathered_values;
    g_stats.overlap_terms += total.overlap_terms;
    g_stats.reevals += total.reevals;
    for (int k = 0; k < 24; ++k) g_stats.level_hist[k] += total.level_hist[k];
}

// image of (comp, channel) under v <-> v' exchange: the component it is read from and the sign
// (su2: action_su2.jl:141-251, the same component with sign +; u1-dm: action_u1_dm.jl:170-339,
// s and t: DM -> -DM, zd -> -dz, dz -> -zd; u: zd -> -zd, dz -> -dz)
inline void swap_image(const Prob& P, int c, int ch, int& src, double& sgn) {
    src = c;
    sgn = 1.0;
    if (P.p->symmetry == 0) return;
    if (ch == 2) {
        if (c == 4 || c == 5) sgn = -1.0;
        return;
    }
    if (c == 2) sgn = -1.0;
    else if (c == 4) { src = 5; sgn = -1.0; }
    else if (c == 5) { src = 4; sgn = -1.0; }
}

// symmetrize! (action_su2.jl:141-173, action_u1_dm.jl:170-214)
void symmetrize(const Prob& P, double* a) {
    const Dims& d = P.d;
    const int Ns = d.Ns, NO = d.NO, Nn = d.Nn;
    // the reference writes component by component in place; for u1-dm, zd and dz of the s and t
    // channels read each other's lower triangle, which neither write touches
    for (int c = 0; c < d.C; ++c) {
        for (int ch = 0; ch < 3; ++ch) {
            int sc;
            double sg;
            swap_image(P, c, ch, sc, sg);
            double* q3 = a + d.Nsig + c * d.comp + d.Ns + ch * d.chan + d.K1 + 2 * d.K2;
            const double* s3 = a + d.Nsig + sc * d.comp + d.Ns + ch * d.chan + d.K1 + 2 * d.K2;
            for (int v = 0; v < Nn; ++v)
                for (int vp = v + 1; vp < Nn; ++vp)
                    for (int w = 0; w < NO; ++w)
                        for (int i = 0; i < Ns; ++i) {
                            int src = (ch == 2) ? i : P.exch[i];
                            q3[i + (int64_t)Ns * (w + (int64_t)NO * (v + (int64_t)Nn * vp))] =
                                sg * s3[src + (int64_t)Ns * (w + (int64_t)NO * (vp + (int64_t)Nn * v))];
                        }
        }
    }
}

// symmetrize_add_to! (action_su2.jl:176-251, action_u1_dm.jl:217-340): a += a_l + (v <-> v') image of a_l
void symmetrize_add_to(const Prob& P, const double* al, double* a) {
    const Dims& d = P.d;
    const int Ns = d.Ns, NO = d.NO, Nn = d.Nn;
    for (int c = 0; c < d.C; ++c) {
        for (int ch = 0; ch < 3; ++ch) {
            int sc;
            double sg;
            swap_image(P, c, ch, sc, sg);
            const int64_t off = d.Nsig + c * d.comp + d.Ns + ch * d.chan;
            const double* l1 = al + off;
            const double* m1 = al + d.Nsig + sc * d.comp + d.Ns + ch * d.chan;  // the image's component
            double* o1 = a + off;
            auto ex = [&](int i) { return ch == 2 ? i : P.exch[i]; };
            for (int w = 0; w < NO; ++w)
                for (int i = 0; i < Ns; ++i)
                    o1[i + (int64_t)Ns * w] += l1[i + (int64_t)Ns * w] + sg * m1[ex(i) + (int64_t)Ns * w];
            const double* l21 = l1 + d.K1;
            const double* l22 = l1 + d.K1 + d.K2;
            const double* m21 = m1 + d.K1;
            const double* m22 = m1 + d.K1 + d.K2;
            double* o21 = o1 + d.K1;
            double* o22 = o1 + d.K1 + d.K2;
            for (int v = 0; v < Nn; ++v)
                for (int w = 0; w < NO; ++w)
                    for (int i = 0; i < Ns; ++i) {
                        int64_t k = i + (int64_t)Ns * (w + (int64_t)NO * v);
                        int64_t ke = ex(i) + (int64_t)Ns * (w + (int64_t)NO * v);
                        o21[k] += l21[k] + sg * m22[ke];
                        o22[k] += l22[k] + sg * m21[ke];
                    }
            const double* l3 = l1 + d.K1 + 2 * d.K2;
            const double* m3 = m1 + d.K1 + 2 * d.K2;
            double* o3 = o1 + d.K1 + 2 * d.K2;
            for (int vp = 0; vp < Nn; ++vp)
                for (int v = 0; v < Nn; ++v)
                    for (int w = 0; w < NO; ++w)
                        for (int i = 0; i < Ns; ++i) {
                            int64_t k = i + (int64_t)Ns * (w + (int64_t)NO * (v + (int64_t)Nn * vp));
                            int64_t ke = ex(i) + (int64_t)Ns * (w + (int64_t)NO * (vp + (int64_t)Nn * v));
                            o3[k] += l3[k] + sg * m3[ke];
                        }
        }
    }
}

// vertex part of an action (everything after Σ, excluding bare)
void axpy_gamma(const Dims& d, double fac, const double* x, double* y) {
    for (int c = 0; c < d.C; ++c) {
        int64_t off = d.Nsig + c * d.comp + d.Ns;
        for (int64_t k = 0; k < 3 * d.chan; ++k) y[off + k] += fac * x[off + k];
    }
}
void set_gamma(const Dims& d, double fac, double* y) {
    for (int c = 0; c < d.C; ++c) {
        int64_t off = d.Nsig + c * d.comp + d.Ns;
        for (int64_t k = 0; k < 3 * d.chan; ++k) y[off + k] = fac == 0.0 ? 0.0 : y[off + k] * fac;
    }
}
void copy_gamma(const Dims& d, const double* x, double* y) {
    for (int c = 0; c < d.C; ++c) {
        int64_t off = d.Nsig + c * d.comp + d.Ns;
        std::memcpy(y + off, x + off, sizeof(double) * 3 * d.chan);
    }
}

PassDesc pass(int ch, PropKind pk, const double* a, const double* da, const double* A1, int m1, const double* A2,
              int m2, const double* A3 = nullptr, int m3 = 7, const double* A4 = nullptr, int m4 = 7) {
    PassDesc p;
    p.ch = ch;
    p.prop = pk;
    p.a = a;
    p.da = da;
    p.A[0] = A1;
    p.A[1] = A2;
    p.A[2] = A3 ? A3 : a;
    p.A[3] = A4 ? A4 : a;
    p.mask[0] = m1;
    p.mask[1] = m2;
    p.mask[2] = m3;
    p.mask[3] = m4;
    return p;
}

const int ALL = CH_S | CH_T | CH_U;

// Katanin 1-loop passes (flow_su2_{s,t,u}.jl:2-55)
void passes_kat(const double* a, const double* da, PassDesc out[3]) {
    out[0] = pass(0, PROP_KAT, a, da, a, ALL, a, ALL);
    out[1] = pass(1, PROP_KAT, a, da, a, ALL, a, ALL, a, ALL, a, ALL);
    out[2] = pass(2, PROP_KAT, a, da, a, ALL, a, ALL);
}
// left passes (flow_su2_s.jl:57-109, t :89-173, u :57-109): slot 1 from da without own channel
void passes_left(const double* a, const double* da, PassDesc out[3]) {
    out[0] = pass(0, PROP_PLAIN, a, nullptr, da, CH_T | CH_U, a, ALL);
    out[1] = pass(1, PROP_PLAIN, a, nullptr, da, CH_S | CH_U, a, ALL, da, CH_S | CH_T, a, ALL);
    out[2] = pass(2, PROP_PLAIN, a, nullptr, da, CH_S | CH_T, a, ALL);
}
// central passes (flow_su2_s.jl:112-159, t :176-255, u :112-159): slot 2 from da_l, own channel
void passes_central(const double* a, const double* dal, PassDesc out[3]) {
    out[0] = pass(0, PROP_PLAIN, a, nullptr, a, ALL, dal, CH_S);
    out[1] = pass(1, PROP_PLAIN, a, nullptr, a, ALL, dal, CH_T, a, ALL, dal, CH_U);
    out[2] = pass(2, PROP_PLAIN, a, nullptr, a, ALL, dal, CH_U);
}
// parquet BSE passes (BSE_su2_{s,t,u}.jl): slot 1 without own channel
void passes_bse(const double* a, PassDesc out[3]) {
    out[0] = pass(0, PROP_PLAIN, a, nullptr, a, CH_T | CH_U, a, ALL);
    out[1] = pass(1, PROP_PLAIN, a, nullptr, a, CH_S | CH_U, a, ALL, a, CH_S | CH_T, a, ALL);
    out[2] = pass(2, PROP_PLAIN, a, nullptr, a, CH_S | CH_T, a, ALL);
}

// ---------------------------------------------------------------------------
// self energy kernels (flow_su2_self.jl, SDE_su2.jl:45-77)
// ---------------------------------------------------------------------------
enum SigmaKind { SIG_FLOW = 0, SIG_CORR1 = 1, SIG_CORR2 = 2, SIG_SDE = 3 };

double sigma_kernel(const Prob& P, SigmaKind kind, double L, double w, double v, const double* a,
                    const double* aux) {
    const oracle_problem* m = P.p;
    const Dims& d = P.d;
    g_stats.sigma_evals += 1;
    Buf b1s, b1t, b1u, b2s, b2t, b2u;
    int m_loc = ALL, m_non = ALL;
    const double* src = a;
    if (kind == SIG_SDE) {
        const double inf = INFINITY;
        b1s = buffer_s(m, v + w, inf, 0.5 * (v - w));
        b2s = buffer_s(m, v + w, inf, 0.5 * (-v + w));
        b1t = b1u = b2t = b2u = empty_buf();
        m_loc = m_non = CH_S;
        src = aux;  // a2 provides the vertex, a1 the propagator
    } else {
        b1s = buffer_s(m, v + w, 0.5 * (-v + w), 0.5 * (v - w));
        b1t = buffer_t(m, 0.0, w, v);
        b1u = buffer_u(m, -v + w, 0.5 * (v + w), 0.5 * (v + w));
        b2s = buffer_s(m, v + w, 0.5 * (-v + w), 0.5 * (-v + w));
        b2t = buffer_t(m, v - w, 0.5 * (v + w), 0.5 * (v + w));
        b2u = buffer_u(m, 0.0, w, v);
        if (kind == SIG_CORR1) {
            src = aux;
            m_loc = CH_S | CH_T;
            m_non = CH_S | CH_U;
        }
    }
    Act A = make_act(d, src);
    double val;
    if (P.p->symmetry == 0) {
        val = 3.0 * gamma_comp_site(P, A, 0, 0, b2s, b2t, b2u, m_loc) + gamma_comp_site(P, A, 1, 0, b2s, b2t, b2u, m_loc);
        for (int j = 0; j < d.Ns; ++j)
            val -= 2.0 * P.mult[j] * (2.0 * P.S) * gamma_comp_site(P, A, 1, j, b1s, b1t, b1u, m_non);
    } else {
        // flow_u1_dm_self.jl:2-33, SDE_u1_dm.jl:59-91: 2 Γxx + Γzz + Γdd on site 1, Γdd over the lattice
        val = 2.0 * gamma_comp_site(P, A, 0, 0, b2s, b2t, b2u, m_loc) + gamma_comp_site(P, A, 1, 0, b2s, b2t, b2u, m_loc) +
              gamma_comp_site(P, A, 3, 0, b2s, b2t, b2u, m_loc);
        for (int j = 0; j < d.Ns; ++j)
            val -= 2.0 * P.mult[j] * gamma_comp_site(P, A, 3, j, b1s, b1t, b1u, m_non);
    }
    switch (kind) {
        case SIG_FLOW: val *= S_single(m, a, L, v) / (2.0 * kPi); break;
        case SIG_CORR1: val *= -G_full(m, a, L, v) / (2.0 * kPi); break;
        case SIG_CORR2: {
            double g = G_full(m, a, L, v);
            val *= g * g * get_sigma(m, aux, v) / (2.0 * kPi);
            break;
        }
        case SIG_SDE: val *= -G_full(m, a, L, v) / (2.0 * kPi); break;
    }
    return val;
}

void sigma_integrals(const Prob& P, SigmaKind kind, double L, const double* a, const double* aux, double atol,
                     double rtol, double* out /* [Nsig], index 0 untouched */) {
    const oracle_problem* m = P.p;
    const int n = P.d.Nsig;
    int64_t evals = 0;
    const oracle_stats saved = g_stats;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(P)) reduction(+ : evals)
    for (int i = 1; i < n; ++i) {
        g_stats.sigma_evals = 0;
        const double w = m->sigma[i];
        auto f = [&](double v) { return sigma_kernel(P, kind, L, w, v, a, aux); };
        const double inf = INFINITY;
        out[i] = quadgk(f, {-inf, -2.0 * L, 0.0, 2.0 * L, inf}, atol, rtol);
        evals += g_stats.sigma_evals;
    }
    g_stats = saved;
    g_stats.sigma_evals += evals;
}


// ---------------------------------------------------------------------------
// correlations χ (src/Observable/correlation_lib/correlation_lib.jl:2-30,
// correlation_su2.jl:14-87).  The reference integrates with Cubature.jl
// (compat 1.5, wrapping S. G. Johnson's "cubature" library, not part of the
// reference tree): hcubature_v, h-adaptive, Genz-Malik degree-7/5 rule for
// dim = 2, split along the dimension with the largest fourth difference, and
// the vectorised ("parallel") refinement that bisects, per round, every
// largest-error region needed to bring the remaining error under the bound.
// ---------------------------------------------------------------------------
struct Region2 {
    double c[2], h[2], vol, val, err;
    int split;
};

constexpr double kGML2 = 0.3585685828003180919906451539079374954541;  // sqrt(9/70)
constexpr double kGML4 = 0.9486832980505137995996680633298155601160;  // sqrt(9/10)
constexpr double kGML5 = 0.6882472016116852977216287342936235251269;  // sqrt(9/19)

// the 17 Genz-Malik points of a 2-D region in the library's order
inline void gm_points(const Region2& R, double pts[17][2]) {
    int k = 0;
    pts[k][0] = R.c[0];
    pts[k][1] = R.c[1];
    ++k;
    for (int d = 0; d < 2; ++d) {
        const double w2 = R.h[d] * kGML2, w4 = R.h[d] * kGML4;
        const double off[4] = {-w2, w2, -w4, w4};
        for (int q = 0; q < 4; ++q) {
            pts[k][0] = R.c[0];
            pts[k][1] = R.c[1];
            pts[k][d] = R.c[d] + off[q];
            ++k;
        }
    }
    const double a = R.h[0] * kGML4, b = R.h[1] * kGML4;
    const double rr[4][2] = {{-a, -b}, {a, -b}, {a, b}, {-a, b}};
    for (int q = 0; q < 4; ++q) {
        pts[k][0] = R.c[0] + rr[q][0];
        pts[k][1] = R.c[1] + rr[q][1];
        ++k;
    }
    const double a5 = R.h[0] * kGML5, b5 = R.h[1] * kGML5;
    const double cs[4][2] = {{a5, b5}, {-a5, b5}, {-a5, -b5}, {a5, -b5}};
    for (int q = 0; q < 4; ++q) {
        pts[k][0] = R.c[0] + cs[q][0];
        pts[k][1] = R.c[1] + cs[q][1];
        ++k;
    }
}

// rule75genzmalik_evalError for dim = 2
inline void gm_eval(Region2& R, const double* v) {
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
    const double ratio = (kGML2 * kGML2) / (kGML4 * kGML4);
    const double val0 = v[0];
    double sum2 = 0.0, sum3 = 0.0, diff[2];
    for (int d = 0; d < 2; ++d) {
        const double v0 = v[1 + 4 * d], v1 = v[2 + 4 * d], v2 = v[3 + 4 * d], v3 = v[4 + 4 * d];
        sum2 += v0 + v1;
        sum3 += v2 + v3;
        diff[d] = std::fabs(v0 + v1 - 2 * val0 - ratio * (v2 + v3 - 2 * val0));
    }
    double sum4 = 0.0, sum5 = 0.0;
    for (int q = 0; q < 4; ++q) sum4 += v[9 + q];
    for (int q = 0; q < 4; ++q) sum5 += v[13 + q];
    const double result = R.vol * (w1 * val0 + w2 * sum2 + w3 * sum3 + w4 * sum4 + w5 * sum5);
    const double res5 = R.vol * (e1 * val0 + e2 * sum2 + e3 * sum3 + e4 * sum4);
    R.val = result;
    R.err = std::fabs(res5 - result);
    R.split = diff[1] > diff[0] ? 1 : 0;
}

// regions waiting to be cut, largest error first; equal errors leave in the order
// they were filed (a counter stamps every push).  The C library's binary heap
// leaves ties in an order set by its layout; this rule is fixed instead, and the
// GPU kernel keeps the same order with a sorted list (stable sort of each round's
// halves, merged after the older entries of equal error).
struct RegionQueue {
    struct E {
        double err;
        long long stamp;
        int idx;
    };
    std::vector<E> h;
    long long next = 0;
    // a has lower priority than b
    static bool lower(const E& a, const E& b) { return a.err < b.err || (a.err == b.err && a.stamp > b.stamp); }
    void push(double err, int i) {
        h.push_back({err, next++, i});
        std::push_heap(h.begin(), h.end(), lower);
    }
    int pop() {
        std::pop_heap(h.begin(), h.end(), lower);
        const int i = h.back().idx;
        h.pop_back();
        return i;
    }
    bool empty() const { return h.empty(); }
};

// the final total: 256 consecutive blocks of regions (index order), each summed in
// order, then the block sums in order (the GPU block's threads sum one block each)
constexpr int kChiSumBlocks = 256;

template <class F>
double hcubature2(F& f, const double xmin[2], const double xmax[2], double abstol, double reltol,
                  long long maxevals) {
    auto eval = [&](Region2& R) {
        double pts[17][2], v[17];
        gm_points(R, pts);
        for (int k = 0; k < 17; ++k) v[k] = f(pts[k][0], pts[k][1]);
        gm_eval(R, v);
    };
    auto converged = [&](double err, double val) { return !(err > abstol && err > std::fabs(val) * reltol); };
    std::vector<Region2> regs(1);
    Region2& R0 = regs[0];
    for (int d = 0; d < 2; ++d) {
        R0.c[d] = 0.5 * (xmin[d] + xmax[d]);
        R0.h[d] = 0.5 * (xmax[d] - xmin[d]);
    }
    R0.vol = (2.0 * R0.h[0]) * (2.0 * R0.h[1]);
    eval(R0);
    RegionQueue heap;
    heap.push(R0.err, 0);
    double tot_val = R0.val, tot_err = R0.err;
    long long numeval = 17;
    while (numeval < maxevals) {
        if (converged(tot_err, tot_val)) break;
        // the round's bound compares the remaining error with the total value at its start
        double ee_err = tot_err;
        const double ee_val = tot_val;
        std::vector<int> cut;  // (first half, second half) per cut region
        do {
            const int bi = heap.pop();
            tot_val -= regs[bi].val;
            tot_err -= regs[bi].err;
            ee_err -= regs[bi].err;
            // cut_region: halve along the split dimension; the first half keeps the index
            Region2 R = regs[bi];
            const int d = R.split;
            Region2 R2 = R;
            R.h[d] *= 0.5;
            R.vol *= 0.5;
            R2.h[d] = R.h[d];
            R2.vol = (2.0 * R2.h[0]) * (2.0 * R2.h[1]);
            R.c[d] -= R.h[d];
            R2.c[d] += R.h[d];
            regs[bi] = R;
            regs.push_back(R2);
            cut.push_back(bi);
            cut.push_back((int)regs.size() - 1);
            numeval += 34;
            if (converged(ee_err, ee_val)) break;
        } while (!heap.empty() && numeval < maxevals);
        for (int r : cut) eval(regs[r]);
        for (int r : cut) {
            heap.push(regs[r].err, r);
            tot_val += regs[r].val;
            tot_err += regs[r].err;
        }
    }
    const int n = (int)regs.size();
    const int c = (n + kChiSumBlocks - 1) / kChiSumBlocks;
    double I = 0.0;
    for (int t = 0; t < kChiSumBlocks; ++t) {
        double p = 0.0;
        for (int q = std::min(n, t * c); q < std::min(n, (t + 1) * c); ++q) p += regs[q].val;
        I += p;
    }
    return I;
}

// integrate_χ_boxes (correlation_lib.jl:2-30): nine boxes of [0,1]^2 around the image of ±width
template <class F>
double chi_boxes(F& f, double width, double abstol, double reltol) {
    const double wp = (width - 2.0 + std::sqrt(width * width + 4.0)) / (2.0 * width);
    const double s = std::fabs(wp - 0.5);
    const double lo[3] = {0.0, 0.5 - s, 0.5 + s}, hi[3] = {0.5 - s, 0.5 + s, 1.0};
    // the reference's order: top line (y high), middle, bottom
    const int rows[3] = {2, 1, 0};
    double I = 0.0;
    bool first = true;
    for (int rr = 0; rr < 3; ++rr) {
        for (int cc = 0; cc < 3; ++cc) {
            const double xmin[2] = {lo[cc], lo[rows[rr]]}, xmax[2] = {hi[cc], hi[rows[rr]]};
            const double v = hcubature2(f, xmin, xmax, abstol, reltol, 10000000LL);
            if (first) { I = v; first = false; }
            else I += v;
        }
    }
    return I;
}

// compute_χ_kernel! (correlation_su2.jl:14-55) at (x, y) in [0,1]^2
double chi_kernel(const Prob& P, const Act& A, const double* Sig, double L, int site, double w, double x, double y) {
    const oracle_problem* m = P.p;
    const double v = (2.0 * x - 1.0) / ((1.0 - x) * x);
    const double vp = (2.0 * y - 1.0) / ((1.0 - y) * y);
    const double dv = (2.0 * x * x - 2.0 * x + 1) / ((1.0 - x) * (1.0 - x) * x * x);
    const double dvp = (2.0 * y * y - 2.0 * y + 1) / ((1.0 - y) * (1.0 - y) * y * y);
    Buf bs1 = buffer_s(m, v + vp, 0.5 * (v - w - vp), 0.5 * (-v - w + vp));
    Buf bt1 = buffer_t(m, w, v, vp);
    Buf bu1 = buffer_u(m, v - vp, 0.5 * (v - w + vp), 0.5 * (v + w + vp));
    const double twoS = 2.0 * P.S;
    const double tp2 = (2.0 * kPi) * (2.0 * kPi);
    double val = -(twoS * twoS) * gamma_comp_site(P, A, 0, site, bs1, bt1, bu1, ALL) / tp2;
    if (site == 0) {
        Buf bs2 = buffer_s(m, v + vp, 0.5 * (v - w - vp), 0.5 * (v + w - vp));
        Buf bt2 = buffer_t(m, -v + vp, 0.5 * (v - w + vp), 0.5 * (v + w + vp));
        Buf bu2 = buffer_u(m, -w, v, vp);
        const double vs = gamma_comp_site(P, A, 0, site, bs2, bt2, bu2, ALL);
        const double vd = gamma_comp_site(P, A, 1, site, bs2, bt2, bu2, ALL);
        val -= twoS * (vs - vd) / (2.0 * tp2);
    }
    val *= G_full(m, Sig, L, v - 0.5 * w) * G_full(m, Sig, L, v + 0.5 * w) * dv;
    val *= G_full(m, Sig, L, vp - 0.5 * w) * G_full(m, Sig, L, vp + 0.5 * w) * dvp;
    return val;
}

// compute_χ_kernel_{xx,zz,xy}! (correlation_u1_dm.jl:14-149) at (x, y) in [0,1]^2; k = 0 xx, 1 zz, 2 xy
double chi_kernel_u1dm(const Prob& P, const Act& A, const double* Sig, double L, int k, int site, double w, double x,
                       double y) {
    const oracle_problem* m = P.p;
    const double v = (2.0 * x - 1.0) / ((1.0 - x) * x);
    const double vp = (2.0 * y - 1.0) / ((1.0 - y) * y);
    const double dv = (2.0 * x * x - 2.0 * x + 1) / ((1.0 - x) * (1.0 - x) * x * x);
    const double dvp = (2.0 * y * y - 2.0 * y + 1) / ((1.0 - y) * (1.0 - y) * y * y);
    Buf bs1 = buffer_s(m, v + vp, 0.5 * (v - w - vp), 0.5 * (-v - w + vp));
    Buf bt1 = buffer_t(m, w, v, vp);
    Buf bu1 = buffer_u(m, v - vp, 0.5 * (v - w + vp), 0.5 * (v + w + vp));
    const double tp2 = (2.0 * kPi) * (2.0 * kPi);
    const int comp1[3] = {0, 1, 2};
    double val = -gamma_comp_site(P, A, comp1[k], site, bs1, bt1, bu1, ALL) / tp2;
    if (site == 0) {
        Buf bs2 = buffer_s(m, v + vp, 0.5 * (v - w - vp), 0.5 * (v + w - vp));
        Buf bt2 = buffer_t(m, -v + vp, 0.5 * (v - w + vp), 0.5 * (v + w + vp));
        Buf bu2 = buffer_u(m, -w, v, vp);
        auto g = [&](int c) { return gamma_comp_site(P, A, c, 0, bs2, bt2, bu2, ALL); };
        if (k == 0) {
            const double vzz = g(1), vdd = g(3);
            val -= (vzz - vdd) / (2.0 * tp2);
        } else if (k == 1) {
            const double vxx = g(0), vzz = g(1), vdd = g(3);
            val -= (2.0 * vxx - vzz - vdd) / (2.0 * tp2);
        } else {
            const double vzd = g(4), vdz = g(5);
            val -= (vzd - vdz) / (2.0 * tp2);
        }
    }
    val *= G_full(m, Sig, L, v - 0.5 * w) * G_full(m, Sig, L, v + 0.5 * w) * dv;
    val *= G_full(m, Sig, L, vp - 0.5 * w) * G_full(m, Sig, L, vp + 0.5 * w) * dvp;
    return val;
}

void reset_stats() { g_stats = oracle_stats{}; }

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int64_t oracle_action_size(const oracle_problem* p) { return make_dims(p).total; }

void oracle_last_stats(oracle_stats* out) { *out = g_stats; }

int oracle_corrs(const oracle_problem* p, int kind, double Lam, const double* a, const double* da, double atol,
                 double rtol, double* corrs) {
    Prob P = make_prob(p);
    compute_corrs(P, kind, Lam, a, da, atol, rtol, corrs);
    return 0;
}

int oracle_dsigma(const oracle_problem* p, double Lam, const double* a, double* da, double atol, double rtol) {
    Prob P = make_prob(p);
    reset_stats();
    sigma_integrals(P, SIG_FLOW, Lam, a, nullptr, atol, rtol, da);
    return 0;
}

int oracle_symmetrize(const oracle_problem* p, double* a) {
    Prob P = make_prob(p);
    symmetrize(P, a);
    return 0;
}

int oracle_symmetrize_add_to(const oracle_problem* p, const double* a_l, double* a) {
    Prob P = make_prob(p);
    symmetrize_add_to(P, a_l, a);
    return 0;
}

int oracle_dgamma(const oracle_problem* p, int loops, double Lam, const double* a, double* da, double* da_l,
                  double* da_c, double* da_temp, double* da_sigma, int eval, double gatol, double grtol,
                  int sigma_corr, double satol, double srtol) {
    Prob P = make_prob(p);
    const Dims& d = P.d;
    reset_stats();
    oracle_stats acc{0, 0, 0, 0};
    std::vector<double> corrs(6 * d.NO);
    // compute_dΓ_1l! (compute.jl:57-112)
    compute_corrs(P, 0, Lam, a, da, gatol, grtol, corrs.data());
    PassDesc pk[3];
    passes_kat(a, da, pk);
    run_pass(P, pk, Lam, false, corrs.data(), eval, gatol, grtol, da);
    symmetrize(P, da);
    if (loops >= 2) {
        // compute_dΓ_2l! (compute.jl:115-174)
        compute_corrs(P, 1, Lam, a, nullptr, gatol, grtol, corrs.data());
        PassDesc pl[3];
        passes_left(a, da, pl);
        run_pass(P, pl, Lam, true, corrs.data(), eval, gatol, grtol, da_l);
        symmetrize_add_to(P, da_l, da);
    }
    if (loops >= 3) {
        // compute_dΓ_ml! (compute.jl:177-287)
        set_gamma(d, 0.0, da_temp);
        set_gamma(d, 0.0, da_sigma);
        symmetrize_add_to(P, da_l, da_temp);
        for (int loop = 3; loop <= loops; ++loop) {
            PassDesc pc[3];
            passes_central(a, da_l, pc);
            run_pass(P, pc, Lam, false, corrs.data(), eval, gatol, grtol, da_c);
            PassDesc pl[3];
            passes_left(a, da_temp, pl);
            run_pass(P, pl, Lam, true, corrs.data(), eval, gatol, grtol, da_l);
            symmetrize(P, da_c);
            copy_gamma(d, da_c, da_temp);
            symmetrize_add_to(P, da_l, da_temp);
            axpy_gamma(d, 1.0, da_c, da_sigma);
            axpy_gamma(d, 1.0, da_temp, da);
        }
        acc = g_stats;
        if (sigma_corr) {
            // compute_dΣ_corr! (flow_self.jl:23-51)
            sigma_integrals(P, SIG_CORR1, Lam, a, da_sigma, satol, srtol, da_sigma);
            std::vector<double> c2(d.Nsig, 0.0);
            sigma_integrals(P, SIG_CORR2, Lam, a, da_sigma, satol, srtol, c2.data());
            for (int i = 1; i < d.Nsig; ++i) {
                da[i] += da_sigma[i];
                da[i] += c2[i];
            }
            acc.sigma_evals = g_stats.sigma_evals;
            g_stats = acc;
        }
    }
    return 0;
}

int oracle_bse(const oracle_problem* p, double Lam, const double* a1, double* a2, const double* corrs,
               int eval, double atol, double rtol) {
    Prob P = make_prob(p);
    reset_stats();
    // compute_Γ! (compute.jl:2-54) has no corrs step of its own: it reuses the
    // buffer filled by the preceding compute_Σ! (parquet.jl:54-68)
    PassDesc pb[3];
    passes_bse(a1, pb);
    run_pass(P, pb, Lam, false, corrs, eval, atol, rtol, a2);
    symmetrize(P, a2);
    return 0;
}

int oracle_sde(const oracle_problem* p, double Lam, const double* a1, double* a2, double* corrs, int eval,
               double gatol, double grtol, double satol, double srtol) {
    Prob P = make_prob(p);
    const Dims& d = P.d;
    reset_stats();
    compute_corrs(P, 1, Lam, a1, nullptr, gatol, grtol, corrs);
    // reduced s bubble (SDE.jl:2-56): slot 1 is the bare vertex, kernels 1 and 3 only
    PassDesc pd = pass(0, PROP_PLAIN, a1, nullptr, a1, 0, a1, ALL);
    pd.reduced = true;
    std::vector<Task> tasks;
    for (int w1 = 1; w1 <= d.NO; ++w1) {
        tasks.push_back({1, w1, -1, -1});
        for (int w3 = 1; w3 <= d.Nn; ++w3) tasks.push_back({3, w1, -1, w3});
    }
#pragma omp parallel num_threads(nthreads(P))
    {
        ThreadScratch ts;
        const int len = d.C * d.Ns;
        ts.tb1.resize(len);
        ts.tb2.resize(len);
        ts.tb3.resize(len);
        ts.temp.resize(2 * len);
#pragma omp for schedule(dynamic, 1)
        for (int64_t j = 0; j < (int64_t)tasks.size(); ++j)
            run_task(P, pd, Lam, tasks[j], corrs, eval, gatol, grtol, a2, ts);
    }
    sigma_integrals(P, SIG_SDE, Lam, a1, a2, satol, srtol, a2);
    return 0;
}

int oracle_chi(const oracle_problem* p, double Lam, const double* a, const double* chi_mesh, int num_chi,
               double atol, double rtol, double* chi) {
    Prob P = make_prob(p);
    const Dims& d = P.d;
    Act A = make_act(d, a);
    const oracle_problem* m = p;
    if (p->symmetry == 1) {
        // compute_χ! (correlation_u1_dm.jl:152-190): χxx, χzz, χxy, each column-major [Ns, num_chi]
        const int64_t plane = (int64_t)d.Ns * num_chi;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(P)) collapse(2)
        for (int w = 0; w < num_chi; ++w) {
            for (int i = 0; i < d.Ns; ++i) {
                const double wv = chi_mesh[w];
                const double ref = Lam + 0.5 * wv;
                for (int k = 0; k < 3; ++k) {
                    auto f = [&](double x, double y) { return chi_kernel_u1dm(P, A, a, Lam, k, i, wv, x, y); };
                    chi[k * plane + i + (int64_t)d.Ns * w] = chi_boxes(f, 4.0 * ref, atol, rtol);
                }
                if (i == 0) {
                    auto g = [&](double v) {
                        return G_full(m, a, Lam, v - 0.5 * wv) * G_full(m, a, Lam, v + 0.5 * wv) / (4.0 * kPi);
                    };
                    const double inf = INFINITY;
                    const double res = quadgk(g, {-inf, -2.0 * ref, 0.0, 2.0 * ref, inf}, atol, rtol);
                    chi[0 * plane + (int64_t)d.Ns * w] += res;
                    chi[1 * plane + (int64_t)d.Ns * w] += res;
                }
            }
        }
        return 0;
    }
    // compute_χ! (correlation_su2.jl:58-86): χ[i, w], column-major [Ns, num_chi]
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(P)) collapse(2)
    for (int w = 0; w < num_chi; ++w) {
        for (int i = 0; i < d.Ns; ++i) {
            const double wv = chi_mesh[w];
            const double ref = Lam + 0.5 * wv;
            auto f = [&](double x, double y) { return chi_kernel(P, A, a, Lam, i, wv, x, y); };
            double c = chi_boxes(f, 4.0 * ref, atol, rtol);
            if (i == 0) {
                auto g = [&](double v) {
                    return (2.0 * P.S) * G_full(m, a, Lam, v - 0.5 * wv) * G_full(m, a, Lam, v + 0.5 * wv) / (4.0 * kPi);
                };
                const double inf = INFINITY;
                c += quadgk(g, {-inf, -2.0 * ref, 0.0, 2.0 * ref, inf}, atol, rtol);
            }
            chi[i + (int64_t)d.Ns * w] = c;
        }
    }
    return 0;
}

int oracle_buffer_kernel(const oracle_problem* p, int ch, double w, double v, double vp) {
    Buf b = ch == 1 ? buffer_s(p, w, v, vp) : (ch == 2 ? buffer_t(p, w, v, vp) : buffer_u(p, w, v, vp));
    return b.kernel;
}

int oracle_gamma_comp(const oracle_problem* p, const double* a, int comp, double ws, double vs, double vsp,
                      double wt, double vt, double vtp, double wu, double vu, double vup, int ch_mask,
                      double* out) {
    Prob P = make_prob(p);
    Act A = make_act(P.d, a);
    Buf bs = buffer_s(p, ws, vs, vsp), bt = buffer_t(p, wt, vt, vtp), bu = buffer_u(p, wu, vu, vup);
    std::vector<double> temp((size_t)P.d.C * P.d.Ns);
    gather_slot(P, A, bs, bt, bu, ch_mask, temp.data(), P.d.Ns);
    for (int i = 0; i < P.d.Ns; ++i) out[i] = temp[(size_t)comp * P.d.Ns + i];
    return 0;
}

int oracle_vertex_channel(const oracle_problem* p, const double* a, int comp, int ch, double w, double v,
                          double vp, double* out) {
    Prob P = make_prob(p);
    Act A = make_act(P.d, a);
    const double* Om = ch == 2 ? p->omega_t : p->omega_s;
    const double* nu = ch == 2 ? p->nu_t : p->nu_s;
    Buf b = get_buffer(w, v, vp, Om, (int)p->num_omega, nu, (int)p->num_nu, false, false, false, false, false);
    std::fill(out, out + P.d.Ns, 0.0);
    interp_add(P, A.q[comp][ch - 1], b, 1.0, out, P.d.Ns);
    return 0;
}

double oracle_get_sigma(const oracle_problem* p, const double* a, double w) { return get_sigma(p, a, w); }

int oracle_test_integrators(int n, double a, double b, int eval, double atol, double rtol, int log_mesh,
                            double* out) {
    std::vector<double> t1(n, 0.0), t2(n), t3(n);
    auto f = [&](double* bb, double x, double dx) {
        for (int i = 0; i < n; ++i) bb[i] += dx * std::pow(x, (double)(i + 1)) * std::exp(-x * x) * std::sin(2.0 * kPi * x);
    };
    if (log_mesh) integrate_log(f, t1.data(), t2.data(), t3.data(), n, a, b, eval, atol, rtol, 1.0);
    else integrate_lin(f, t1.data(), t2.data(), t3.data(), n, a, b, eval, atol, rtol);
    for (int i = 0; i < n; ++i) out[i] = t1[i];
    return 0;
}

double oracle_test_hcubature(int which, double x0, double x1, double y0, double y1, double atol, double rtol) {
    auto f = [&](double x, double y) {
        if (which == 0) return std::exp(-x * x - 2.0 * y * y) * std::cos(3.0 * x * y);
        return 1.0 / std::sqrt(x * x + y * y + 1e-3);
    };
    const double xmin[2] = {x0, y0}, xmax[2] = {x1, y1};
    return hcubature2(f, xmin, xmax, atol, rtol, 10000000LL);
}

double oracle_test_quadgk(int power, double a, double b, double atol, double rtol) {
    auto f = [&](double x) { return std::pow(x, (double)power) * std::exp(-x * x) * std::sin(2.0 * kPi * x); };
    return quadgk(f, {a, b}, atol, rtol);
}

}  // extern "C"

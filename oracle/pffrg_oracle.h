/*
 * CPU FP64 restatement of the PFFRGSolver.jl flow right-hand side.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle and the timed
 * CPU baseline; only tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * may load it.  The product path (libpffrg_gpu.so) never links or calls it.
 *
 * Memory layout of an Action (SU(2): ncomp = 2) in one contiguous FP64 buffer,
 * each array in Julia column-major order (site index fastest), exactly the
 * order of the reference's arrays (src/Action/channel.jl:26-29,
 * src/Action/vertex.jl:10-15, src/Action/action_lib/action_su2.jl:8-12):
 *
 *   Sigma[Nsig]
 *   for comp c: bare[Ns]
 *               for channel in (s, t, u):
 *                   q1[Ns,NO]  q2_1[Ns,NO,Nnu]  q2_2[Ns,NO,Nnu]  q3[Ns,NO,Nnu,Nnu]
 *
 * Lattice index tables are passed 1-based, as the reference stores them.
 */
#ifndef PFFRG_ORACLE_H
#define PFFRG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_problem {
    /* lattice (src/Lattice/reduced.jl:13-24) */
    int64_t num_sites;
    const int64_t* exchange;        /* [Ns]   1-based */
    const int64_t* mult;            /* [Ns] */
    const int64_t* overlap_offsets; /* [Ns+1] row offsets into overlap_rows */
    const int64_t* overlap_rows;    /* [R*3]  (site a, site b, multiplicity), 1-based */
    /* meshes (src/Frequency/mesh.jl:16-27); num_* are array lengths */
    int64_t num_sigma, num_omega, num_nu;
    const double* sigma;
    const double* omega_s;
    const double* nu_s;
    const double* omega_t;
    const double* nu_t;
    /* model */
    int32_t symmetry; /* 0 = su2 */
    double S;
    int32_t num_threads; /* <= 0: all available */
    int32_t task_stride; /* > 1: run only every task_stride-th channel task of a pass (timing samples) */
} oracle_problem;

/* statistics of the last call on this thread */
typedef struct oracle_stats {
    int64_t integrand_evals;  /* bubble integrand evaluations (incl. boundary nodes) */
    int64_t gathered_values;  /* vertex values read by the interpolation (corners x sites) */
    int64_t overlap_terms;    /* t-channel overlap products */
    int64_t sigma_evals;      /* self-energy kernel evaluations */
    int64_t reevals;          /* integrand evaluations of residual! at nodes evaluated before */
    int64_t level_hist[24];   /* Simpson subdomains by final refinement level (n = 2^level new nodes) */
} oracle_stats;

int64_t oracle_action_size(const oracle_problem* p);

/* corrs[2,3,NO] column-major, kind 0 = Katanin (needs da), 1 = plain */
int oracle_corrs(const oracle_problem* p, int kind, double Lam, const double* a, const double* da,
                 double atol, double rtol, double* corrs);

/* compute_dΣ! (src/Flow/flow_self.jl:2-20): writes da.Σ[2:end] */
int oracle_dsigma(const oracle_problem* p, double Lam, const double* a, double* da,
                  double atol, double rtol);

/* compute_dΓ_{1l,2l,ml}! (src/Flow/compute.jl:57-287).  Scratch actions
 * (da_l, da_c, da_temp, da_sigma) are caller buffers of oracle_action_size.
 * For loops >= 3 with sigma_corr != 0, compute_dΣ_corr! (flow_self.jl:23-51)
 * is applied afterwards as in launcher_ml.jl:94-96. */
int oracle_dgamma(const oracle_problem* p, int loops, double Lam, const double* a, double* da,
                  double* da_l, double* da_c, double* da_temp, double* da_sigma, int eval,
                  double gamma_atol, double gamma_rtol, int sigma_corr, double sigma_atol,
                  double sigma_rtol);

/* parquet: compute_Γ! (compute.jl:2-54) and compute_Σ! (SDE.jl:58-96) */
/* compute_Σ! writes a2's s-channel q1/q2_2 and Σ[2:end] and leaves the plain corrs[2,3,NO]
 * it computed in ``corrs``; compute_Γ! reuses that buffer (parquet.jl:54-68) */
int oracle_bse(const oracle_problem* p, double Lam, const double* a1, double* a2, const double* corrs,
               int eval, double atol, double rtol);
int oracle_sde(const oracle_problem* p, double Lam, const double* a1, double* a2, double* corrs,
               int eval, double gamma_atol, double gamma_rtol, double sigma_atol, double sigma_rtol);

/* compute_χ! (src/Observable/correlation_lib/correlation_su2.jl:58-86): χ[Ns, num_chi] column-major */
int oracle_chi(const oracle_problem* p, double Lam, const double* a, const double* chi_mesh, int num_chi,
               double atol, double rtol, double* chi);

/* symmetrize! and symmetrize_add_to! (action_su2.jl:141-251) */
int oracle_symmetrize(const oracle_problem* p, double* a);
int oracle_symmetrize_add_to(const oracle_problem* p, const double* a_l, double* a);

/* ---- unit-level hooks used by the known-answer tests ---- */
/* get_buffer_{s,t,u} kernel selection (src/Frequency/buffer.jl:51-199); ch 1,2,3 */
int oracle_buffer_kernel(const oracle_problem* p, int ch, double w, double v, double vp);
/* interpolated vertex component on all sites, as get_Γ_comp_avx! (Action.jl:110-167) with
 * all three channels enabled; out[Ns] */
int oracle_gamma_comp(const oracle_problem* p, const double* a, int comp, double ws, double vs,
                      double vsp, double wt, double vt, double vtp, double wu, double vu, double vup,
                      int ch_mask, double* out);
/* single-channel read-out as get_vertex_avx! (vertex.jl:63-82), no flags */
int oracle_vertex_channel(const oracle_problem* p, const double* a, int comp, int ch, double w,
                          double v, double vp, double* out);
double oracle_get_sigma(const oracle_problem* p, const double* a, double w);
/* integrate_lin!/integrate_log! (quadrature.jl:84-139) on the reference test kernel
 * b[i] += dx * x^i exp(-x^2) sin(2 pi x), i = 1..n (src/Flow/test.jl:1-13) */
int oracle_test_integrators(int n, double a, double b, int eval, double atol, double rtol,
                            int log_mesh, double* out);
/* the 2-D h-adaptive cubature on a test integrand: 0 = exp(-x^2-2y^2) cos(3xy), 1 = 1/sqrt(x^2+y^2+1e-3) */
double oracle_test_hcubature(int which, double x0, double x1, double y0, double y1, double atol, double rtol);
/* QuadGK-equivalent scalar integral of the same test function, i = power */
double oracle_test_quadgk(int power, double a, double b, double atol, double rtol);

void oracle_last_stats(oracle_stats* out);

#ifdef __cplusplus
}
#endif

#endif

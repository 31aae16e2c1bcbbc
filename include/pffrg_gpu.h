/*
 * libpffrg_gpu: GB300 (sm_103a) flow right-hand side of the pseudo-fermion
 * functional renormalisation group, as a C ABI for the host code of
 * PFFRGSolver.jl (Julia ccall) or any other host language.
 *
 * Data ownership follows the reference: the caller owns every host array
 * (Julia Vector/Array{Float64}, column-major, site index fastest) and the
 * output arrays are overwritten in place.  Index tables are passed 1-based
 * exactly as the reference stores them.  A context owns all device memory
 * (device-resident actions and scratch) and its CUDA streams (one, plus a
 * second one that the χ calls use for their largest integrals); calls on one
 * context are synchronous on return and must come from one host thread at a
 * time; separate contexts are independent.
 *
 * Errors: every int-returning entry point returns 0 on success and a
 * PFFRG_E_* code otherwise; pffrg_last_error() gives the message.  (The
 * reference raises Julia AssertionErrors; a Julia shim turns a nonzero code
 * into error(pffrg_last_error(ctx)).)  There is no CPU fallback: without a
 * usable CUDA device pffrg_create() returns NULL and
 * pffrg_last_error(NULL) says why.
 */
#ifndef PFFRG_GPU_H
#define PFFRG_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFFRG_OK 0
#define PFFRG_E_ARGS 1     /* bad dimensions / arguments (reference: @assert) */
#define PFFRG_E_CUDA 2     /* CUDA runtime error */
#define PFFRG_E_LIMIT 3    /* a fixed capacity was exceeded (mesh length, sites, GK segments) */
#define PFFRG_E_NONFINITE 4

#define PFFRG_FP64 0       /* FP64 integrand (the comparator path) */
#define PFFRG_MIXED 1      /* FP32 integrand + compensated sums, FP64 quadrature bookkeeping */

#define PFFRG_SU2 0
#define PFFRG_U1_DM 1

typedef struct pffrg_ctx pffrg_ctx;

/* Reduced_lattice tables (src/Lattice/reduced.jl:13-24). overlap_rows holds
 * the rows of r.overlap[i] (a, b, multiplicity) for i = 1..Ns back to back,
 * overlap_offsets[i] the first row of site i (offsets[Ns] = total rows). */
typedef struct pffrg_lattice_view {
    int64_t num_sites;
    const int64_t* exchange;        /* [Ns], 1-based */
    const int64_t* mult;            /* [Ns] */
    const int64_t* overlap_offsets; /* [Ns+1] */
    const int64_t* overlap_rows;    /* [3*R], 1-based site indices */
} pffrg_lattice_view;

/* Mesh (src/Frequency/mesh.jl:16-27); num_* are the array lengths. */
typedef struct pffrg_mesh_view {
    int64_t num_sigma, num_omega, num_nu;
    const double* sigma;
    const double* omega_s;
    const double* nu_s;
    const double* omega_t;
    const double* nu_t;
} pffrg_mesh_view;

/* Action_su2 / Action_u1_dm (src/Action/action_lib/action_su2.jl:8-12):
 * a.Σ, a.Γ[c].bare and a.Γ[c].ch_{s,t,u}.{q1,q2_1,q2_2,q3}; channel index
 * 0 = s, 1 = t, 2 = u; components 0..1 (su2) or 0..5 (u1-dm).  The pointers
 * may alias one packed buffer (then a single copy moves the whole action). */
typedef struct pffrg_action_view {
    double* sigma;
    double* bare[6];
    double* q1[6][3];
    double* q2_1[6][3];
    double* q2_2[6][3];
    double* q3[6][3];
} pffrg_action_view;

/* Create a context for one lattice / mesh size / symmetry.  Replaces the
 * set-up of compute buffers in launch_1l!/2l!/ml! (src/Launcher/launcher_1l.jl:37-54).
 * device: CUDA device ordinal.  precision: PFFRG_FP64 or PFFRG_MIXED. */
pffrg_ctx* pffrg_create(const pffrg_lattice_view* lattice, const pffrg_mesh_view* mesh, int symmetry, double S,
                        int precision, int device);
void pffrg_destroy(pffrg_ctx* ctx);
const char* pffrg_last_error(const pffrg_ctx* ctx);

/* New frequency meshes after every accepted ODE step (resample_from_to,
 * src/Action/Action.jl:451-527; launcher_1l.jl:177); sizes must not change. */
int pffrg_set_mesh(pffrg_ctx* ctx, const pffrg_mesh_view* mesh);
int pffrg_set_precision(pffrg_ctx* ctx, int precision);

/* compute_dΣ!(Λ, r, m, a, da, Σ_tol) (src/Flow/flow_self.jl:2-20): writes da.Σ[2:end]. */
int pffrg_dsigma(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a, pffrg_action_view* da, double atol,
                 double rtol);

/* compute_dΓ_1l!/2l!/ml! (src/Flow/compute.jl:57-287) for loops = 1, 2, >= 3.
 * da.Σ must already hold compute_dΣ!'s result (the Katanin propagator reads it).
 * Writes every vertex entry of da (bare untouched).  For loops >= 3 and
 * sigma_corr != 0 also applies compute_dΣ_corr! (flow_self.jl:23-51) to
 * da.Σ, as launcher_ml.jl:95 does.  The scratch actions da_l, da_c, da_temp,
 * da_Σ of the reference live on the device inside the context. */
int pffrg_dgamma(pffrg_ctx* ctx, int loops, double Lam, const pffrg_action_view* a, pffrg_action_view* da,
                 int eval, double gamma_atol, double gamma_rtol, int sigma_corr, double sigma_atol,
                 double sigma_rtol);

/* Parquet iteration kernels (src/Launcher/parquet.jl:43-80):
 * compute_Σ!(Λ, r, m, a1, a2, ...) (src/Flow/SDE.jl:58-96) writes a2's
 * s-channel q1/q2_2 and a2.Σ[2:end]; compute_Γ!(Λ, r, m, a1, a2, ...)
 * (src/Flow/compute.jl:2-54) writes a2's vertex, reusing the boundary
 * corrections of the last pffrg_sde call on this context, as the reference
 * reuses its corrs buffer. */
int pffrg_sde(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a1, pffrg_action_view* a2, int eval,
              double gamma_atol, double gamma_rtol, double sigma_atol, double sigma_rtol);
int pffrg_bse(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a1, pffrg_action_view* a2, int eval,
              double atol, double rtol);

/* The parquet fixed point of launch_parquet! (src/Launcher/parquet.jl:43-80)
 * on the device: the action in slot A is the starting vertex and is replaced
 * by the iterate; every iteration converges the SDE (compute_Σ!, damped
 * Σ update, Σ errors), evaluates the BSEs (compute_Γ!), takes the residual
 * abs = max|ap.q3 - a.q3|, rel = abs / max(max|a.q3|, max|ap.q3|) and damps
 * a = (1 - beta) a + beta ap on the vertex, until abs < tol_abs or
 * rel < tol_rel or max_iter iterations (the reference's beta is min(Λ, 1)).
 * Slots DA and ERR are overwritten.  The actions stay on the device; only the
 * three error norms of an iteration are read back to steer the loop.  Returns
 * the iterations run and the last residuals; residuals (NULL or max_iter
 * entries) receives the absolute residual of every iteration. */
int pffrg_parquet(pffrg_ctx* ctx, double Lam, int eval, double gamma_atol, double gamma_rtol, double sigma_atol,
                  double sigma_rtol, double tol_abs, double tol_rel, double beta, int max_iter, int* iterations,
                  double* abs_err, double* rel_err, double* residuals);

/* ---- device-resident interface (no host copies inside the step) ---- */

/* Number of doubles of one packed action (Σ, then per component bare and
 * ch_s, ch_t, ch_u each as q1, q2_1, q2_2, q3, all column-major). */
int64_t pffrg_action_size(const pffrg_ctx* ctx);

/* Device-resident action slots owned by the context. */
#define PFFRG_SLOT_A 0       /* state a */
#define PFFRG_SLOT_DA 1      /* derivative / stage result */
#define PFFRG_SLOT_INTER 2   /* a_inter of the ODE step */
#define PFFRG_SLOT_ERR 3     /* a_err of the ODE step */
#define PFFRG_SLOT_NEXT 4    /* da of the ODE step (the 3rd-order solution) */
#define PFFRG_NUM_SLOTS 5
int pffrg_upload(pffrg_ctx* ctx, int slot, const pffrg_action_view* a);
int pffrg_download(pffrg_ctx* ctx, int slot, pffrg_action_view* a);

/* One full RHS on device slots: compute_dΣ! then compute_dΓ_*! (and
 * compute_dΣ_corr! for loops >= 3 when sigma_corr != 0). */
int pffrg_rhs(pffrg_ctx* ctx, int loops, double Lam, int a_slot, int da_slot, int eval, double gamma_atol,
              double gamma_rtol, double sigma_atol, double sigma_rtol, int sigma_corr);

/* One Bogacki-Shampine step of launch_1l!/2l!/ml! (src/Launcher/launcher_1l.jl:80-116)
 * on the device from slot A at cutoff Lam with step dLam: leaves the
 * 3rd-order solution in PFFRG_SLOT_NEXT (the reference's a_inter after k4)
 * and returns the error ratio err = max|a_err| / (atol + max(|a_next|,|a|) rtol)
 * and max|q3| of the new solution. */
int pffrg_bs_step(pffrg_ctx* ctx, int loops, double Lam, double dLam, int eval, double gamma_atol,
                  double gamma_rtol, double sigma_atol, double sigma_rtol, int sigma_corr, double ode_atol,
                  double ode_rtol, double* err, double* abs_max_next);
/* accept the step: slot A <- slot NEXT (the reference keeps a_inter for the resampling) */
int pffrg_accept(pffrg_ctx* ctx);

/* Mesh scanning and resampling between accepted steps (resample_from_to,
 * src/Action/Action.jl:483-557) without a host copy of the action.
 * pffrg_scan_cuts returns what the scans of Action.jl:361-480 read: Σ of the
 * slot (sigma[num_sigma]), for every component c and channel ch (index
 * 3 c + ch) the 0-based column-major index of max |q3| (argmax[3 C]; first of
 * equal maxima) and the cuts through it (cuts[3 C][num_omega + 3 num_nu]:
 * q3[s,:,v,v'], q3[s,w,k,k] - q3[s,w,end,end], q3[s,w,:,v'] - q3[s,w,end,v'],
 * q3[s,w,v,:] - q3[s,w,v,end]).  pffrg_resample interpolates the action in
 * src_slot (on the context's meshes) onto `mesh` into dst_slot (get_Σ for Σ,
 * the multilinear read-out of channel.jl:416-471 for every q, bare copied) and
 * makes `mesh` the context's meshes. */
int pffrg_scan_cuts(pffrg_ctx* ctx, int slot, double* sigma, int64_t* argmax, double* cuts);
int pffrg_resample(pffrg_ctx* ctx, int src_slot, int dst_slot, const pffrg_mesh_view* mesh);

/* Quadrature levels driven by the device (default 1): the passes read their work
 * counts on the device and need no host round trip per level, so a whole
 * right-hand side is one asynchronous launch sequence; 0 selects the
 * host-driven loop (host reads the level's counts and stops at the last
 * level).  Both give identical results.  No counterpart in the reference. */
int pffrg_set_async_waves(pffrg_ctx* ctx, int on);

/* Team shape of the quadrature passes: `lanes` threads share a batch of nodes
 * and each holds `sites_per_lane` sites (built: 8x1, 16x1, 16x3, 16x4, 32x1,
 * 32x2, 32x3, 32x4, 32x8; 0x0 = chosen from the number of sites).  A shape that
 * does not cover the sites is ignored.  Results agree to rounding (the
 * t-channel overlap sums are split over the lanes differently).  No
 * counterpart in the reference. */
int pffrg_set_team_shape(pffrg_ctx* ctx, int lanes, int sites_per_lane);

/* Autotuner of the team shape: times one right-hand side (as pffrg_rhs on
 * a_slot into da_slot, without Σ corrections) for every built shape that
 * covers the sites with at most twice as many lane slots as sites, keeps the
 * fastest as the context's shape and returns it.  da_slot is overwritten.
 * No counterpart in the reference. */
int pffrg_autotune_team_shape(pffrg_ctx* ctx, int loops, double Lam, int a_slot, int da_slot, int eval,
                              double gamma_atol, double gamma_rtol, double sigma_atol, double sigma_rtol,
                              int* lanes, int* sites_per_lane);

/* Capacities of the context's scratch: chunks of one quadrature level's
 * queue (0: 8 nsub + 65536 for nsub Simpson subdomains, which a call that
 * overflows it repeats with 4x, up to 128 nsub + 65536) and the first segment
 * capacity of each adaptive Gauss-Kronrod integral (0: 2048; otherwise at
 * least 16).  A level that needs more chunks than a set queue returns
 * PFFRG_E_LIMIT; integrals
 * that run out of segments are repeated with 8x the segments, up to the
 * reference's 10^7 evaluations, as always.  For tests of those paths and for
 * callers that bound the context's memory.  No counterpart in the reference. */
int pffrg_set_capacities(pffrg_ctx* ctx, int64_t queue_chunks, int64_t gk_segments);

/* Overlap rows of the t-channel sums (flow_su2_t.jl:66-75): 0 = staged in
 * shared memory when the block's staging still lets the FP32 eval kernel's
 * blocks fit an SM (55 KB for SU(2) teams of up to two sites per lane, 75 KB
 * otherwise; default), 1 =
 * read through L1/L2, 2 = staged whenever they fit the 227 KB of a block.
 * Results agree to rounding.  No counterpart in the reference. */
int pffrg_set_overlap_staging(pffrg_ctx* ctx, int mode);

/* Mixed path: a Simpson subdomain whose convergence test is closer to its
 * bounds than eps (the relative rounding allowed for the FP32 node values)
 * could be decided the other way in FP64; such subdomains are evaluated again
 * in FP64 on the FP64 actions, so every adaptive decision of the mixed path is
 * the FP64 path's and the two differ by FP32 arithmetic only.  Default 1e-6;
 * 0 turns the hand-off off (FP32 decisions).  No counterpart in the reference. */
int pffrg_set_fp64_handoff(pffrg_ctx* ctx, double eps);

/* χ cubature: the passes whose region capacity is at least min_regions
 * (default 32768: the few integrals that approach the evaluation cap) run
 * each integral on a cluster of `blocks` blocks (8 or 16, default 8; a
 * 16-block cluster that does not launch falls back to 8) instead of one
 * block; min_regions 0 = always.  Results are identical.  No counterpart in
 * the reference. */
int pffrg_set_chi_cluster(pffrg_ctx* ctx, int64_t min_regions, int blocks);

/* Precision of the χ integrand of a PFFRG_MIXED context: PFFRG_FP64 (default)
 * or PFFRG_MIXED (FP32 on the FP32 copy of the state with the float-float node
 * setup; about 1.6x faster, but near the 10^7-evaluation cap, where the
 * cubature does not converge, its refinement differs from the FP64 one:
 * 3.7e-6 of max|χ| measured at Λ = 0.15 on square L=3).  The cubature's
 * coordinates, rules and sums are FP64 either way.  No counterpart in the
 * reference. */
int pffrg_set_chi_integrand(pffrg_ctx* ctx, int precision);

/* compute_χ! (src/Observable/correlation_lib/correlation_su2.jl:58-86,
 * correlation_u1_dm.jl:152-190): static spin correlations χ[i, w] of the
 * action `a` at Λ on the frequencies chi_mesh[0..num_chi), written
 * column-major into chi (host): Ns * num_chi values for su2, three such
 * blocks χxx | χzz | χxy for u1-dm.  Tolerances are χ_tol = (atol, rtol)
 * (default (1e-8, 1e-4) in src/Launcher/Launcher.jl:111).  The context
 * remembers each integral's region capacity from its previous χ call with
 * the same number of sites and frequencies and starts there (the results do
 * not depend on it). */
int pffrg_chi(pffrg_ctx* ctx, double Lam, const pffrg_action_view* a, const double* chi_mesh, int num_chi,
              double atol, double rtol, double* chi);
/* the same on the device-resident action in `slot` (the measure step of
 * src/Launcher/launcher_1l.jl:128-145 without a host copy of the state) */
int pffrg_chi_slot(pffrg_ctx* ctx, double Lam, int slot, const double* chi_mesh, int num_chi, double atol,
                   double rtol, double* chi);

/* Integrand evaluations of the last pffrg_rhs / pffrg_dgamma (dΓ passes only),
 * for throughput and algorithmic-byte accounting. */
int64_t pffrg_last_integrand_evals(const pffrg_ctx* ctx);

/* Work counters and optional CUDA-event timing (recorded on the context's stream). */
typedef struct pffrg_stats {
    int64_t integrand_evals;    /* bubble integrand evaluations of the last RHS / dΓ call */
    int64_t algorithmic_values; /* vertex values those evaluations read (corners x sites x components,
                                   bare and output values, t-channel overlap operands) */
    double pass_ms;             /* summed duration of the channel-task kernels since the last reset */
    double rhs_ms;              /* summed duration of pffrg_rhs calls since the last reset */
    int64_t pass_launches;      /* channel-task passes (each a sequence of level kernels) since the last reset */
    int64_t launches;           /* kernels this library launched since the last reset */
    int64_t chi_evals;          /* χ integrand evaluations (cubature points) of the last pffrg_chi call */
    int64_t chi_regions_max;    /* largest region count of one χ integral in that call */
    int64_t chi_rounds;         /* refinement rounds of all χ integrals in that call */
    int64_t chi_rounds_max;     /* most rounds of one χ integral in that call */
} pffrg_stats;
int pffrg_set_timing(pffrg_ctx* ctx, int on);
int pffrg_read_stats(pffrg_ctx* ctx, pffrg_stats* out, int reset);

/* One-loop dΓ without any device allocation.  This entry point has no
 * counterpart in the reference.  It is meant for callers that cannot call
 * cudaMalloc: hosts whose device memory is owned by another framework's pool
 * allocator (a second allocator fragments that pool and can fail under its
 * reservations), and embedders with a device-memory budget fixed at start-up.
 *
 * Computes what pffrg_dgamma(loops = 1) computes in FP64 -- compute_dΓ_1l!'s
 * boundary corrections, the Katanin bubbles of all channel tasks and the
 * symmetrisation -- on packed actions already in device memory: a_dev is the
 * state a, da_dev holds dΣ in its Σ part on entry (from compute_dΣ!) and
 * receives the vertex derivative (bare entries untouched).  lattice and mesh
 * are host views as for pffrg_create.  stream: a cudaStream_t (NULL: legacy
 * default stream).  The call copies its tables from pageable host memory,
 * reads the status of its boundary integrals between kernels and returns
 * after the stream has drained.
 *
 * All scratch (tables, integration bounds, boundary corrections, adaptive
 * quadrature workspace) lives in one static device array of
 * pffrg_noalloc_scratch_bytes() = 128 MiB that every GPU loading this library
 * holds until the process exits.  Problems needing more return PFFRG_E_LIMIT
 * with the required size in pffrg_noalloc_last_error() (square L = 3 with the
 * 50/15/10 default-size meshes at eval <= 10 fits); so do a level of the
 * adaptive quadrature with more chunks than the array's queue (2 nsub + 4096
 * for nsub Simpson subdomains, a quarter of the regular path's) and boundary
 * integrals that need more than 2048 Gauss-Kronrod segments (the regular entry
 * points grow their buffers and repeat instead).  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress); make that first
 * call before capturing a stream.  Every call reuses the same array, so calls
 * whose GPU work overlaps (other streams, other host threads) race and must be
 * serialised by the caller. */
int pffrg_dgamma_1l_noalloc(const pffrg_lattice_view* lattice, const pffrg_mesh_view* mesh, double S, double Lam,
                            const double* a_dev, double* da_dev, int eval, double atol, double rtol, void* stream);
int64_t pffrg_noalloc_scratch_bytes(void);
const char* pffrg_noalloc_last_error(void);

/* Pinned host memory for fast copies (cudaHostAlloc); NULL on failure. */
void* pffrg_host_alloc(int64_t bytes);
void pffrg_host_free(void* p);

/* Learned parquet warm start.  No counterpart in the reference: a multilayer
 * perceptron (dense layers, tanh on all but the last, FP32) maps a model's
 * couplings to the principal-component coordinates of its converged parquet
 * vertex; a fixed affine decoder (basis[k][d], mean[d]) turns them into the
 * vertex that starts the parquet iteration of src/Launcher/parquet.jl, which
 * stays the judge of convergence.  sizes[0..nlayers] are the layer widths;
 * parameters are stored layer by layer as W[n_in][n_out] then b[n_out].
 * Training minimises the mean squared error over the whole batch with Adam. */
typedef struct pffrg_mlp pffrg_mlp;
pffrg_mlp* pffrg_mlp_create(int nlayers, const int* sizes, unsigned seed);
void pffrg_mlp_destroy(pffrg_mlp* net);
const char* pffrg_mlp_last_error(const pffrg_mlp* net);
int64_t pffrg_mlp_num_params(const pffrg_mlp* net);
int pffrg_mlp_get_params(pffrg_mlp* net, float* params);
int pffrg_mlp_set_params(pffrg_mlp* net, const float* params);
int pffrg_mlp_forward(pffrg_mlp* net, const float* x, int batch, float* y);
int pffrg_mlp_gradient(pffrg_mlp* net, const float* x, const float* target, int batch, float* grads, float* loss);
int pffrg_mlp_train(pffrg_mlp* net, const float* x, const float* target, int batch, int epochs, float lr,
                    float* loss);
int pffrg_mlp_set_decoder(pffrg_mlp* net, const float* basis, const float* mean, int k, int64_t d);
int pffrg_mlp_predict(pffrg_mlp* net, const float* x, float* out);

#ifdef __cplusplus
}
#endif

#endif

/*
 * r2d3c.h -- C-ABI of the GB300 (sm_103a) Rot2D3C time-step hot path.
 *
 * The reference (Fortran 90, MPI, FFTW 2) has no plugin system: its operator
 * interface is the set of subroutines its main program calls.  Every entry
 * point below names the reference routine it replaces (file:line, paths
 * relative to the reference's src/).  A Fortran caller binds them with
 * ISO_C_BINDING interface blocks; a Python caller with ctypes.
 *
 * Conventions
 *   - Every function returns an int status: R2D3C_OK (0) or a negative code.
 *     No exception or abort crosses the ABI.  r2d3c_last_error() gives text.
 *   - Host buffers are caller-owned FP64 arrays in the reference's Fortran
 *     layouts and are complete when the call returns:
 *       spectral  C(n, n/2+1) complex*16, ky fastest  -> 2*n*(n/2+1) doubles,
 *                 interleaved (re, im) (fftp2D.f90:153)
 *       physical  R(n, n) real*8, x fastest           -> n*n doubles
 *                 (fftp2D.f90:157)
 *   - A context owns all device memory and one private CUDA stream.  It is
 *     not thread-safe: use one context per host thread.  Distinct contexts may
 *     run concurrently.
 *   - Transforms are unnormalised with forward sign -1; a C2R(R2C(x)) round
 *     trip returns n*n*x; C2R ignores Im at kx = 0 and kx = n/2 (FFTW).
 *   - Supported grids: n = 16, 32, ..., 8192 (powers of two).
 *   - Precision: R2D3C_FP64 computes everything in FP64 (the drop-in path);
 *     R2D3C_FP32 keeps the fields and transforms in FP32 (compensated
 *     twiddles) and every diagnostic reduction in FP64.
 */
#ifndef R2D3C_H
#define R2D3C_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  R2D3C_OK = 0,
  R2D3C_EINVAL = -1,   /* bad argument */
  R2D3C_ECUDA = -2,    /* CUDA runtime error */
  R2D3C_ENOMEM = -3,   /* device allocation failed */
  R2D3C_ETIMEOUT = -4, /* a bounded device wait gave up */
  R2D3C_EIO = -5,      /* file input/output error */
  R2D3C_ESTATE = -6    /* call not valid in the current state */
};

enum { R2D3C_FP64 = 0, R2D3C_FP32 = 1 };

/* FFT directions: FFTW_REAL_TO_COMPLEX (-1), FFTW_COMPLEX_TO_REAL (+1)
   (fftw_f77.i:10-11). */
enum { R2D3C_R2C = -1, R2D3C_C2R = 1 };

/* time-step selection for r2d3c_advance */
enum { R2D3C_DT_CFL = 0, R2D3C_DT_FIXED = 1 };

/* field selection for r2d3c_get_field (Rot2D3C.para.f90:476-519) */
enum { R2D3C_FIELD_PS = 0, R2D3C_FIELD_VZ = 1, R2D3C_FIELD_WW = 2, R2D3C_FIELD_INVLAP_PSI = 3 };

/* The 25 positional values of parameter.inp (read at Rot2D3C.para.f90:136-160)
   plus the grid size n (compile-time module grid in the reference,
   pseudospec2D_mod.f90:7-14; a run-time value here). */
typedef struct r2d3c_params {
  int n;
  double cfl;      /*  1 (commented "dt" in parameter.inp, read as CFL) */
  int step;        /*  2 */
  int cstep;       /*  3 */
  int sstep;       /*  4 */
  int tstep;       /*  5 */
  double fp0;      /*  6 */
  double fz0;      /*  7 */
  double u0;       /*  8 */
  double v0;       /*  9 */
  double kdn;      /* 10 */
  double kup;      /* 11 */
  double nu;       /* 12 */
  double hnu;      /* 13 */
  int nn;          /* 14 */
  int mm;          /* 15 */
  double nuv;      /* 16 */
  double hnuv;     /* 17 */
  int nnv;         /* 18 */
  int mmv;         /* 19 */
  double omega;    /* 20 */
  int seed;        /* 21 */
  int iflow;       /* 22 */
  double prm1;     /* 23 (unused by the reference) */
  double prm2;     /* 24 (unused by the reference) */
  double dt_corr;  /* 25 (unused by the reference) */
} r2d3c_params;

typedef struct r2d3c_ctx r2d3c_ctx;
typedef struct r2d3c_plan r2d3c_plan;

/* ---- library ---------------------------------------------------------- */
const char* r2d3c_version(void);
/* Text of the last error of any call on this host thread. */
const char* r2d3c_last_error(void);
/* Number of this library's kernels launched so far on this context. */
int r2d3c_kernel_launches(const r2d3c_ctx* ctx, long long* count);

/* ---- Level 1: layout-compatible 2-D FFT (fftp2D.f90) ------------------ */
/* replaces fftp2d_create_plan (fftp2D.f90:30-63); flags (FFTW_ESTIMATE /
   FFTW_MEASURE) are accepted and ignored. */
int r2d3c_fft_plan_create(int n, int dir, int flags, int precision, r2d3c_plan** plan);
/* replaces fftp2d_destroy_plan (fftp2D.f90:66-86) */
int r2d3c_fft_plan_destroy(r2d3c_plan* plan);
/* replaces fftp2d_real_to_complex (fftp2D.f90:133-211): in R(n,n) -> out C(n,n/2+1) */
int r2d3c_fft_r2c(r2d3c_plan* plan, const double* in, double* out);
/* replaces fftp2d_complex_to_real (fftp2D.f90:214-290): in C(n,n/2+1) -> out R(n,n).
   The reference destroys its input; this one leaves it unchanged. */
int r2d3c_fft_c2r(r2d3c_plan* plan, double* in, double* out);
/* Same transforms on device FP64 buffers (same layouts) on `stream`
   (a cudaStream_t, or NULL for the plan's stream); asynchronous. */
int r2d3c_fft_r2c_dev(r2d3c_plan* plan, const double* d_in, double* d_out, void* stream);
int r2d3c_fft_c2r_dev(r2d3c_plan* plan, const double* d_in, double* d_out, void* stream);

/* ---- Level 2: the hot path -------------------------------------------- */
/* Module state of the reference main program (Rot2D3C.para.f90:102-238):
   wavenumbers, dealiasing bounds, plans and the state/forcing/work arrays. */
int r2d3c_create(const r2d3c_params* params, int precision, r2d3c_ctx** ctx);
int r2d3c_destroy(r2d3c_ctx* ctx);
/* Bytes of device memory held by the context. */
int r2d3c_device_bytes(const r2d3c_ctx* ctx, long long* bytes);

/* State psi^, vz^ (spectral).  set_state marks the state "not truncated":
   the next step applies the 2/3 truncation as the reference's first RK step
   does (Rot2D3C.para.f90:578-611). */
int r2d3c_set_state(r2d3c_ctx* ctx, const double* ps_hat, const double* vz_hat);
int r2d3c_get_state(r2d3c_ctx* ctx, double* ps_hat, double* vz_hat);
/* Restart path (Rot2D3C.para.f90:322-329): physical psi, vz -> R2C, no mask. */
int r2d3c_set_state_physical(r2d3c_ctx* ctx, const double* ps, const double* vz);
/* Forcing fp^, fz^ (spectral). */
int r2d3c_set_forcing(r2d3c_ctx* ctx, const double* fp_hat, const double* fz_hat);
int r2d3c_get_forcing(r2d3c_ctx* ctx, double* fp_hat, double* fz_hat);

/* Seeded initial condition, stat == 0 branch (Rot2D3C.para.f90:245-299).
   *seed is advanced exactly as the reference's randu calls advance it. */
int r2d3c_initial_conditions(r2d3c_ctx* ctx, int* seed);
/* Forcing set-up before the loop by iflow (Rot2D3C.para.f90:343-381):
   iflow 1 deterministic, 2 const_inj, 3 CFL + rand_force.  Seeds advance as
   in the reference; *seed1 receives seed+1 (and its advanced value). */
int r2d3c_forcing_init(r2d3c_ctx* ctx, int* seed, int* seed1);

/* replaces CFL_condition (pseudospec2D_Rot2D3C.f90:840-899) */
int r2d3c_cfl(r2d3c_ctx* ctx, double cfl, double* dt);
/* replaces the two rand_force calls of one step (Rot2D3C.para.f90:413-416,
   pseudospec2D_Rot2D3C.f90:1063-1126) with the given dt */
int r2d3c_force_random(r2d3c_ctx* ctx, double dt, int* seed, int* seed1);
/* One RK step of order 4 (Rot2D3C.para.f90:545-611) with the given dt.
   For iflow == 2 the forcing is rebuilt by const_inj at every substep
   (:565-569) and *seed, *seed1 advance as in the reference. */
int r2d3c_step(r2d3c_ctx* ctx, double dt, int* seed, int* seed1);
/* nsteps iterations of the main loop body without diagnostics
   (Rot2D3C.para.f90:399, :413-416, :537, :545-611): dt from the CFL condition
   (dt_mode R2D3C_DT_CFL, cfl_or_dt = CFL factor) or fixed (R2D3C_DT_FIXED),
   rand_force every step when iflow == 3, time += dt.  One step is captured in
   a CUDA graph and replayed.  On return *time and *dt_last hold the device
   values (either may be NULL). */
int r2d3c_advance(r2d3c_ctx* ctx, int nsteps, int dt_mode, double cfl_or_dt, double* time,
                  double* dt_last, int* seed, int* seed1);
int r2d3c_set_time(r2d3c_ctx* ctx, double time);

/* replaces cond_check (pseudospec2D_Rot2D3C.f90:455-612): the 30 values the
   reference appends to energy_bal.txt (12), enstrophy_bal.txt (5),
   helicity_bal.txt (8) and max_min.txt (5), in file order. */
int r2d3c_cond_check(r2d3c_ctx* ctx, double time, double out[30]);
/* replaces spectrum (:615-712): Ek, Ezk with n/2+1 shells each */
int r2d3c_spectrum(r2d3c_ctx* ctx, double* Ek, double* Ezk);
/* replaces transfers (:715-837): per-shell Fl0, Fl1, Fl2 (n/2+1 each);
   fluxes are their running sums (:824-830) */
int r2d3c_transfers(r2d3c_ctx* ctx, double* Fl0, double* Fl1, double* Fl2);
/* Field output of Rot2D3C.para.f90:476-519 (ps, vz, ww, invlap_psi), each
   scaled by 1/n^2 before the C2R, as R(n,n). */
int r2d3c_get_field(r2d3c_ctx* ctx, int which, double* R);

/* ---- Ensembles of independent runs ------------------------------------- */
/* No counterpart in the reference (it runs one field per MPI job).  Several
   runs of possibly different sizes advance together: runs of the same n are
   batched into the same kernel launches (one CTA row per run), and one step
   of every size group is captured in one CUDA graph with the groups on
   parallel streams.  Each run has its own parameters (n, nu, Omega, ...),
   state, forcing (held constant, iflow 0/1 semantics), dt and time.  Runs
   are numbered group by group in the order given. */
typedef struct r2d3c_ensemble r2d3c_ensemble;
/* ngroups size groups; group g has runs[g] runs of grid n[g]; params holds
   one r2d3c_params per run (params[r].n must equal its group's n). */
int r2d3c_ensemble_create(int ngroups, const int* n, const int* runs, const r2d3c_params* params,
                          int precision, r2d3c_ensemble** ens);
int r2d3c_ensemble_destroy(r2d3c_ensemble* ens);
int r2d3c_ensemble_set_state(r2d3c_ensemble* ens, int run, const double* ps_hat, const double* vz_hat);
int r2d3c_ensemble_get_state(r2d3c_ensemble* ens, int run, double* ps_hat, double* vz_hat);
int r2d3c_ensemble_set_forcing(r2d3c_ensemble* ens, int run, const double* fp_hat, const double* fz_hat);
/* nsteps steps of every run (dt per run from its CFL condition, or fixed);
   times (may be NULL) receives each run's time. */
int r2d3c_ensemble_advance(r2d3c_ensemble* ens, int nsteps, int dt_mode, double cfl_or_dt, double* times);
int r2d3c_ensemble_set_time(r2d3c_ensemble* ens, int run, double time);
/* cond_check / spectrum of one run (as r2d3c_cond_check, r2d3c_spectrum) */
int r2d3c_ensemble_cond_check(r2d3c_ensemble* ens, int run, double time, double out[30]);
int r2d3c_ensemble_spectrum(r2d3c_ensemble* ens, int run, double* Ek, double* Ezk);
int r2d3c_ensemble_kernel_launches(const r2d3c_ensemble* ens, long long* count);
/* The plan of every size group (as r2d3c_plan_report): JSON list of
   {"n", "runs", "plan"} objects, NUL-terminated in buf. */
int r2d3c_ensemble_plan_report(const r2d3c_ensemble* ens, char* buf, int len);

/* ---- Learned subgrid closure (no counterpart in the reference) --------- */
/* A periodic CNN of six 3x3 convolutions, 8 -> 32 -> 32 -> 32 -> 32 -> 32 -> 2
   channels with GELU between layers, BF16 operands and FP32 accumulation on
   the tensor cores, FP32 master parameters trained with Adam.  Tensors are
   device FP32 NHWC arrays on an H x W periodic grid (H % 8 == 0,
   W % 16 == 0): inputs [batch][H][W][8], outputs/targets [batch][H][W][2].
   The parameter vector is layer by layer: weights [9][cin][cout] (tap =
   3*dy + dx, input pixel (y+dy-1, x+dx-1)) then biases [cout]. */
typedef struct r2d3c_cnn r2d3c_cnn;
int r2d3c_cnn_create(int H, int W, int max_batch, int seed, r2d3c_cnn** cnn);
int r2d3c_cnn_destroy(r2d3c_cnn* cnn);
int r2d3c_cnn_num_params(const r2d3c_cnn* cnn, long long* n);
int r2d3c_cnn_get_params(r2d3c_cnn* cnn, float* host);
int r2d3c_cnn_set_params(r2d3c_cnn* cnn, const float* host);
int r2d3c_cnn_forward(r2d3c_cnn* cnn, const float* d_x, int batch, float* d_out);
/* loss = mean squared error over all outputs; host_grad (may be NULL)
   receives dloss/dparams */
int r2d3c_cnn_gradients(r2d3c_cnn* cnn, const float* d_x, const float* d_y, int batch, float* host_grad,
                        double* loss);
/* Vector-Jacobian product at the inputs d_x: given d_gout = dL/d(output)
   ([batch][H][W][2], physical output units), d_gx (may be NULL) receives
   dL/dx ([batch][H][W][8]) and host_grad (may be NULL) dL/dparams.  The
   forward pass is recomputed inside, so the call needs nothing kept from an
   earlier forward; operands are BF16 as in training.  Synchronous on
   return.  For autograd bindings (rot2d3c_gb300/torch_ops.py). */
int r2d3c_cnn_backward(r2d3c_cnn* cnn, const float* d_x, const float* d_gout, int batch, float* d_gx,
                       float* host_grad);
/* forward, backward and one Adam step (beta 0.9/0.999, eps 1e-8) */
int r2d3c_cnn_train_step(r2d3c_cnn* cnn, const float* d_x, const float* d_y, int batch, float lr, double* loss);
/* per-channel standardisation applied inside the network: inputs are mapped
   to (x - in_mean)/in_std, targets likewise, outputs back to physical units
   (the loss is in standardised units); identity by default */
int r2d3c_cnn_set_normalization(r2d3c_cnn* cnn, const float* in_mean, const float* in_std, const float* out_mean,
                                const float* out_std);
/* Closure data of a coarse run (device FP32 NHWC on its n x n grid): the 8
   network inputs of its current state (omega, vz, d/dx and d/dy of psi,
   omega, vz); a training sample from a finer run -- the coarse state is set
   to the sharp spectral filter (k^2 <= (nc/3)^2) of the fine state and the
   targets are the subgrid parts of the two brackets,
   P_c([psi,-k^2 psi]_fine) - [psi_c,-k^2 psi_c] and P_c([psi,vz]_fine) - [psi_c,vz_c];
   and the tendencies (physical [n][n][2]) that the following steps add to
   the two brackets of the RK update (NULL switches them off). */
int r2d3c_closure_inputs(r2d3c_ctx* ctx, float* d_x);
int r2d3c_closure_sample(r2d3c_ctx* fine, r2d3c_ctx* coarse, float* d_x, float* d_y);
int r2d3c_closure_set_tendency(r2d3c_ctx* ctx, const float* d_t);
/* Per-shell weights of the tendencies: from now on the two tendencies are
   multiplied, in spectral space, on shell b (kmn = int(sqrt(ka2)+.5),
   b < nshells) by w[b] (omega tendency) and w[nshells + b] (vz tendency),
   and by 0 beyond; nshells = 0 switches the weighting off (the default).
   The closure experiment uses it to confine the network's tendencies to
   the shells next to the cutoff, where the subgrid transfer acts.  Host
   array of 2 nshells floats, copied before return (call it outside any
   stream capture).  No counterpart in the reference. */
int r2d3c_closure_set_band(r2d3c_ctx* ctx, const float* w, int nshells);
/* nsteps LES steps with the network in the loop: before every RK step the
   8 inputs of the current state are formed, the network cnn (grid n x n) is
   evaluated on them and its two outputs are added to the brackets of that
   step.  All of it (inputs, network, tendencies, step) is captured as one
   CUDA graph and replayed nsteps times, with dt from the CFL condition or
   fixed as in r2d3c_advance; constant forcing only (iflow 0 or 1).  The
   network's buffers are in use until the call returns; the tendencies are
   switched off on return. */
int r2d3c_closure_advance(r2d3c_ctx* ctx, r2d3c_cnn* cnn, int nsteps, int dt_mode, double cfl_or_dt,
                          double* time, double* dt_last);
/* The same with the network evaluated before every `every`-th step only (its
   tendencies held for `every` steps; one CUDA graph of the evaluation and
   `every` steps); nsteps must be a multiple of every.  every = 1 is
   r2d3c_closure_advance.  No counterpart in the reference. */
int r2d3c_closure_advance_every(r2d3c_ctx* ctx, r2d3c_cnn* cnn, int nsteps, int every, int dt_mode,
                                double cfl_or_dt, double* time, double* dt_last);
/* The same with the network one step behind the solver and running beside
   it: the first step of the call takes the tendencies of its own state;
   step s > 0 takes those of the state before step s - 1, evaluated on a
   second stream while step s - 1 runs (inside the captured graph, joined
   before step s).  The network and the RK step are both latency-bound at
   LES sizes, so the two overlap.  n <= 512, constant forcing.  No
   counterpart in the reference. */
int r2d3c_closure_advance_overlapped(r2d3c_ctx* ctx, r2d3c_cnn* cnn, int nsteps, int dt_mode, double cfl_or_dt,
                                     double* time, double* dt_last);

/* ---- Regridding (regrid_slices.f90) ------------------------------------ */
/* The reference's slice regridder applied to a whole field
   (regrid_slices.f90:95-104): out(j,k) = in((j+1)*n/m, (k+1)*n/m) with
   1-based indices and integer division, in R(n,n), out R(m,m), host FP64
   buffers; n < m <= 2n (the map reads outside the field beyond 2n). */
int r2d3c_regrid_physical(int n, int m, const double* in, double* out);
/* the same on device buffers, queued on `stream` */
int r2d3c_regrid_physical_dev(int n, int m, const double* d_in, double* d_out, void* stream);
/* No reference counterpart: spectral zero-padding of src's state (ps, vz)
   onto the finer grid of dst (modes |kx|,|ky| < n_src/2, scaled by
   (n_dst/n_src)^2 so that the physical fields agree on the common points). */
int r2d3c_regrid_spectral(r2d3c_ctx* src, r2d3c_ctx* dst);

/* ---- Level 2 operators (reference subroutines on host arrays) ---------- */
/* derivk2 (pseudospec2D_Rot2D3C.f90:6-68) */
int r2d3c_derivk2(r2d3c_ctx* ctx, const double* a, double* b, int dir);
/* laplak2 (:71-95) */
int r2d3c_laplak2(r2d3c_ctx* ctx, const double* a, double* b);
/* inv_laplak2 (:98-127) */
int r2d3c_inv_laplak2(r2d3c_ctx* ctx, const double* a, double* b);
/* poisson (:169-226) */
int r2d3c_poisson(r2d3c_ctx* ctx, const double* a, const double* b, double* c);
/* energy (:336-396) */
int r2d3c_energy(r2d3c_ctx* ctx, const double* a, int kin, double* b);
/* inerprod (:400-451) */
int r2d3c_inerprod(r2d3c_ctx* ctx, const double* a, const double* b, int kin, double* rslt);
/* randu (pseudospec2D_mod.f90:52-71): one draw, *seed updated */
float r2d3c_randu(int* seed);

/* ---- allocation-free variant ------------------------------------------- */
/* FP64 complex-to-real 2-D transform on device buffers (same layouts and
   result as r2d3c_fft_c2r_dev) that performs no device allocation.  No
   counterpart in the reference.  For callers that cannot allocate device
   memory (memory owned by another allocator, or no implicit synchronisation
   allowed); its scratch is a fixed file-scope device array, so n <= 512
   (larger n returns R2D3C_EINVAL), all calls on a device share that scratch
   (calls whose GPU work overlaps race), and the first call on each device
   does the set-up, which ends with a device synchronisation (make it before
   any stream capture).  stream may be NULL. */
int r2d3c_fft_c2r_noalloc(int n, const double* d_in, double* d_out, void* stream);

/* ---- measurement ------------------------------------------------------ */
/* Average device time per launch of the three passes of the RK substep
   (ms_per_launch[0] pass A, [1] pass B, [2] pass C, [3] other kernels) over
   nsteps steps with a fixed dt, from CUDA events recorded on the context
   stream around every launch; launches[4] receives the launch counts.
   No counterpart in the reference (it has no timers). */
int r2d3c_profile_passes(r2d3c_ctx* ctx, int nsteps, double dt, double* ms_per_launch,
                         long long* launches);
/* Measured FP64 FMA throughput of the current device in TFLOP/s (dependent
   FMA chains on every SM), the denominator of the FP64 path's roofline.
   No counterpart in the reference. */
int r2d3c_fp64_fma_peak(double* tflops);

/* Device pointer of a context plane for GPU-resident callers:
   which = 0 ps, 1 vz, 2 fp, 3 fz (spectral planes of the context's compute
   type, complex interleaved [kx][ky]). */
int r2d3c_dev_ptr(r2d3c_ctx* ctx, int which, void** ptr);
/* The plan chosen when the context was created (the counterpart of FFTW's
   measured plans, fftp2D.f90:54-56): each launch-schedule variant of the
   derivative pass, the bracket pass and the update pass that computes
   bit-identical results (transform groups per CTA, field chunks, persistent
   CTAs) is timed on this GPU and the fastest kept.  JSON text of the timings
   and the choices, NUL-terminated in buf (R2D3C_EINVAL if len is too
   small). */
int r2d3c_plan_report(r2d3c_ctx* ctx, char* buf, int len);
/* The context's CUDA stream (cudaStream_t). */
int r2d3c_stream(r2d3c_ctx* ctx, void** stream);
/* Block until all queued work of the context is done. */
int r2d3c_synchronize(r2d3c_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* R2D3C_H */

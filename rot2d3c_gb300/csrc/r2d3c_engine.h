// Precision-independent interface between the C-ABI layer and the device
// engine of one context (FP64 or FP32 compute type).  All planes live in
// device memory owned by the engine; all work is queued on the engine's
// stream.  Methods throw r2d3c::Error on CUDA failures; the C-ABI layer turns
// them into status codes.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

namespace r2d3c {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// status codes mirrored from include/r2d3c.h
constexpr int kOK = 0, kEINVAL = -1, kECUDA = -2, kENOMEM = -3, kETIMEOUT = -4, kEIO = -5,
              kESTATE = -6;

void cuda_check(cudaError_t e, const char* what);

// Spectral planes: complex [kx][ky], (n/2+1) x n.
// (C1, C2 and C3, C4: the substep state, ping-ponged between the substeps)
enum Plane : int { P_PS = 0, P_VZ, P_FP, P_FZ, P_C1, P_C2, P_C3, P_C4, P_W1, P_W2, P_B5, P_B6, P_T5, P_T6, P_COUNT };
// Real planes: [y][x], n x n.
enum RPlane : int { R_1 = 0, R_2, R_3, R_COUNT };

struct ModelCoef {
  double nu, hnu, nuv, hnuv, omega;
  int nn, mm, nnv, mmv;
};

struct RandForceHost {  // one field of one rand_force call
  int nset;
  int set[4];
  int conj[4];
  double c0, kpow, cph, sph;
};

struct IcModeHost {
  double kr, ph1, ph2, ph3, ph4;
  int ir, jr;
};

class IEngine {
 public:
  virtual ~IEngine() {}
  virtual int n() const = 0;
  virtual int precision() const = 0;  // 0 = FP64, 1 = FP32
  virtual cudaStream_t stream() const = 0;
  virtual void* plane_ptr(int plane) = 0;
  virtual void* rplane_ptr(int rplane) = 0;
  virtual size_t bytes_allocated() const = 0;

  // host <-> device (FP64 host arrays, synchronous on return)
  virtual void upload_spec(int plane, const double* host) = 0;    // 2*(n/2+1)*n doubles
  virtual void download_spec(int plane, double* host) = 0;
  virtual void upload_real(int rplane, const double* host) = 0;   // n*n doubles
  virtual void download_real(int rplane, double* host) = 0;
  // device FP64 <-> planes (for callers that keep data on the GPU)
  virtual void spec_from_dev64(int plane, const double* dev) = 0;
  virtual void spec_to_dev64(int plane, double* dev) = 0;
  virtual void real_from_dev64(int rplane, const double* dev) = 0;
  virtual void real_to_dev64(int rplane, double* dev) = 0;

  // generic operators
  virtual void specop(int src, int dst, int op, double s) = 0;
  virtual void zero_spec(int plane) = 0;
  virtual void r2c(int rsrc, int dst) = 0;
  virtual void c2r(int src, int rdst, double* mx, double* mn) = 0;  // rdst<0: no store
  virtual void poisson(int a, int b, int c) = 0;
  virtual void halfplane_sums(int nterms, const int* kind, const int* ia, const int* ib,
                              const int* kin, double band_lo, double band_hi, const int* planes4,
                              double* out) = 0;
  virtual void shells(bool transfers, double* out5) = 0;  // (n/2+1) x 5
  virtual double cfl(double cfl, const ModelCoef& mc) = 0;

  // hot path
  virtual void set_dt(double dt) = 0;
  virtual void set_time(double t) = 0;
  virtual double get_dt() = 0;
  virtual double get_time() = 0;
  virtual void get_dt_time(double* dt, double* time) = 0;  // both with one copy
  virtual void mark_state_untruncated() = 0;
  // Batched engines hold nruns() runs of the same n that advance together;
  // per-run operations (state, forcing, diagnostics, dt, time) act on the run
  // chosen by select_run.  Each run has its own coefficients.
  virtual int nruns() const = 0;
  virtual void select_run(int r) = 0;
  virtual void set_run_coefs(const std::vector<ModelCoef>& mc) = 0;
  virtual void set_dt_all(double dt) = 0;
  virtual void get_scalars(double* dt, double* time) = 0;  // per run
  // Two-phase step for capture into an outer CUDA graph: prepare (uploads,
  // truncation; synchronises) before the capture, then enqueue one step of
  // every run on stream() while the capture is open.
  virtual void prepare_steps(double cfl) = 0;
  virtual void enqueue_steps(bool cfl_mode) = 0;

  // learned closure (coarse runs): 8 CNN input channels of the current state
  // (physical, FP32 NHWC [n][n][8]); the subgrid targets against a finer run
  // (FP32 NHWC [n][n][2]); the tendencies added to the two brackets by the
  // following steps (physical FP32 [n][n][2]; null switches them off)
  // (wait = false: queue the work and return, for capture into a graph)
  virtual void closure_inputs(float* d_x, bool wait) = 0;
  // Fused forms for the captured LES step (where closure_fused() is true):
  // the inputs straight into the network's bf16 first activation
  // ([n][n][16], standardised with in_mean/in_sd), and the tendencies
  // straight from the network's standardised output ([n][n][2] FP32, with
  // out_mean/out_sd); the same results as closure_inputs / set_closure with
  // the network's own conversions
  virtual bool closure_fused() const = 0;
  virtual void closure_inputs_cnn(void* act0, const float* in_mean, const float* in_sd) = 0;
  virtual void set_closure_cnn(const float* y, const float* out_mean, const float* out_sd) = 0;
  virtual void brackets() = 0;  // [psi,-k^2 psi] -> P_B5, [psi,vz] -> P_B6 (full plane)
  virtual void coarsen_from(IEngine* fine, int fine_plane, int dst_plane) = 0;
  virtual void refine_from(IEngine* coarse, int coarse_plane, int dst_plane) = 0;  // spectral zero-pad
  virtual void closure_targets(IEngine* fine, float* d_y) = 0;
  virtual void set_closure(const float* d_t, bool wait) = 0;
  // Per-shell weights (shell b = int(sqrt(ka2)+.5), b < nw; beyond nw: 0)
  // applied to the tendency planes by every later set_closure /
  // set_closure_cnn: w[b] to the first, w[nw + b] to the second; nw = 0
  // switches the weighting off.  Host array of 2 nw floats, copied
  // (synchronously: call outside any capture).
  virtual void set_closure_band(const float* w, int nw) = 0;
  // Work queued on the engine stream before every step of advance(), inside
  // the captured graph (id != 0; id identifies the hook for the graph cache,
  // and id 0 removes it).
  virtual void set_step_hook(std::function<void(cudaStream_t)> hook, unsigned long long id) = 0;
  // The hook runs before every k-th step only: advance() then replays one
  // graph of the hook and k steps, and nsteps must be a multiple of k
  // (constant forcing only).  k = 1 is the default.
  virtual void set_hook_every(int k) = 0;
  // The hook beside the step instead of before it (interval 1, constant
  // forcing, closure scratch allocated): advance() queues the hook once for
  // the first step, then every captured step runs the hook for the next step
  // on a forked stream from the state the step starts from, so step s > 0
  // takes the hook's result for the state before step s - 1
  virtual void set_hook_overlap(bool on) = 0;
  virtual void rand_force(const RandForceHost f[2]) = 0;
  // One RK4 step.  cfl_mode: dt from the CFL condition of the current state
  // (fused into the first substep), else the dt already set.  add_time:
  // time += dt on the device.  rf: per-step forcing draws (iflow = 3) or null.
  virtual void step(const ModelCoef& mc, bool cfl_mode, double cfl, bool add_time,
                    const RandForceHost* rf) = 0;
  // nsteps steps replayed from one captured CUDA graph; rf holds 2*nsteps
  // forcing draws (iflow = 3) or is null.
  virtual void advance(const ModelCoef& mc, int nsteps, bool cfl_mode, double cfl,
                       const RandForceHost* rf) = 0;
  virtual void initial_condition_phys(const std::vector<IcModeHost>& modes) = 0;  // -> R_1, R_2
  virtual void iflow1_phys(double kup) = 0;                                        // -> R_1, R_2
  virtual void scale_mask2(int a, int b, double sa, double sb) = 0;
  // const_inj (iflow = 2): configure the band (loop-order element list, kx=0
  // mirrors, random factors); when enabled every RK substep rebuilds fp, fz.
  virtual void set_const_inj(bool on, double kdn, double kup, double fp0, double fz0,
                             const std::vector<int>& band_idx, const std::vector<int>& mirror,
                             const std::vector<float>& rnd) = 0;
  virtual void const_inj(int src, int dst, int kin, double f0) = 0;
  virtual void sync() = 0;
  virtual int kernel_launches() const = 0;
  // JSON text of the launch-schedule autotuner's measurements and choices
  virtual std::string plan_report() const = 0;
  // Re-derive the launch choices from the autotuner's timings: policy 0 the
  // fastest of every candidate, 1 only full CTAs or persistent CTAs (for
  // ensembles whose size groups run concurrently)
  virtual void set_plan_policy(int policy) = 0;
  // Per-kernel device time of nsteps RK4 steps with the dt already set,
  // measured with CUDA events recorded on the engine stream around every
  // launch: ms[k] = total milliseconds, cnt[k] = launches, for k = 0 pass A,
  // 1 pass B, 2 pass C, 3 everything else.
  virtual void profile_steps(const ModelCoef& mc, int nsteps, double ms[4], long long cnt[4]) = 0;
};

// full = false allocates only what the Level-1 transforms need; nb > 1 makes
// a batched engine of nb runs.
IEngine* make_engine_f64(int n, int device, bool full, int nb = 1);
IEngine* make_engine_f32(int n, int device, bool full, int nb = 1);
bool supported_n(int n);

}  // namespace r2d3c

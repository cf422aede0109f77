// C-ABI of the Rot2D3C GB300 hot path (declared in include/r2d3c.h).
//
// Host-side logic that the reference keeps in Fortran and that is not device
// work lives here: parameter checks, the randu generator and the forcing
// draws, the order of the reference's calls inside each entry point, and the
// mapping of errors to status codes.  Device work goes to the engine of the
// context (r2d3c_engine_impl.cuh).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/r2d3c.h"
#include "r2d3c_engine.h"

namespace r2d3c {

void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  cudaGetLastError();
  const int code = (e == cudaErrorMemoryAllocation) ? kENOMEM : kECUDA;
  throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

bool supported_n(int n) { return n >= 16 && n <= 8192 && (n & (n - 1)) == 0; }

}  // namespace r2d3c

using namespace r2d3c;

namespace {

thread_local std::string g_err;
void set_err(const std::string& s) { g_err = s; }

}  // namespace

namespace r2d3c {
// error text slot shared with the entry points defined in other files
std::string& last_error_slot() { return g_err; }
}  // namespace r2d3c

namespace {

constexpr double kPi = 3.1415926535897932384;  // module var (pseudospec2D_mod.f90:34-39)

// randu (pseudospec2D_mod.f90:52-71): XOR-masked Park-Miller step with
// Schrage's factorisation in 32-bit integers; REAL (float) arithmetic for the
// result.  *idum is updated in place like the Fortran INTEGER argument.
float randu_impl(int* idum) {
  const int iq = 127773, ir = 2836, mask = 123459876;
  const int ia = 16807, im = 2147483647;
  const float am = 1.0f / (float)im;  // REAL parameter am = 1./im
  int s = *idum ^ mask;
  const int k = s / iq;  // truncates toward zero, as Fortran INTEGER division
  const long long t = (long long)ia * (long long)(s - k * iq) - (long long)ir * k;
  s = (int)(unsigned)(unsigned long long)t;  // 32-bit two's-complement wrap
  if (s < 0) s += im;
  float r = am * (float)s;
  r = (r - 0.5f) * 2.0f;
  *idum = s ^ mask;
  return r;
}

double ipow(double x, int k) {  // REAL**INTEGER by repeated squaring
  if (k == 0) return 1.0;
  unsigned e = k < 0 ? (unsigned)(-k) : (unsigned)k;
  double r = 1.0, b = x;
  while (true) {
    if (e & 1u) r = r * b;
    e >>= 1;
    if (!e) break;
    b = b * b;
  }
  return k < 0 ? 1.0 / r : r;
}

}  // namespace

struct r2d3c_ctx {
  r2d3c_params p{};
  std::unique_ptr<IEngine> eng;
  int ci_final_seed = 0;  // seed value left by one const_inj call
  // closure-graph scratch: network inputs [n][n][8] and tendencies [n][n][2]
  float* cl_x = nullptr;
  float* cl_t = nullptr;
  ModelCoef mc() const { return ModelCoef{p.nu, p.hnu, p.nuv, p.hnuv, p.omega, p.nn, p.mm, p.nnv, p.mmv}; }
  ~r2d3c_ctx() {
    eng.reset();
    if (cl_x) cudaFree(cl_x);
    if (cl_t) cudaFree(cl_t);
  }
};

namespace r2d3c {
void cnn_forward_on(r2d3c_cnn* c, const float* d_x, int batch, float* d_out, cudaStream_t stream);
void cnn_shape(const r2d3c_cnn* c, int* H, int* W, int* max_batch, unsigned long long* serial);
void cnn_check_err(r2d3c_cnn* c);
void cnn_io(r2d3c_cnn* c, void** act0, const float** out, const float** norm);
void cnn_layers_on(r2d3c_cnn* c, int batch, cudaStream_t stream);
}  // namespace r2d3c

struct r2d3c_plan {
  int n = 0, dir = 0;
  std::unique_ptr<IEngine> eng;
};

struct r2d3c_ensemble {
  struct Group {
    int n = 0, runs = 0, first = 0;
    std::unique_ptr<IEngine> eng;
  };
  std::vector<Group> groups;
  std::vector<r2d3c_params> params;
  cudaStream_t master = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t graph = nullptr;
  int graph_cfl = -1;
  long long graph_launches = 0, launches = 0;
  ~r2d3c_ensemble() {
    if (graph) cudaGraphExecDestroy(graph);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (master) cudaStreamDestroy(master);
  }
  // (group, local run) of a global run index
  Group& locate(int run, int* local) {
    for (Group& g : groups)
      if (run >= g.first && run < g.first + g.runs) {
        *local = run - g.first;
        g.eng->select_run(*local);
        return g;
      }
    throw r2d3c::Error(r2d3c::kEINVAL, "run index out of range");
  }
};

#define API_BEGIN try {
#define API_END                                                  \
  }                                                              \
  catch (const Error& e) {                                       \
    set_err(e.what());                                           \
    return e.code;                                               \
  }                                                              \
  catch (const std::bad_alloc&) {                                \
    set_err("host allocation failed");                           \
    return R2D3C_ENOMEM;                                         \
  }                                                              \
  catch (const std::exception& e) {                              \
    set_err(e.what());                                           \
    return R2D3C_EINVAL;                                         \
  }                                                              \
  catch (...) {                                                  \
    set_err("unknown error");                                    \
    return R2D3C_EINVAL;                                         \
  }                                                              \
  return R2D3C_OK;

#define REQUIRE(cond, msg)                   \
  do {                                       \
    if (!(cond)) throw Error(kEINVAL, msg);  \
  } while (0)

namespace {

IEngine* new_engine(int n, int precision, bool full) {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  return precision == R2D3C_FP64 ? make_engine_f64(n, dev, full) : make_engine_f32(n, dev, full);
}

// One rand_force draw (pseudospec2D_Rot2D3C.f90:1086-1099, one rank): the
// mode (kx, ky) of length kup, the phase, and the entries it sets
// (:1100-1122).  *seed advances by one randu call; the phase uses the
// temporary seed+1.
RandForceHost rand_force_draw(const r2d3c_params& p, double f0, int kin, int* seed) {
  const int n = p.n;
  const double theta = (double)randu_impl(seed) * kPi;
  int tmpseed = *seed + 1;
  const double phase = (double)randu_impl(&tmpseed) * kPi;
  const double kx = std::floor(p.kup * std::cos(theta) + 0.5);
  const double ky = std::floor(p.kup * std::sin(theta) + 0.5);
  RandForceHost f{};
  f.c0 = std::sqrt(2.0 * f0);
  f.kpow = ipow(p.kup, kin);
  f.cph = std::cos(phase);
  f.sph = std::sin(phase);
  auto ka = [n](int j) { return (double)(j < n / 2 ? j : j - n); };
  auto add = [&f](int idx, int cj) {
    if (f.nset < 4) {
      f.set[f.nset] = idx;
      f.conj[f.nset] = cj;
      ++f.nset;
    }
  };
  for (int i = 1; i <= n / 2; ++i) {  // columns i != 1 of the reference
    const double kai = ka(i);
    if (kai == ky || kai == -ky)
      for (int j = 0; j < n; ++j)
        if (ka(j) == kx) add(i * n + j, 0);
  }
  if (ky == 0.0)  // column i = 1 (kx = 0), :1109-1121
    for (int j = 1; j < n / 2; ++j)
      if (ka(j) == kx) {
        add(j, 0);
        add(n - j, 1);
      }
  return f;
}

void rand_force_pair(r2d3c_ctx* c, int* seed, int* seed1, RandForceHost out[2]) {
  out[0] = rand_force_draw(c->p, c->p.fp0, 1, seed);   // fp with seed (:414)
  out[1] = rand_force_draw(c->p, c->p.fz0, 0, seed1);  // fz with seed1 (:415)
}

// Band list of const_inj in the reference's loop order (kx = 0 column first,
// j = 2..n/2; then columns 2..n/2+1, j = 1..n), its kx = 0 mirrors and the
// randu factors drawn from the seed myrank = 0 (:1032-1057).
void setup_const_inj(r2d3c_ctx* c, bool on) {
  const int n = c->p.n;
  const double lo = c->p.kdn * c->p.kdn, hi = c->p.kup * c->p.kup;
  auto ka = [n](int j) { return (double)(j < n / 2 ? j : j - n); };
  std::vector<int> idx, mir;
  std::vector<float> rnd;
  int s = 0;  // seed1 = myrank
  for (int j = 1; j < n / 2; ++j) {
    const double k2 = ka(j) * ka(j);
    if (k2 <= hi && k2 >= lo) {
      idx.push_back(j);
      mir.push_back(n - j);
      rnd.push_back(randu_impl(&s));
    }
  }
  for (int i = 1; i <= n / 2; ++i)
    for (int j = 0; j < n; ++j) {
      const double k2 = ka(i) * ka(i) + ka(j) * ka(j);
      if (k2 <= hi && k2 >= lo) {
        idx.push_back(i * n + j);
        mir.push_back(-1);
        rnd.push_back(randu_impl(&s));
      }
    }
  c->ci_final_seed = s;
  c->eng->set_const_inj(on, c->p.kdn, c->p.kup, c->p.fp0, c->p.fz0, idx, mir, rnd);
}

void check_params(const r2d3c_params* p) {
  REQUIRE(p, "params is NULL");
  REQUIRE(supported_n(p->n), "n must be a power of two in [16, 8192]");
  REQUIRE(p->nn >= -64 && p->nn <= 64 && p->mm >= -64 && p->mm <= 64 && p->nnv >= -64 &&
              p->nnv <= 64 && p->mmv >= -64 && p->mmv <= 64,
          "dissipation orders out of range");
  REQUIRE(p->iflow >= 0 && p->iflow <= 3, "iflow must be 0..3");
}

}  // namespace

extern "C" {

const char* r2d3c_version(void) { return "rot2d3c_gb300 0.1 (sm_103a)"; }
const char* r2d3c_last_error(void) { return g_err.c_str(); }
float r2d3c_randu(int* seed) { return seed ? randu_impl(seed) : 0.0f; }

int r2d3c_kernel_launches(const r2d3c_ctx* ctx, long long* count) {
  API_BEGIN
  REQUIRE(ctx && count, "NULL argument");
  *count = ctx->eng->kernel_launches();
  API_END
}

// ---------------------------------------------------------------- Level 1
int r2d3c_fft_plan_create(int n, int dir, int flags, int precision, r2d3c_plan** plan) {
  (void)flags;
  API_BEGIN
  REQUIRE(plan, "plan is NULL");
  *plan = nullptr;
  REQUIRE(supported_n(n), "n must be a power of two in [16, 8192]");
  REQUIRE(dir == R2D3C_R2C || dir == R2D3C_C2R, "dir must be -1 (R2C) or +1 (C2R)");
  REQUIRE(precision == R2D3C_FP64 || precision == R2D3C_FP32, "bad precision");
  std::unique_ptr<r2d3c_plan> pl(new r2d3c_plan());
  pl->n = n;
  pl->dir = dir;
  pl->eng.reset(new_engine(n, precision, false));
  *plan = pl.release();
  API_END
}

int r2d3c_fft_plan_destroy(r2d3c_plan* plan) {
  API_BEGIN
  delete plan;
  API_END
}

int r2d3c_fft_r2c(r2d3c_plan* plan, const double* in, double* out) {
  API_BEGIN
  REQUIRE(plan && in && out, "NULL argument");
  REQUIRE(plan->dir == R2D3C_R2C, "plan direction is not R2C");
  plan->eng->upload_real(R_1, in);
  plan->eng->r2c(R_1, P_W1);
  plan->eng->download_spec(P_W1, out);
  API_END
}

int r2d3c_fft_c2r(r2d3c_plan* plan, double* in, double* out) {
  API_BEGIN
  REQUIRE(plan && in && out, "NULL argument");
  REQUIRE(plan->dir == R2D3C_C2R, "plan direction is not C2R");
  plan->eng->upload_spec(P_W1, in);
  plan->eng->c2r(P_W1, R_1, nullptr, nullptr);
  plan->eng->download_real(R_1, out);
  API_END
}

namespace {
// order the plan's stream after `user` and `user` after the plan's work
struct StreamJoin {
  cudaStream_t user, own;
  cudaEvent_t ev = nullptr;
  StreamJoin(void* u, cudaStream_t o) : user((cudaStream_t)u), own(o) {
    if (user && user != own) {
      cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
      cuda_check(cudaEventRecord(ev, user), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(own, ev, 0), "cudaStreamWaitEvent");
    }
  }
  void done() {
    if (ev) {
      cuda_check(cudaEventRecord(ev, own), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(user, ev, 0), "cudaStreamWaitEvent");
    }
  }
  ~StreamJoin() {
    if (ev) cudaEventDestroy(ev);
  }
};
}  // namespace

int r2d3c_fft_r2c_dev(r2d3c_plan* plan, const double* d_in, double* d_out, void* stream) {
  API_BEGIN
  REQUIRE(plan && d_in && d_out, "NULL argument");
  REQUIRE(plan->dir == R2D3C_R2C, "plan direction is not R2C");
  StreamJoin j(stream, plan->eng->stream());
  plan->eng->real_from_dev64(R_1, d_in);
  plan->eng->r2c(R_1, P_W1);
  plan->eng->spec_to_dev64(P_W1, d_out);
  j.done();
  API_END
}

int r2d3c_fft_c2r_dev(r2d3c_plan* plan, const double* d_in, double* d_out, void* stream) {
  API_BEGIN
  REQUIRE(plan && d_in && d_out, "NULL argument");
  REQUIRE(plan->dir == R2D3C_C2R, "plan direction is not C2R");
  StreamJoin j(stream, plan->eng->stream());
  plan->eng->spec_from_dev64(P_W1, d_in);
  plan->eng->c2r(P_W1, R_1, nullptr, nullptr);
  plan->eng->real_to_dev64(R_1, d_out);
  j.done();
  API_END
}

// ---------------------------------------------------------------- Level 2
int r2d3c_create(const r2d3c_params* params, int precision, r2d3c_ctx** ctx) {
  API_BEGIN
  REQUIRE(ctx, "ctx is NULL");
  *ctx = nullptr;
  check_params(params);
  REQUIRE(precision == R2D3C_FP64 || precision == R2D3C_FP32, "bad precision");
  std::unique_ptr<r2d3c_ctx> c(new r2d3c_ctx());
  c->p = *params;
  c->eng.reset(new_engine(params->n, precision, true));
  if (params->iflow == 2) setup_const_inj(c.get(), true);
  *ctx = c.release();
  API_END
}

int r2d3c_destroy(r2d3c_ctx* ctx) {
  API_BEGIN
  delete ctx;
  API_END
}

int r2d3c_device_bytes(const r2d3c_ctx* ctx, long long* bytes) {
  API_BEGIN
  REQUIRE(ctx && bytes, "NULL argument");
  *bytes = (long long)ctx->eng->bytes_allocated();
  API_END
}

int r2d3c_set_state(r2d3c_ctx* ctx, const double* ps_hat, const double* vz_hat) {
  API_BEGIN
  REQUIRE(ctx && ps_hat && vz_hat, "NULL argument");
  ctx->eng->upload_spec(P_PS, ps_hat);
  ctx->eng->upload_spec(P_VZ, vz_hat);
  ctx->eng->mark_state_untruncated();
  API_END
}

int r2d3c_get_state(r2d3c_ctx* ctx, double* ps_hat, double* vz_hat) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  if (ps_hat) ctx->eng->download_spec(P_PS, ps_hat);
  if (vz_hat) ctx->eng->download_spec(P_VZ, vz_hat);
  API_END
}

int r2d3c_set_state_physical(r2d3c_ctx* ctx, const double* ps, const double* vz) {
  API_BEGIN
  REQUIRE(ctx && ps && vz, "NULL argument");
  ctx->eng->upload_real(R_1, ps);
  ctx->eng->r2c(R_1, P_PS);  // :324-325
  ctx->eng->upload_real(R_1, vz);
  ctx->eng->r2c(R_1, P_VZ);  // :328-329
  ctx->eng->mark_state_untruncated();
  ctx->eng->sync();
  API_END
}

int r2d3c_set_forcing(r2d3c_ctx* ctx, const double* fp_hat, const double* fz_hat) {
  API_BEGIN
  REQUIRE(ctx && fp_hat && fz_hat, "NULL argument");
  ctx->eng->upload_spec(P_FP, fp_hat);
  ctx->eng->upload_spec(P_FZ, fz_hat);
  API_END
}

int r2d3c_get_forcing(r2d3c_ctx* ctx, double* fp_hat, double* fz_hat) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  if (fp_hat) ctx->eng->download_spec(P_FP, fp_hat);
  if (fz_hat) ctx->eng->download_spec(P_FZ, fz_hat);
  API_END
}

namespace {
double energy_of(IEngine* e, int plane, int kin) {
  const int kind = 0 /* S_ENERGY */, ia = 0, ib = 0;
  const int pl[4] = {plane, -1, -1, -1};
  double out = 0.0;
  e->halfplane_sums(1, &kind, &ia, &ib, &kin, 0.0, 0.0, pl, &out);
  return out;
}
}  // namespace

int r2d3c_initial_conditions(r2d3c_ctx* ctx, int* seed) {
  API_BEGIN
  REQUIRE(ctx && seed, "NULL argument");
  const r2d3c_params& p = ctx->p;
  std::vector<IcModeHost> modes;
  const int kend = (int)(p.kup + 1);  // DO ir = 1,kup+1 with kup DOUBLE
  for (int ir = 1; ir <= kend; ++ir)
    for (int jr = 1; jr <= kend; ++jr) {
      IcModeHost m{};
      m.ir = ir;
      m.jr = jr;
      m.kr = std::sqrt((double)(ir * ir + jr * jr));
      m.ph1 = (double)randu_impl(seed) * 2.0 * kPi;
      m.ph2 = (double)randu_impl(seed) * 2.0 * kPi;
      m.ph3 = (double)randu_impl(seed) * 2.0 * kPi;
      m.ph4 = (double)randu_impl(seed) * 2.0 * kPi;
      modes.push_back(m);
    }
  IEngine* e = ctx->eng.get();
  e->initial_condition_phys(modes);  // :255-279
  e->r2c(R_1, P_PS);                 // :280
  e->r2c(R_2, P_VZ);                 // :281
  const double ener = energy_of(e, P_PS, 1);
  const double enerv = energy_of(e, P_VZ, 0);
  e->scale_mask2(P_PS, P_VZ, p.u0 / std::sqrt(ener), p.v0 / std::sqrt(enerv));  // :286-298
  e->sync();
  API_END
}

int r2d3c_forcing_init(r2d3c_ctx* ctx, int* seed, int* seed1) {
  API_BEGIN
  REQUIRE(ctx && seed && seed1, "NULL argument");
  r2d3c_params& p = ctx->p;
  IEngine* e = ctx->eng.get();
  if (p.iflow == 1) {  // :343-371
    p.kdn = p.kup;
    e->iflow1_phys(p.kup);
    e->r2c(R_1, P_FP);
    const double eneru = energy_of(e, P_FP, 1);
    e->r2c(R_2, P_FZ);
    const double enerv = energy_of(e, P_FZ, 0);
    e->scale_mask2(P_FP, P_FZ, p.fp0 / std::sqrt(eneru), p.fz0 / std::sqrt(enerv));
  } else if (p.iflow == 2) {  // :372-375
    *seed1 = *seed + 1;
    e->const_inj(P_PS, P_FP, 1, p.fp0);
    e->const_inj(P_VZ, P_FZ, 0, p.fz0);
    *seed1 = ctx->ci_final_seed;
    *seed = ctx->ci_final_seed;
  } else if (p.iflow == 3) {  // :376-380
    *seed1 = *seed + 1;
    e->cfl(p.cfl, ctx->mc());
    RandForceHost f[2];
    rand_force_pair(ctx, seed, seed1, f);
    e->rand_force(f);
  } else {
    e->zero_spec(P_FP);
    e->zero_spec(P_FZ);
  }
  e->sync();
  API_END
}

int r2d3c_cfl(r2d3c_ctx* ctx, double cfl, double* dt) {
  API_BEGIN
  REQUIRE(ctx && dt, "NULL argument");
  *dt = ctx->eng->cfl(cfl, ctx->mc());
  API_END
}

int r2d3c_force_random(r2d3c_ctx* ctx, double dt, int* seed, int* seed1) {
  API_BEGIN
  REQUIRE(ctx && seed && seed1, "NULL argument");
  REQUIRE(dt > 0.0, "dt must be positive");
  ctx->eng->set_dt(dt);
  RandForceHost f[2];
  rand_force_pair(ctx, seed, seed1, f);
  ctx->eng->rand_force(f);
  ctx->eng->sync();
  API_END
}

int r2d3c_step(r2d3c_ctx* ctx, double dt, int* seed, int* seed1) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  REQUIRE(dt > 0.0 && std::isfinite(dt), "dt must be positive and finite");
  ctx->eng->set_dt(dt);
  ctx->eng->step(ctx->mc(), false, 0.0, false, nullptr);
  if (ctx->p.iflow == 2 && seed && seed1) *seed = *seed1 = ctx->ci_final_seed;
  ctx->eng->sync();
  API_END
}

int r2d3c_advance(r2d3c_ctx* ctx, int nsteps, int dt_mode, double cfl_or_dt, double* time,
                  double* dt_last, int* seed, int* seed1) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  REQUIRE(nsteps >= 0, "nsteps must be >= 0");
  REQUIRE(dt_mode == R2D3C_DT_CFL || dt_mode == R2D3C_DT_FIXED, "bad dt_mode");
  REQUIRE(cfl_or_dt > 0.0 && std::isfinite(cfl_or_dt), "cfl_or_dt must be positive and finite");
  IEngine* e = ctx->eng.get();
  std::vector<RandForceHost> rf;
  if (ctx->p.iflow == 3) {
    REQUIRE(seed && seed1, "iflow 3 needs seed and seed1");
    rf.resize(2 * (size_t)nsteps);
    for (int s = 0; s < nsteps; ++s) rand_force_pair(ctx, seed, seed1, &rf[2 * (size_t)s]);
  }
  if (dt_mode == R2D3C_DT_FIXED) e->set_dt(cfl_or_dt);
  e->advance(ctx->mc(), nsteps, dt_mode == R2D3C_DT_CFL, cfl_or_dt, rf.empty() ? nullptr : rf.data());
  if (ctx->p.iflow == 2 && seed && seed1 && nsteps > 0) *seed = *seed1 = ctx->ci_final_seed;
  double dt = 0.0, t = 0.0;
  e->get_dt_time(&dt, &t);  // one copy, one synchronisation
  if (time) *time = t;
  if (dt_last) *dt_last = dt;
  API_END
}

int r2d3c_set_time(r2d3c_ctx* ctx, double time) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  ctx->eng->set_time(time);
  API_END
}

int r2d3c_cond_check(r2d3c_ctx* ctx, double time, double out[30]) {
  API_BEGIN
  REQUIRE(ctx && out, "NULL argument");
  const r2d3c_params& p = ctx->p;
  IEngine* e = ctx->eng.get();
  // slots 0 ps, 1 vz, 2 fp, 3 fz; kinds: 0 energy, 1 inerprod, 2 inerprod(a, d_y b),
  // 3 band ka2|a|^2, 4 band |a|^2   (pseudospec2D_Rot2D3C.f90:484-568)
  const int kind[22] = {0, 1, 0, 0, 0, 1, 0, 0, 2, 0, 1, 0, 0, 1, 1, 1, 1, 1, 1, 1, 3, 4};
  const int ia[22] = {0, 0, 0, 0, 1, 1, 1, 1, 1, 0, 0, 0, 0, 1, 1, 0, 1, 1, 0, 0, 0, 1};
  const int ib[22] = {0, 2, 0, 0, 1, 3, 1, 1, 0, 0, 2, 0, 0, 0, 2, 3, 0, 0, 1, 1, 0, 1};
  const int kin[22] = {1,          1,          p.nn + 1,   1 - p.mm,   0, 0, p.nnv, -p.mmv,
                       0,          2,          2,          p.nn + 2,   2 - p.mm, 1, 1, 1,
                       p.nn + 1,   1 - p.mm,   p.nnv + 1,  1 - p.mmv,  0, 0};
  const int planes[4] = {P_PS, P_VZ, P_FP, P_FZ};
  double s[22];
  const double band_hi = 2.01 * p.kup * p.kup, band_lo = p.kup * p.kup;
  e->halfplane_sums(22, kind, ia, ib, kin, band_lo, band_hi, planes, s);
  const double Ep1 = s[0], injp1 = s[1], Dsp = s[2], Hds = s[3], Epv = s[4], injz = s[5];
  const double Dspv = s[6], Hdsv = s[7], coup = s[8], Ep2 = s[9], injp2 = s[10], Dspw = s[11];
  const double Hdsw = s[12], Eph = s[13], injh1 = s[14], injh2 = s[15], Dsph1 = s[16];
  const double Hdsh1 = s[17], Dsph2 = s[18], Hdsh2 = s[19], Efp = s[20], Efpz = s[21];
  double maxw, minw, maxv, minv;
  e->specop(P_PS, P_W1, 3 /* laplak2 */, 0.0);  // :573-576
  e->c2r(P_W1, -1, &maxw, &minw);
  e->specop(P_VZ, P_W1, 0 /* derivk2 dir 0 */, 0.0);  // :581-584
  e->c2r(P_W1, -1, &maxv, &minv);
  const double w2 = 2 * p.omega;
  const double v[30] = {time, Ep1, Epv, injp1, injz, p.nu * Dsp, p.nuv * Dspv, p.hnu * Hds,
                        p.hnuv * Hdsv, w2 * coup, Efp, Efpz,
                        time, Ep2, injp2, p.nu * Dspw, p.hnu * Hdsw,
                        time, -Eph, -injh1, -injh2, -p.nu * Dsph1, -p.nuv * Dsph2, -p.hnu * Hdsh1,
                        -p.hnuv * Hdsh2,
                        time, maxw, minw, maxv, minv};
  std::memcpy(out, v, sizeof(v));
  API_END
}

int r2d3c_spectrum(r2d3c_ctx* ctx, double* Ek, double* Ezk) {
  API_BEGIN
  REQUIRE(ctx && Ek && Ezk, "NULL argument");
  const int nb = ctx->p.n / 2 + 1;
  std::vector<double> o5((size_t)nb * 5);
  ctx->eng->shells(false, o5.data());
  for (int b = 0; b < nb; ++b) {
    Ek[b] = o5[(size_t)b * 5 + 0];
    Ezk[b] = o5[(size_t)b * 5 + 1];
  }
  API_END
}

int r2d3c_transfers(r2d3c_ctx* ctx, double* Fl0, double* Fl1, double* Fl2) {
  API_BEGIN
  REQUIRE(ctx && Fl0 && Fl1 && Fl2, "NULL argument");
  const int nb = ctx->p.n / 2 + 1;
  std::vector<double> o5((size_t)nb * 5);
  ctx->eng->shells(true, o5.data());
  for (int b = 0; b < nb; ++b) {
    Fl0[b] = o5[(size_t)b * 5 + 2];
    Fl1[b] = o5[(size_t)b * 5 + 3];
    Fl2[b] = o5[(size_t)b * 5 + 4];
  }
  API_END
}

int r2d3c_get_field(r2d3c_ctx* ctx, int which, double* R) {
  API_BEGIN
  REQUIRE(ctx && R, "NULL argument");
  REQUIRE(which >= 0 && which <= 3, "bad field selector");
  IEngine* e = ctx->eng.get();
  const double n = (double)ctx->p.n;
  const double tmp = 1.0 / (n * n);  // :476
  switch (which) {
    case R2D3C_FIELD_PS: e->specop(P_PS, P_W1, 5, tmp); break;
    case R2D3C_FIELD_VZ: e->specop(P_VZ, P_W1, 5, tmp); break;
    case R2D3C_FIELD_WW: e->specop(P_PS, P_W1, 6, tmp); break;
    default:
      e->specop(P_PS, P_W2, 4, 0.0);  // inv_laplak2 (:509)
      e->specop(P_W2, P_W1, 5, tmp);
      break;
  }
  e->c2r(P_W1, R_1, nullptr, nullptr);
  e->download_real(R_1, R);
  API_END
}

// ---------------------------------------------------------------- ensembles
// One step of every group captured into the ensemble's graph, the groups
// forked onto their own streams.
static void ens_capture(r2d3c_ensemble* ens, bool cfl) {
  if (ens->graph) cudaGraphExecDestroy(ens->graph);
  ens->graph = nullptr;
  // one step of every group, the groups forked onto their own streams
  long long before = 0;
  for (auto& g : ens->groups) before += g.eng->kernel_launches();
  cudaGraph_t graph = nullptr;
  cuda_check(cudaStreamBeginCapture(ens->master, cudaStreamCaptureModeThreadLocal), "BeginCapture");
  try {
    cuda_check(cudaEventRecord(ens->fork, ens->master), "cudaEventRecord");
    for (size_t i = 0; i < ens->groups.size(); ++i) {
      IEngine* eng = ens->groups[i].eng.get();
      cuda_check(cudaStreamWaitEvent(eng->stream(), ens->fork, 0), "cudaStreamWaitEvent");
      eng->enqueue_steps(cfl);
      cuda_check(cudaEventRecord(ens->joins[i], eng->stream()), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(ens->master, ens->joins[i], 0), "cudaStreamWaitEvent");
    }
  } catch (...) {
    cudaStreamEndCapture(ens->master, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  cuda_check(cudaStreamEndCapture(ens->master, &graph), "EndCapture");
  const cudaError_t ie = cudaGraphInstantiate(&ens->graph, graph, 0);
  cudaGraphDestroy(graph);
  cuda_check(ie, "GraphInstantiate");
  long long after = 0;
  for (auto& g : ens->groups) after += g.eng->kernel_launches();
  ens->graph_launches = after - before;
  ens->graph_cfl = (int)cfl;
}

// Seconds per ensemble step (graph replay, fixed dt) under the engines'
// current plans.
static double ens_time_step(r2d3c_ensemble* ens, int steps) {
  ens_capture(ens, false);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
  cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
  for (int s = 0; s < 2; ++s) cuda_check(cudaGraphLaunch(ens->graph, ens->master), "GraphLaunch");
  cuda_check(cudaEventRecord(e0, ens->master), "cudaEventRecord");
  for (int s = 0; s < steps; ++s) cuda_check(cudaGraphLaunch(ens->graph, ens->master), "GraphLaunch");
  cuda_check(cudaEventRecord(e1, ens->master), "cudaEventRecord");
  cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
  float ms = 0.f;
  cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 1e-3 * ms / steps;
}

int r2d3c_ensemble_create(int ngroups, const int* n, const int* runs, const r2d3c_params* params,
                          int precision, r2d3c_ensemble** ens) {
  API_BEGIN
  REQUIRE(ens && n && runs && params, "NULL argument");
  *ens = nullptr;
  REQUIRE(ngroups >= 1 && ngroups <= 16, "ngroups must be 1..16");
  REQUIRE(precision == R2D3C_FP64 || precision == R2D3C_FP32, "bad precision");
  std::unique_ptr<r2d3c_ensemble> e(new r2d3c_ensemble());
  int total = 0;
  for (int g = 0; g < ngroups; ++g) {
    REQUIRE(supported_n(n[g]), "n must be a power of two in [16, 8192]");
    REQUIRE(runs[g] >= 1 && runs[g] <= 4096, "runs per group must be 1..4096");
    total += runs[g];
  }
  e->params.assign(params, params + total);
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  int first = 0;
  for (int g = 0; g < ngroups; ++g) {
    std::vector<ModelCoef> mc;
    for (int r = first; r < first + runs[g]; ++r) {
      const r2d3c_params& p = e->params[r];
      check_params(&p);
      REQUIRE(p.n == n[g], "params[r].n differs from its group's n");
      REQUIRE(p.iflow == 0 || p.iflow == 1, "ensemble runs hold their forcing constant (iflow 0 or 1)");
      mc.push_back(ModelCoef{p.nu, p.hnu, p.nuv, p.hnuv, p.omega, p.nn, p.mm, p.nnv, p.mmv});
    }
    r2d3c_ensemble::Group gr;
    gr.n = n[g];
    gr.runs = runs[g];
    gr.first = first;
    gr.eng.reset(precision == R2D3C_FP64 ? make_engine_f64(n[g], dev, true, runs[g])
                                         : make_engine_f32(n[g], dev, true, runs[g]));
    gr.eng->set_run_coefs(mc);
    e->groups.push_back(std::move(gr));
    first += runs[g];
  }
  cuda_check(cudaStreamCreateWithFlags(&e->master, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming), "cudaEventCreate");
  e->joins.resize(ngroups);
  for (auto& j : e->joins) cuda_check(cudaEventCreateWithFlags(&j, cudaEventDisableTiming), "cudaEventCreate");
  if (ngroups > 1) {
    // The graph runs the size groups side by side, where launch shapes timed
    // alone are no guide: the whole step is timed under each plan policy
    // (per-pass best; full CTAs or persistent; persistent passes B and C
    // wherever they exist) with fixed dt on the new ensemble's zero state,
    // which stays zero, and the fastest is kept; the runs' times are reset
    // afterwards.
    double best = 0.0;
    int pick = 0;
    for (int pol = 0; pol < 3; ++pol) {
      for (auto& g : e->groups) {
        g.eng->set_plan_policy(pol);
        g.eng->set_dt_all(1e-9);
        g.eng->prepare_steps(0.0);
      }
      const double t = ens_time_step(e.get(), 3);
      if (pol == 0 || t < best) {
        best = t;
        pick = pol;
      }
    }
    for (auto& g : e->groups) {
      g.eng->set_plan_policy(pick);
      for (int r = 0; r < g.runs; ++r) {
        g.eng->select_run(r);
        g.eng->set_time(0.0);
      }
    }
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
    e->graph_cfl = -1;
    e->launches = 0;
  }
  *ens = e.release();
  API_END
}

int r2d3c_ensemble_destroy(r2d3c_ensemble* ens) {
  API_BEGIN
  delete ens;
  API_END
}

int r2d3c_ensemble_set_state(r2d3c_ensemble* ens, int run, const double* ps_hat, const double* vz_hat) {
  API_BEGIN
  REQUIRE(ens && ps_hat && vz_hat, "NULL argument");
  int l = 0;
  auto& g = ens->locate(run, &l);
  g.eng->upload_spec(P_PS, ps_hat);
  g.eng->upload_spec(P_VZ, vz_hat);
  g.eng->mark_state_untruncated();
  API_END
}

int r2d3c_ensemble_get_state(r2d3c_ensemble* ens, int run, double* ps_hat, double* vz_hat) {
  API_BEGIN
  REQUIRE(ens, "NULL argument");
  int l = 0;
  auto& g = ens->locate(run, &l);
  if (ps_hat) g.eng->download_spec(P_PS, ps_hat);
  if (vz_hat) g.eng->download_spec(P_VZ, vz_hat);
  API_END
}

int r2d3c_ensemble_set_forcing(r2d3c_ensemble* ens, int run, const double* fp_hat, const double* fz_hat) {
  API_BEGIN
  REQUIRE(ens && fp_hat && fz_hat, "NULL argument");
  int l = 0;
  auto& g = ens->locate(run, &l);
  g.eng->upload_spec(P_FP, fp_hat);
  g.eng->upload_spec(P_FZ, fz_hat);
  API_END
}

int r2d3c_ensemble_set_time(r2d3c_ensemble* ens, int run, double time) {
  API_BEGIN
  REQUIRE(ens, "NULL argument");
  int l = 0;
  auto& g = ens->locate(run, &l);
  g.eng->set_time(time);
  API_END
}

int r2d3c_ensemble_advance(r2d3c_ensemble* ens, int nsteps, int dt_mode, double cfl_or_dt, double* times) {
  API_BEGIN
  REQUIRE(ens, "NULL argument");
  REQUIRE(nsteps >= 0, "nsteps must be >= 0");
  REQUIRE(dt_mode == R2D3C_DT_CFL || dt_mode == R2D3C_DT_FIXED, "bad dt_mode");
  REQUIRE(cfl_or_dt > 0.0 && std::isfinite(cfl_or_dt), "cfl_or_dt must be positive and finite");
  const bool cfl = dt_mode == R2D3C_DT_CFL;
  for (auto& g : ens->groups) {
    if (!cfl) g.eng->set_dt_all(cfl_or_dt);
    g.eng->prepare_steps(cfl ? cfl_or_dt : 0.0);
  }
  if (!ens->graph || ens->graph_cfl != (int)cfl) ens_capture(ens, cfl);
  for (int s = 0; s < nsteps; ++s) {
    cuda_check(cudaGraphLaunch(ens->graph, ens->master), "GraphLaunch");
    ens->launches += ens->graph_launches;
  }
  cuda_check(cudaStreamSynchronize(ens->master), "cudaStreamSynchronize");
  if (times) {
    for (auto& g : ens->groups) {
      std::vector<double> t(g.runs);
      g.eng->get_scalars(nullptr, t.data());
      for (int r = 0; r < g.runs; ++r) times[g.first + r] = t[r];
    }
  }
  API_END
}

int r2d3c_ensemble_cond_check(r2d3c_ensemble* ens, int run, double time, double out[30]) {
  API_BEGIN
  REQUIRE(ens && out, "NULL argument");
  int l = 0;
  auto& g = ens->locate(run, &l);
  r2d3c_ctx view;
  view.p = ens->params[run];
  view.eng.reset(g.eng.get());
  const int rc = r2d3c_cond_check(&view, time, out);
  view.eng.release();
  if (rc != R2D3C_OK) return rc;
  API_END
}

int r2d3c_ensemble_spectrum(r2d3c_ensemble* ens, int run, double* Ek, double* Ezk) {
  API_BEGIN
  REQUIRE(ens && Ek && Ezk, "NULL argument");
  int l = 0;
  auto& g = ens->locate(run, &l);
  r2d3c_ctx view;
  view.p = ens->params[run];
  view.eng.reset(g.eng.get());
  const int rc = r2d3c_spectrum(&view, Ek, Ezk);
  view.eng.release();
  if (rc != R2D3C_OK) return rc;
  API_END
}

int r2d3c_ensemble_kernel_launches(const r2d3c_ensemble* ens, long long* count) {
  API_BEGIN
  REQUIRE(ens && count, "NULL argument");
  *count = ens->launches;
  API_END
}

int r2d3c_ensemble_plan_report(const r2d3c_ensemble* ens, char* buf, int len) {
  API_BEGIN
  REQUIRE(ens && buf && len > 0, "NULL argument");
  std::string r = "[";
  for (size_t g = 0; g < ens->groups.size(); ++g) {
    const auto& gr = ens->groups[g];
    r += (g ? ", " : "") + std::string("{\"n\": ") + std::to_string(gr.n) + ", \"runs\": " + std::to_string(gr.runs) +
         ", \"plan\": " + gr.eng->plan_report() + "}";
  }
  r += "]";
  const size_t k = std::min(r.size(), (size_t)len - 1);
  std::memcpy(buf, r.data(), k);
  buf[k] = 0;
  REQUIRE(r.size() < (size_t)len, "buffer too small for the report");
  API_END
}

// ---------------------------------------------------------------- operators
int r2d3c_derivk2(r2d3c_ctx* ctx, const double* a, double* b, int dir) {
  API_BEGIN
  REQUIRE(ctx && a && b, "NULL argument");
  REQUIRE(dir >= 0 && dir <= 2, "dir must be 0, 1 or 2");
  ctx->eng->upload_spec(P_C1, a);
  ctx->eng->specop(P_C1, P_C2, dir, 0.0);
  ctx->eng->download_spec(P_C2, b);
  API_END
}

int r2d3c_laplak2(r2d3c_ctx* ctx, const double* a, double* b) {
  API_BEGIN
  REQUIRE(ctx && a && b, "NULL argument");
  ctx->eng->upload_spec(P_C1, a);
  ctx->eng->specop(P_C1, P_C2, 3, 0.0);
  ctx->eng->download_spec(P_C2, b);
  API_END
}

int r2d3c_inv_laplak2(r2d3c_ctx* ctx, const double* a, double* b) {
  API_BEGIN
  REQUIRE(ctx && a && b, "NULL argument");
  ctx->eng->upload_spec(P_C1, a);
  ctx->eng->specop(P_C1, P_C2, 4, 0.0);
  ctx->eng->download_spec(P_C2, b);
  API_END
}

int r2d3c_poisson(r2d3c_ctx* ctx, const double* a, const double* b, double* c) {
  API_BEGIN
  REQUIRE(ctx && a && b && c, "NULL argument");
  ctx->eng->upload_spec(P_C1, a);
  ctx->eng->upload_spec(P_C2, b);
  ctx->eng->poisson(P_C1, P_C2, P_B5);
  ctx->eng->download_spec(P_B5, c);
  API_END
}

int r2d3c_energy(r2d3c_ctx* ctx, const double* a, int kin, double* b) {
  API_BEGIN
  REQUIRE(ctx && a && b, "NULL argument");
  ctx->eng->upload_spec(P_C1, a);
  *b = energy_of(ctx->eng.get(), P_C1, kin);
  API_END
}

int r2d3c_inerprod(r2d3c_ctx* ctx, const double* a, const double* b, int kin, double* rslt) {
  API_BEGIN
  REQUIRE(ctx && a && b && rslt, "NULL argument");
  ctx->eng->upload_spec(P_C1, a);
  ctx->eng->upload_spec(P_C2, b);
  const int kind = 1, ia = 0, ib = 1;
  const int pl[4] = {P_C1, P_C2, -1, -1};
  ctx->eng->halfplane_sums(1, &kind, &ia, &ib, &kin, 0.0, 0.0, pl, rslt);
  API_END
}

int r2d3c_profile_passes(r2d3c_ctx* ctx, int nsteps, double dt, double* ms_per_launch,
                         long long* launches) {
  API_BEGIN
  REQUIRE(ctx && ms_per_launch && launches, "NULL argument");
  REQUIRE(nsteps >= 1, "nsteps must be >= 1");
  REQUIRE(dt > 0.0 && std::isfinite(dt), "dt must be positive and finite");
  REQUIRE(ctx->p.iflow != 2, "profiling covers the step without const_inj");
  ctx->eng->set_dt(dt);
  double ms[4];
  ctx->eng->profile_steps(ctx->mc(), nsteps, ms, launches);
  for (int k = 0; k < 4; ++k) ms_per_launch[k] = launches[k] ? ms[k] / (double)launches[k] : 0.0;
  API_END
}

namespace {
// Dependent FMA chains: 8 independent accumulators per thread, `iters`
// iterations of 8 FMAs each.  The result is stored so nothing is elided.
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = (double)(threadIdx.x + i) * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

int r2d3c_fp64_fma_peak(double* tflops) {
  API_BEGIN
  REQUIRE(tflops, "NULL argument");
  int dev = 0, sms = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double* d = nullptr;
  cuda_check(cudaMalloc(&d, sizeof(double) * (size_t)blocks * threads), "cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_fma<<<blocks, threads>>>(d, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fp64_fma<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  const cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  cuda_check(err, "fp64 peak kernel");
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  API_END
}

// ---------------------------------------------------------------- closure
int r2d3c_closure_inputs(r2d3c_ctx* ctx, float* d_x) {
  API_BEGIN
  REQUIRE(ctx && d_x, "NULL argument");
  ctx->eng->closure_inputs(d_x, true);
  API_END
}

int r2d3c_closure_sample(r2d3c_ctx* fine, r2d3c_ctx* coarse, float* d_x, float* d_y) {
  API_BEGIN
  REQUIRE(fine && coarse && d_x && d_y, "NULL argument");
  REQUIRE(fine->p.n > coarse->p.n, "the fine grid must be larger than the coarse grid");
  IEngine* c = coarse->eng.get();
  c->coarsen_from(fine->eng.get(), P_PS, P_PS);
  c->coarsen_from(fine->eng.get(), P_VZ, P_VZ);
  c->closure_inputs(d_x, true);
  c->closure_targets(fine->eng.get(), d_y);
  API_END
}

}  // extern "C"

namespace {
// The reference's slice regridder (regrid_slices.f90:95-104) on a whole
// field: out(j, k) = in((j+1)*n/m, (k+1)*n/m) in 1-based Fortran indices
// with integer division, out m x m, in n x n (n < m <= 2n).  Column-major
// R(x, y) = row-major [y][x].
__global__ void k_regrid_phys(const double* __restrict__ in, int n, double* __restrict__ out, int m) {
  const size_t total = (size_t)m * m;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const long long y = (long long)(idx / m), x = (long long)(idx % m);
    const long long sx = (x + 2) * n / m - 1, sy = (y + 2) * n / m - 1;  // 0-based
    out[idx] = in[sy * n + sx];
  }
}

}  // namespace

extern "C" {

int r2d3c_regrid_spectral(r2d3c_ctx* src, r2d3c_ctx* dst) {
  API_BEGIN
  REQUIRE(src && dst, "NULL argument");
  REQUIRE(dst->p.n > src->p.n, "the destination grid must be finer than the source grid");
  REQUIRE(src->eng->precision() == dst->eng->precision(), "both contexts must have the same precision");
  src->eng->sync();
  IEngine* e = dst->eng.get();
  e->refine_from(src->eng.get(), P_PS, P_PS);
  e->refine_from(src->eng.get(), P_VZ, P_VZ);
  e->mark_state_untruncated();
  e->sync();
  API_END
}

int r2d3c_regrid_physical_dev(int n, int m, const double* d_in, double* d_out, void* stream) {
  API_BEGIN
  REQUIRE(d_in && d_out, "NULL argument");
  REQUIRE(n >= 1 && m > n && m <= 2 * n, "sizes must satisfy n < m <= 2n");
  const size_t total = (size_t)m * m;
  const int blocks = (int)std::min<size_t>((total + 255) / 256, 65535);
  k_regrid_phys<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_in, n, d_out, m);
  cuda_check(cudaGetLastError(), "k_regrid_phys");
  API_END
}

int r2d3c_regrid_physical(int n, int m, const double* in, double* out) {
  API_BEGIN
  REQUIRE(in && out, "NULL argument");
  REQUIRE(n >= 1 && m > n && m <= 2 * n, "sizes must satisfy n < m <= 2n");
  double *d_in = nullptr, *d_out = nullptr;
  const size_t bi = sizeof(double) * (size_t)n * n, bo = sizeof(double) * (size_t)m * m;
  cudaError_t err = cudaMalloc(&d_in, bi);
  if (err == cudaSuccess) err = cudaMalloc(&d_out, bo);
  if (err == cudaSuccess) err = cudaMemcpy(d_in, in, bi, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) {
    const size_t total = (size_t)m * m;
    k_regrid_phys<<<(int)std::min<size_t>((total + 255) / 256, 65535), 256>>>(d_in, n, d_out, m);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpy(out, d_out, bo, cudaMemcpyDeviceToHost);
  if (d_in) cudaFree(d_in);
  if (d_out) cudaFree(d_out);
  cuda_check(err, "regrid_physical");
  API_END
}

int r2d3c_closure_set_tendency(r2d3c_ctx* ctx, const float* d_t) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  ctx->eng->set_closure(d_t, true);
  API_END
}

int r2d3c_closure_set_band(r2d3c_ctx* ctx, const float* w, int nshells) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  REQUIRE(nshells >= 0 && nshells <= ctx->p.n / 2 + 1, "nshells must be in [0, n/2+1]");
  REQUIRE(nshells == 0 || w, "NULL weights");
  ctx->eng->set_closure_band(w, nshells);
  API_END
}

int r2d3c_closure_advance(r2d3c_ctx* ctx, r2d3c_cnn* cnn, int nsteps, int dt_mode, double cfl_or_dt,
                          double* time, double* dt_last) {
  return r2d3c_closure_advance_every(ctx, cnn, nsteps, 1, dt_mode, cfl_or_dt, time, dt_last);
}

namespace {
// the LES steps of r2d3c_closure_advance_every / _overlapped
int closure_advance_impl(r2d3c_ctx* ctx, r2d3c_cnn* cnn, int nsteps, int every, bool overlap, int dt_mode,
                         double cfl_or_dt, double* time, double* dt_last) {
  API_BEGIN
  REQUIRE(ctx && cnn, "NULL argument");
  REQUIRE(nsteps >= 0, "nsteps must be >= 0");
  REQUIRE(every >= 1 && nsteps % every == 0, "every must be >= 1 and divide nsteps");
  REQUIRE(dt_mode == R2D3C_DT_CFL || dt_mode == R2D3C_DT_FIXED, "bad dt_mode");
  REQUIRE(cfl_or_dt > 0.0 && std::isfinite(cfl_or_dt), "cfl_or_dt must be positive and finite");
  REQUIRE(ctx->p.iflow == 0 || ctx->p.iflow == 1, "the closure advance takes constant forcing (iflow 0 or 1)");
  int H = 0, W = 0, bmax = 0;
  unsigned long long serial = 0;
  cnn_shape(cnn, &H, &W, &bmax, &serial);
  const int n = ctx->p.n;
  REQUIRE(H == n && W == n, "the network's grid must be the context's n x n");
  IEngine* e = ctx->eng.get();
  REQUIRE(!overlap || e->closure_fused(), "the overlapped LES step takes the fused closure path (n <= 512)");
  if (!ctx->cl_x) {
    cuda_check(cudaMalloc(&ctx->cl_x, sizeof(float) * 8 * (size_t)n * n), "cudaMalloc closure inputs");
    cuda_check(cudaMalloc(&ctx->cl_t, sizeof(float) * 2 * (size_t)n * n), "cudaMalloc closure tendencies");
  }
  cuda_check(cudaMemsetAsync(ctx->cl_t, 0, sizeof(float) * 2 * (size_t)n * n, (cudaStream_t)e->stream()),
             "memset");
  e->set_closure(ctx->cl_t, true);  // closure on; the hook refreshes the tendencies before every step
  float* x = ctx->cl_x;
  float* t = ctx->cl_t;
  if (e->closure_fused()) {
    // inputs straight into the network's first activation, tendencies
    // straight from its output: two conversion kernels fewer on each side
    void* act0 = nullptr;
    const float* out = nullptr;
    const float* norm = nullptr;
    cnn_io(cnn, &act0, &out, &norm);
    e->set_step_hook(
        [e, cnn, act0, out, norm](cudaStream_t s) {
          e->closure_inputs_cnn(act0, norm, norm + 8);
          cnn_layers_on(cnn, 1, s);
          e->set_closure_cnn(out, norm + 16, norm + 18);
        },
        serial);
  } else {
    e->set_step_hook(
        [e, cnn, x, t](cudaStream_t s) {
          e->closure_inputs(x, false);
          cnn_forward_on(cnn, x, 1, t, s);
          e->set_closure(t, false);
        },
        serial);
  }
  try {
    if (dt_mode == R2D3C_DT_FIXED) e->set_dt(cfl_or_dt);
    e->set_hook_every(every);
    e->set_hook_overlap(overlap);
    e->advance(ctx->mc(), nsteps, dt_mode == R2D3C_DT_CFL, cfl_or_dt, nullptr);
  } catch (...) {
    e->set_hook_every(1);
    e->set_hook_overlap(false);
    e->set_step_hook(nullptr, 0);
    e->set_closure(nullptr, true);
    throw;
  }
  e->set_hook_every(1);
  e->set_hook_overlap(false);
  e->set_step_hook(nullptr, 0);
  e->set_closure(nullptr, true);
  if (time) *time = e->get_time();
  if (dt_last) *dt_last = e->get_dt();
  e->sync();
  cnn_check_err(cnn);
  API_END
}
}  // namespace

int r2d3c_closure_advance_every(r2d3c_ctx* ctx, r2d3c_cnn* cnn, int nsteps, int every, int dt_mode,
                                double cfl_or_dt, double* time, double* dt_last) {
  return closure_advance_impl(ctx, cnn, nsteps, every, false, dt_mode, cfl_or_dt, time, dt_last);
}

int r2d3c_closure_advance_overlapped(r2d3c_ctx* ctx, r2d3c_cnn* cnn, int nsteps, int dt_mode, double cfl_or_dt,
                                     double* time, double* dt_last) {
  return closure_advance_impl(ctx, cnn, nsteps, 1, true, dt_mode, cfl_or_dt, time, dt_last);
}

int r2d3c_plan_report(r2d3c_ctx* ctx, char* buf, int len) {
  API_BEGIN
  REQUIRE(ctx && buf && len > 0, "NULL argument");
  const std::string r = ctx->eng->plan_report();
  const size_t k = std::min(r.size(), (size_t)len - 1);
  std::memcpy(buf, r.data(), k);
  buf[k] = 0;
  REQUIRE(r.size() < (size_t)len, "buffer too small for the report");
  API_END
}

int r2d3c_dev_ptr(r2d3c_ctx* ctx, int which, void** ptr) {
  API_BEGIN
  REQUIRE(ctx && ptr, "NULL argument");
  REQUIRE(which >= 0 && which <= 3, "which must be 0..3");
  *ptr = ctx->eng->plane_ptr(which);
  API_END
}

int r2d3c_stream(r2d3c_ctx* ctx, void** stream) {
  API_BEGIN
  REQUIRE(ctx && stream, "NULL argument");
  *stream = (void*)ctx->eng->stream();
  API_END
}

int r2d3c_synchronize(r2d3c_ctx* ctx) {
  API_BEGIN
  REQUIRE(ctx, "NULL argument");
  ctx->eng->sync();
  API_END
}

}  // extern "C"

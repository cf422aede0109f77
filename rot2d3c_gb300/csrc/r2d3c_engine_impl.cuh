// Device engine of one Rot2D3C context, templated on the compute type
// (double: the FP64 drop-in path; float: the FP32 path with compensated
// twiddles and FP64 reductions).  Included by one translation unit per type.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

#include "r2d3c_aux.cuh"
#include "r2d3c_engine.h"

namespace r2d3c {

template <typename F>
void dispatch_n(int n, F&& f) {
  switch (n) {
    case 16: f(std::integral_constant<int, 16>{}); break;
    case 32: f(std::integral_constant<int, 32>{}); break;
    case 64: f(std::integral_constant<int, 64>{}); break;
    case 128: f(std::integral_constant<int, 128>{}); break;
    case 256: f(std::integral_constant<int, 256>{}); break;
    case 512: f(std::integral_constant<int, 512>{}); break;
    case 1024: f(std::integral_constant<int, 1024>{}); break;
    case 2048: f(std::integral_constant<int, 2048>{}); break;
    case 4096: f(std::integral_constant<int, 4096>{}); break;
    case 8192: f(std::integral_constant<int, 8192>{}); break;
    default: throw Error(kEINVAL, "unsupported grid size n");
  }
}

template <typename K>
inline void set_smem_attr(K kernel, size_t smem) {
  if (smem > 48 * 1024)
    cuda_check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
               "cudaFuncSetAttribute(max dynamic smem)");
}

// max over x of r1^2 + r2^2 (CFL_condition :867-874), encoded for atomicMax
template <typename T>
__global__ void k_max_sq2(const T* __restrict__ r1, const T* __restrict__ r2, size_t count,
                          unsigned long long* enc) {
  double m = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
       i += (size_t)gridDim.x * blockDim.x) {
    const double a = (double)r1[i], b = (double)r2[i];
    m = fmax(m, a * a + b * b);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(enc, enc_ordered(m));
}

// rand_force for step *ctr of a precomputed sequence (graph replay)
template <typename T>
__global__ void k_randforce_seq(cpx<T>* fp, cpx<T>* fz, const double* __restrict__ scal,
                                const RandForceArgs* __restrict__ seq, int* ctr) {
  const int s = *ctr;
  const RandForceArgs a = seq[s];
  const double dt = scal[0];
  for (int fi = 0; fi < 2; ++fi) {
    cpx<T>* dst = fi == 0 ? fp : fz;
    const RandForceField& f = a.f[fi];
    for (int c = 0; c < f.nclear; ++c) dst[f.clear[c]] = czero<T>();
    const double tmp = __ddiv_rn(f.c0, __dmul_rn(sqrt(dt), f.kpow));
    const double t1 = __dmul_rn(__dmul_rn(tmp, f.cph), a.nsq);
    const double t2 = __dmul_rn(__dmul_rn(tmp, f.sph), a.nsq);
    for (int c = 0; c < f.nset; ++c) dst[f.set[c]] = mkc<T>((T)t1, (T)(f.conj[c] ? -t2 : t2));
  }
  *ctr = s + 1;
}

template <typename T>
class EngineT final : public IEngine {
 public:
  EngineT(int n, int device, bool full, int nb = 1) : n_(n), dev_(device), full_(full), nb_(nb) {
    if (nb < 1 || (nb > 1 && !full)) throw Error(kEINVAL, "bad batch size");
    if (!supported_n(n)) throw Error(kEINVAL, "unsupported grid size n");
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    cuda_check(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute");
    cuda_check(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking), "cudaStreamCreate");
    gd_.n = n;
    gd_.nh = n / 2 + 1;
    const double kmax = ((double)n / 3.0) * ((double)n / 3.0);  // (n/3)**2
    gd_.kmaxi = (int)std::floor(kmax);
    gd_.L = (int)std::floor((double)n / 3.0);
    gd_.M = gd_.L + 1;
    S_ = (size_t)gd_.nh * n;
    try {
      for (int p = 0; p < P_COUNT; ++p)
        if (full || p == P_W1) pbase_[p] = planes_[p] = alloc<cpx<T>>(S_ * (batched(p) ? nb_ : 1));
      for (int r = 0; r < R_COUNT; ++r)
        if (full || r == R_1) rplanes_[r] = alloc<T>((size_t)n * n);
      if (full) {
        tf_ = alloc<cpx<T>>((size_t)6 * gd_.M * n * nb_);
        pb_ = alloc<cpx<T>>(2 * S_ * nb_);
      }
      tg_ = alloc<cpx<T>>(S_);
      tw_ = alloc<tw_t<T>>((size_t)n);
      tw_a_ = alloc<tw_t<T>>((size_t)n);  // pass A's stage schedule
      stage_count_ = std::max(2 * S_, (size_t)n * n);
      if (!std::is_same<T, double>::value) stage64_ = alloc<double>(stage_count_);
      scal_base_ = scal_ = alloc<double>((size_t)kScalStride * nb_);
      enc_base_ = enc_ = alloc<unsigned long long>((size_t)kScalStride * nb_);
      d_sc_ = alloc<StepCoef>(nb_);
      d_cfl_ = alloc<CflCoef>(nb_);
      dirty_.assign(nb_, 0);
      partials_ = alloc<double>((size_t)kSumBlocks * kMaxTerms);
      small_ = alloc<double>((size_t)kMaxTerms + 5 * (size_t)gd_.nh);
      cuda_check(cudaMallocHost(&hsmall_, sizeof(double) * (kMaxTerms + 5 * (size_t)gd_.nh + 16)),
                 "cudaMallocHost");
      cuda_check(cudaMemsetAsync(scal_base_, 0, kScalStride * nb_ * sizeof(double), st_), "memset");
      for (int p = 0; p < P_COUNT; ++p)
        if (pbase_[p])
          cuda_check(cudaMemsetAsync(pbase_[p], 0, S_ * (batched(p) ? nb_ : 1) * sizeof(cpx<T>), st_),
                     "memset plane");
      build_twiddles();
      set_kernel_attrs();
      if (full) autotune();
      sync();
    } catch (...) {
      release();
      throw;
    }
  }
  ~EngineT() override { release(); }

  int n() const override { return n_; }
  int precision() const override { return std::is_same<T, double>::value ? 0 : 1; }
  cudaStream_t stream() const override { return st_; }
  void* plane_ptr(int p) override { return planes_[p]; }
  void* rplane_ptr(int r) override { return rplanes_[r]; }
  size_t bytes_allocated() const override { return bytes_; }
  int kernel_launches() const override { return launches_; }

  // ---------------------------------------------------------------- transfers
  void upload_spec(int p, const double* host) override {
    if (std::is_same<T, double>::value) {
      cuda_check(cudaMemcpyAsync(planes_[p], host, S_ * 2 * sizeof(double), cudaMemcpyHostToDevice, st_),
                 "H2D spec");
    } else {
      cuda_check(cudaMemcpyAsync(stage64_, host, S_ * 2 * sizeof(double), cudaMemcpyHostToDevice, st_),
                 "H2D spec");
      convert(stage64_, reinterpret_cast<T*>(planes_[p]), 2 * S_);
    }
    sync();
  }
  void download_spec(int p, double* host) override {
    if (std::is_same<T, double>::value) {
      cuda_check(cudaMemcpyAsync(host, planes_[p], S_ * 2 * sizeof(double), cudaMemcpyDeviceToHost, st_),
                 "D2H spec");
    } else {
      convert(reinterpret_cast<const T*>(planes_[p]), stage64_, 2 * S_);
      cuda_check(cudaMemcpyAsync(host, stage64_, S_ * 2 * sizeof(double), cudaMemcpyDeviceToHost, st_),
                 "D2H spec");
    }
    sync();
  }
  void upload_real(int r, const double* host) override {
    const size_t cnt = (size_t)n_ * n_;
    if (std::is_same<T, double>::value) {
      cuda_check(cudaMemcpyAsync(rplanes_[r], host, cnt * sizeof(double), cudaMemcpyHostToDevice, st_), "H2D real");
    } else {
      cuda_check(cudaMemcpyAsync(stage64_, host, cnt * sizeof(double), cudaMemcpyHostToDevice, st_), "H2D real");
      convert(stage64_, rplanes_[r], cnt);
    }
    sync();
  }
  void download_real(int r, double* host) override {
    const size_t cnt = (size_t)n_ * n_;
    if (std::is_same<T, double>::value) {
      cuda_check(cudaMemcpyAsync(host, rplanes_[r], cnt * sizeof(double), cudaMemcpyDeviceToHost, st_), "D2H real");
    } else {
      convert(rplanes_[r], stage64_, cnt);
      cuda_check(cudaMemcpyAsync(host, stage64_, cnt * sizeof(double), cudaMemcpyDeviceToHost, st_), "D2H real");
    }
    sync();
  }
  void spec_from_dev64(int p, const double* dev) override {
    if (std::is_same<T, double>::value)
      cuda_check(cudaMemcpyAsync(planes_[p], dev, S_ * 2 * sizeof(double), cudaMemcpyDeviceToDevice, st_), "D2D");
    else
      convert(dev, reinterpret_cast<T*>(planes_[p]), 2 * S_);
  }
  void spec_to_dev64(int p, double* dev) override {
    if (std::is_same<T, double>::value)
      cuda_check(cudaMemcpyAsync(dev, planes_[p], S_ * 2 * sizeof(double), cudaMemcpyDeviceToDevice, st_), "D2D");
    else
      convert(reinterpret_cast<const T*>(planes_[p]), dev, 2 * S_);
  }
  void real_from_dev64(int r, const double* dev) override {
    const size_t cnt = (size_t)n_ * n_;
    if (std::is_same<T, double>::value)
      cuda_check(cudaMemcpyAsync(rplanes_[r], dev, cnt * sizeof(double), cudaMemcpyDeviceToDevice, st_), "D2D");
    else
      convert(dev, rplanes_[r], cnt);
  }
  void real_to_dev64(int r, double* dev) override {
    const size_t cnt = (size_t)n_ * n_;
    if (std::is_same<T, double>::value)
      cuda_check(cudaMemcpyAsync(dev, rplanes_[r], cnt * sizeof(double), cudaMemcpyDeviceToDevice, st_), "D2D");
    else
      convert(rplanes_[r], dev, cnt);
  }

  // ---------------------------------------------------------------- operators
  void specop(int src, int dst, int op, double s) override {
    k_specop<T><<<elem_blocks(S_), 256, 0, st_>>>(planes_[src], planes_[dst], gd_, op, s);
    post("k_specop");
  }
  void zero_spec(int p) override {
    cuda_check(cudaMemsetAsync(planes_[p], 0, S_ * sizeof(cpx<T>), st_), "memset plane");
  }
  void r2c(int rsrc, int dst) override {
    launch_rowr2c(rplanes_[rsrc], tg_);
    launch_colfft<-1>(tg_, planes_[dst], gd_.nh);
  }
  void c2r(int src, int rdst, double* mx, double* mn) override {
    launch_colfft<+1>(planes_[src], tg_, gd_.nh);
    if (mx) cuda_check(cudaMemsetAsync(enc_ + 1, 0, 2 * sizeof(unsigned long long), st_), "memset");
    launch_rowc2r(tg_, rdst >= 0 ? rplanes_[rdst] : nullptr, mx ? enc_ + 1 : nullptr);
    if (mx) {
      unsigned long long e[2];
      cuda_check(cudaMemcpyAsync(e, enc_ + 1, sizeof(e), cudaMemcpyDeviceToHost, st_), "D2H minmax");
      sync();
      *mx = dec_host(e[0]);
      *mn = -dec_host(e[1]);
    }
  }
  void poisson(int a, int b, int c) override {
    const size_t cnt = (size_t)n_ * n_;
    const double inv4 = 1.0 / ((double)n_ * n_ * n_ * n_);
    specop(a, P_W1, OP_DERIV_X, 0.0);
    specop(b, P_W2, OP_DERIV_Y, 0.0);
    c2r(P_W1, R_1, nullptr, nullptr);
    c2r(P_W2, R_2, nullptr, nullptr);
    k_realprod<T><<<elem_blocks(cnt), 256, 0, st_>>>(rplanes_[R_3], rplanes_[R_1], rplanes_[R_2], cnt, 0, 1.0);
    post("k_realprod");
    specop(a, P_W1, OP_DERIV_Y, 0.0);
    specop(b, P_W2, OP_DERIV_X, 0.0);
    c2r(P_W1, R_1, nullptr, nullptr);
    c2r(P_W2, R_2, nullptr, nullptr);
    k_realprod<T><<<elem_blocks(cnt), 256, 0, st_>>>(rplanes_[R_3], rplanes_[R_1], rplanes_[R_2], cnt, 1, inv4);
    post("k_realprod");
    r2c(R_3, c);
  }
  void halfplane_sums(int nterms, const int* kind, const int* ia, const int* ib, const int* kin,
                      double band_lo, double band_hi, const int* planes4, double* out) override {
    enqueue_sums(nterms, kind, ia, ib, kin, band_lo, band_hi, planes4);
    cuda_check(cudaMemcpyAsync(hsmall_, small_, nterms * sizeof(double), cudaMemcpyDeviceToHost, st_), "D2H sums");
    sync();
    std::memcpy(out, hsmall_, nterms * sizeof(double));
  }
  // sums into small_[0..nterms) on the device
  void enqueue_sums(int nterms, const int* kind, const int* ia, const int* ib, const int* kin,
                    double band_lo, double band_hi, const int* planes4) {
    if (nterms < 1 || nterms > kMaxTerms) throw Error(kEINVAL, "bad number of sum terms");
    SumList sl;
    std::memset(&sl, 0, sizeof(sl));
    sl.nterms = nterms;
    for (int t = 0; t < nterms; ++t) sl.t[t] = SumTerm{kind[t], ia[t], ib[t], kin[t]};
    sl.band_lo = band_lo;
    sl.band_hi = band_hi;
    const cpx<T>* p[4];
    for (int i = 0; i < 4; ++i) p[i] = planes4[i] >= 0 ? planes_[planes4[i]] : nullptr;
    k_halfplane_sums<T><<<kSumBlocks, kSumThreads, 0, st_>>>(p[0], p[1], p[2], p[3], gd_, sl, partials_);
    post("k_halfplane_sums");
    const double inv4 = 1.0 / ((double)n_ * n_ * n_ * n_);
    k_finalize_sums<<<1, 32, 0, st_>>>(partials_, kSumBlocks, nterms, inv4, small_);
    post("k_finalize_sums");
  }

  void set_const_inj(bool on, double kdn, double kup, double fp0, double fz0,
                     const std::vector<int>& band_idx, const std::vector<int>& mirror,
                     const std::vector<float>& rnd) override {
    ci_on_ = false;
    for (void* p : {(void*)ci_idx_, (void*)ci_mir_, (void*)ci_rnd_})
      if (p) cudaFree(p);
    ci_idx_ = nullptr;
    ci_mir_ = nullptr;
    ci_rnd_ = nullptr;
    ci_n_ = (int)band_idx.size();
    ci_lo_ = kdn * kdn;
    ci_hi_ = kup * kup;
    ci_fp0_ = fp0;
    ci_fz0_ = fz0;
    const size_t c = std::max<size_t>(band_idx.size(), 1);
    cuda_check(cudaMalloc(&ci_idx_, c * sizeof(int)), "cudaMalloc band");
    cuda_check(cudaMalloc(&ci_mir_, c * sizeof(int)), "cudaMalloc band");
    cuda_check(cudaMalloc(&ci_rnd_, c * sizeof(float)), "cudaMalloc band");
    if (ci_n_ > 0) {
      cuda_check(cudaMemcpyAsync(ci_idx_, band_idx.data(), ci_n_ * sizeof(int), cudaMemcpyHostToDevice, st_), "H2D");
      cuda_check(cudaMemcpyAsync(ci_mir_, mirror.data(), ci_n_ * sizeof(int), cudaMemcpyHostToDevice, st_), "H2D");
      cuda_check(cudaMemcpyAsync(ci_rnd_, rnd.data(), ci_n_ * sizeof(float), cudaMemcpyHostToDevice, st_), "H2D");
    }
    sync();
    ci_on_ = on;
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
  }
  void const_inj(int src, int dst, int kin, double f0) override {
    if (!ci_idx_) throw Error(kESTATE, "const_inj band not configured");
    enqueue_const_inj(planes_[src], src, dst, kin, f0);
  }
  void enqueue_const_inj(const cpx<T>* srcp, int src_slot_plane, int dst, int kin, double f0) {
    k_ci_base<T><<<elem_blocks(S_), 256, 0, st_>>>(srcp, planes_[dst], gd_, ci_lo_, ci_hi_);
    post("k_ci_base");
    // Efp = inerprod(ps, fp, kin) (:1030), kept on the device
    const int kind = S_INERPROD, ia = 0, ib = 1;
    const int pl[4] = {src_slot_plane, dst, -1, -1};
    enqueue_sums(1, &kind, &ia, &ib, &kin, 0.0, 0.0, pl);
    if (ci_n_ > 0) {
      k_ci_rescale<T><<<(ci_n_ + 255) / 256, 256, 0, st_>>>(srcp, planes_[dst], ci_idx_, ci_mir_, ci_rnd_,
                                                            ci_n_, f0, small_, n_);
      post("k_ci_rescale");
    }
  }
  void brackets_full() {
    // [psi, -k^2 psi] -> B5 and [psi, vz] -> B6 over the whole half plane
    launch_passA(planes_[P_PS], planes_[P_VZ], tf_, 1);
    launch_passB<false>(gd_.nh, tf_, pb_, 1);
    launch_colfft_mixed(pb_, planes_[P_B5]);
    launch_colfft_mixed(pb_ + S_, planes_[P_B6]);
  }
  void shells(bool transfers, double* out5) override {
    if (transfers) brackets_full();
    const double inv4 = 1.0 / ((double)n_ * n_ * n_ * n_);
    double* dout = small_ + kMaxTerms;
    k_shells<T><<<gd_.nh, kShellThreads, 0, st_>>>(planes_[P_PS], planes_[P_VZ],
                                                    transfers ? planes_[P_B5] : nullptr,
                                                    transfers ? planes_[P_B6] : nullptr, gd_, inv4, dout);
    post("k_shells");
    cuda_check(cudaMemcpyAsync(hsmall_, dout, 5 * (size_t)gd_.nh * sizeof(double), cudaMemcpyDeviceToHost, st_),
               "D2H shells");
    sync();
    std::memcpy(out5, hsmall_, 5 * (size_t)gd_.nh * sizeof(double));
  }
  CflCoef cfl_coef(double cfl, const ModelCoef& mc) const {
    CflCoef c;
    c.cfl = cfl;
    c.kcut = (double)n_ / 3.0;
    c.nrm = (double)n_ * (double)n_;
    c.nuk = mc.nu * ipow(c.kcut, 2 * mc.nn);
    c.nuvk = mc.nuv * ipow(c.kcut, 2 * mc.nnv);
    c.w2 = 2 * mc.omega;
    return c;
  }
  double cfl(double cfl, const ModelCoef& mc) override {
    const size_t cnt = (size_t)n_ * n_;
    specop(P_PS, P_W1, OP_DERIV_X, 0.0);
    specop(P_PS, P_W2, OP_DERIV_Y, 0.0);
    c2r(P_W1, R_1, nullptr, nullptr);
    c2r(P_W2, R_2, nullptr, nullptr);
    cuda_check(cudaMemsetAsync(enc_, 0, sizeof(unsigned long long), st_), "memset");
    k_max_sq2<T><<<elem_blocks(cnt), 256, 0, st_>>>(rplanes_[R_1], rplanes_[R_2], cnt, enc_);
    post("k_max_sq2");
    const CflCoef cc = cfl_coef(cfl, mc);
    cuda_check(cudaMemcpyAsync(d_cfl_ + run_, &cc, sizeof(cc), cudaMemcpyHostToDevice, st_), "H2D cfl coef");
    coefs_valid_ = false;  // the device coefficients differ from the last upload_coefs
    k_cfl_dt<<<1, 1, 0, st_>>>(enc_, d_cfl_ + run_, scal_, 0, 1);
    post("k_cfl_dt");
    return get_dt();
  }

  // ---------------------------------------------------------------- hot path
  void set_dt(double dt) override { set_scal(0, dt); }
  void set_time(double t) override { set_scal(1, t); }
  double get_dt() override { return get_scal(0); }
  double get_time() override { return get_scal(1); }
  void get_dt_time(double* dt, double* time) override {
    cuda_check(cudaMemcpyAsync(hsmall_, scal_, 2 * sizeof(double), cudaMemcpyDeviceToHost, st_), "D2H scal");
    sync();
    *dt = hsmall_[0];
    *time = hsmall_[1];
  }
  void mark_state_untruncated() override { dirty_[run_] = 1; }
  int nruns() const override { return nb_; }
  void select_run(int r) override {
    if (r < 0 || r >= nb_) throw Error(kEINVAL, "run index out of range");
    run_ = r;
    for (int p = 0; p < P_COUNT; ++p)
      if (pbase_[p] && batched(p)) planes_[p] = pbase_[p] + (size_t)r * S_;
    scal_ = scal_base_ + (size_t)r * kScalStride;
    enc_ = enc_base_ + (size_t)r * kScalStride;
  }
  void set_run_coefs(const std::vector<ModelCoef>& mc) override {
    if ((int)mc.size() != nb_) throw Error(kEINVAL, "one coefficient set per run");
    coefs_ = mc;
  }
  void set_dt_all(double dt) override {
    std::vector<double> h((size_t)kScalStride * nb_);
    cuda_check(cudaMemcpyAsync(h.data(), scal_base_, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st_),
               "D2H scal");
    sync();
    for (int r = 0; r < nb_; ++r) h[(size_t)r * kScalStride] = dt;
    cuda_check(cudaMemcpyAsync(scal_base_, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st_),
               "H2D scal");
    sync();
  }
  void prepare_steps(double cfl) override {
    truncate_if_dirty();
    upload_coefs(coefs_.empty() ? ModelCoef{} : coefs_[0], cfl);
  }
  void enqueue_steps(bool cfl_mode) override { enqueue_step(cfl_mode, true, 0, nullptr); }
  void get_scalars(double* dt, double* time) override {
    std::vector<double> h((size_t)kScalStride * nb_);
    cuda_check(cudaMemcpyAsync(h.data(), scal_base_, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st_),
               "D2H scal");
    sync();
    for (int r = 0; r < nb_; ++r) {
      if (dt) dt[r] = h[(size_t)r * kScalStride];
      if (time) time[r] = h[(size_t)r * kScalStride + 1];
    }
  }

  void rand_force(const RandForceHost f[2]) override {
    RandForceArgs a = make_rf_args(f);
    k_randforce<T><<<1, 1, 0, st_>>>(planes_[P_FP], planes_[P_FZ], scal_, a);
    post("k_randforce");
  }

  void step(const ModelCoef& mc, bool cfl_mode, double cfl, bool add_time,
            const RandForceHost* rf) override {
    truncate_if_dirty();
    upload_coefs(mc, cfl);
    enqueue_step(cfl_mode, add_time, rf ? 1 : 0, rf);
  }

  void advance(const ModelCoef& mc, int nsteps, bool cfl_mode, double cfl,
               const RandForceHost* rf) override {
    if (nsteps <= 0) return;
    truncate_if_dirty();
    if (rf) {
      if (rf_cap_ < nsteps) {
        if (d_rf_) cudaFree(d_rf_);
        d_rf_ = nullptr;
        rf_cap_ = 0;
        cuda_check(cudaMalloc(&d_rf_, sizeof(RandForceArgs) * (size_t)nsteps), "cudaMalloc rf");
        rf_cap_ = nsteps;
        if (!d_ctr_) cuda_check(cudaMalloc(&d_ctr_, sizeof(int)), "cudaMalloc ctr");
      }
      std::vector<RandForceArgs> seq((size_t)nsteps);
      for (int s = 0; s < nsteps; ++s) seq[s] = make_rf_args(rf + 2 * s);
      cuda_check(cudaMemcpyAsync(d_rf_, seq.data(), sizeof(RandForceArgs) * (size_t)nsteps,
                                 cudaMemcpyHostToDevice, st_), "H2D rf");
      cuda_check(cudaMemsetAsync(d_ctr_, 0, sizeof(int), st_), "memset ctr");
      sync();  // seq goes out of scope
    }
    upload_coefs(mc, cfl);
    const int every = hook_ ? hook_every_ : 1;
    const bool overlap = hook_ && hook_overlap_;
    if (nsteps % every != 0) throw Error(kEINVAL, "nsteps must be a multiple of the hook interval");
    if (every > 1 && rf) throw Error(kEINVAL, "a hook interval above 1 takes constant forcing");
    if (overlap && (every != 1 || rf || !ov_stream_))
      throw Error(kEINVAL, "an overlapped hook takes interval 1, constant forcing and the closure scratch");
    // overlapped: the first step of the call takes the hook's result for its
    // own state, queued here outside the graph
    if (overlap) hook_(st_);
    // pass C with the next substep's pass A: the graph's steps start at pass
    // B, and the first pass A of the call is queued here
    const bool fuse = fuse_ca();
    if (fuse) launch_passA(pbase_[P_PS], pbase_[P_VZ], tf_, nb_);
    GraphKey key{cfl_mode, rf != nullptr, closure_on_, band_nw_ > 0, hook_ ? hook_id_ : 0ull, every, overlap, fuse};
    if (!graph_ || !key.same(gkey_)) {
      if (graph_) cudaGraphExecDestroy(graph_);
      graph_ = nullptr;
      cudaGraph_t g = nullptr;
      const int before = launches_;
      cuda_check(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal), "BeginCapture");
      cudaStream_t main = st_;
      try {
        if (overlap) {
          // The hook on a forked stream, beside the step: it reads the state
          // the step starts from (the step's last pass C, which overwrites
          // it, waits for the inputs kernel) and writes the next step's
          // tendencies into their own planes, copied (band-weighted) into
          // the live ones after the join
          cuda_check(cudaEventRecord(ov_fork_, main), "event fork");
          cuda_check(cudaStreamWaitEvent(ov_stream_, ov_fork_, 0), "wait fork");
          st_ = ov_stream_;
          ov_capture_ = true;
          hook_(st_);
          ov_capture_ = false;
          st_ = main;
          ov_wait_ = true;
          enqueue_step(cfl_mode, true, 0, nullptr, fuse);
          ov_wait_ = false;
          cuda_check(cudaEventRecord(ov_join_, ov_stream_), "event join");
          cuda_check(cudaStreamWaitEvent(main, ov_join_, 0), "wait join");
          k_shell_weight2<T><<<elem_blocks(S_), 256, 0, st_>>>(cl_tn_, cl_tn_ + S_, planes_[P_T5], planes_[P_T6], gd_,
                                                               band_w_, band_nw_);
          post("k_shell_weight2");
        } else {
          if (hook_) hook_(st_);
          for (int k = 0; k < every; ++k) enqueue_step(cfl_mode, true, rf ? -1 : 0, nullptr, fuse);
        }
      } catch (...) {
        st_ = main;
        ov_capture_ = ov_wait_ = false;
        cudaStreamEndCapture(st_, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      cuda_check(cudaStreamEndCapture(st_, &g), "EndCapture");
      cuda_check(cudaGraphInstantiate(&graph_, g, 0), "GraphInstantiate");
      cudaGraphDestroy(g);
      graph_launches_ = launches_ - before;
      launches_ = before;
      gkey_ = key;
    }
    for (int s = 0; s < nsteps; s += every) {
      cuda_check(cudaGraphLaunch(graph_, st_), "GraphLaunch");
      launches_ += graph_launches_;
    }
  }
  void set_hook_every(int k) override {
    if (k < 1) throw Error(kEINVAL, "hook interval must be >= 1");
    hook_every_ = k;
  }
  void set_hook_overlap(bool on) override { hook_overlap_ = on; }

  void initial_condition_phys(const std::vector<IcModeHost>& modes) override {
    IcMode* d = nullptr;
    const size_t bytes = sizeof(IcMode) * std::max<size_t>(modes.size(), 1);
    cuda_check(cudaMalloc(&d, bytes), "cudaMalloc ic modes");
    std::vector<IcMode> hm(modes.size());
    for (size_t i = 0; i < modes.size(); ++i)
      hm[i] = IcMode{modes[i].kr, modes[i].ph1, modes[i].ph2, modes[i].ph3, modes[i].ph4, modes[i].ir, modes[i].jr};
    try {
      if (!hm.empty())
        cuda_check(cudaMemcpyAsync(d, hm.data(), sizeof(IcMode) * hm.size(), cudaMemcpyHostToDevice, st_), "H2D ic");
      k_ic_phys<T><<<elem_blocks((size_t)n_ * n_), 256, 0, st_>>>(d, (int)hm.size(), n_, kPi,
                                                                   rplanes_[R_1], rplanes_[R_2]);
      post("k_ic_phys");
      sync();
    } catch (...) {
      cudaFree(d);
      throw;
    }
    cudaFree(d);
  }
  void iflow1_phys(double kup) override {
    k_iflow1_phys<T><<<elem_blocks((size_t)n_ * n_), 256, 0, st_>>>(n_, kup, kPi, rplanes_[R_1], rplanes_[R_2]);
    post("k_iflow1_phys");
  }
  void scale_mask2(int a, int b, double sa, double sb) override {
    k_scale_mask2<T><<<elem_blocks(S_), 256, 0, st_>>>(planes_[a], planes_[b], gd_, sa, sb);
    post("k_scale_mask2");
  }
  void sync() override { cuda_check(cudaStreamSynchronize(st_), "cudaStreamSynchronize"); }

  void profile_steps(const ModelCoef& mc, int nsteps, double ms[4], long long cnt[4]) override {
    truncate_if_dirty();
    for (int k = 0; k < 4; ++k) {
      ms[k] = 0.0;
      cnt[k] = 0;
    }
    prof_.clear();
    profiling_ = true;
    try {
      upload_coefs(mc, 0.0);
      for (int s = 0; s < nsteps; ++s) enqueue_step(false, false, 0, nullptr);
    } catch (...) {
      profiling_ = false;
      for (auto& e : prof_) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
      }
      prof_.clear();
      throw;
    }
    profiling_ = false;
    sync();
    for (auto& e : prof_) {
      float t = 0.f;
      cuda_check(cudaEventElapsedTime(&t, e.a, e.b), "cudaEventElapsedTime");
      ms[e.kind] += t;
      cnt[e.kind] += 1;
      cudaEventDestroy(e.a);
      cudaEventDestroy(e.b);
    }
    prof_.clear();
  }

 private:
  static constexpr int kSumBlocks = 304;  // 2 CTAs per SM on 152 SMs
  static constexpr double kPi = 3.1415926535897932384;

  // The captured step depends only on these; coefficients and dt live in
  // device arrays read by the kernels, so changing them needs no recapture.
  struct GraphKey {
    bool cfl_mode = false, rf = false, closure = false, band = false;
    unsigned long long hook = 0;
    int every = 1;         // steps per graph (the hook's interval)
    bool overlap = false;  // the hook beside the step (one step of lag)
    bool fuse = false;     // pass C carries the next substep's pass A
    bool same(const GraphKey& o) const {
      return cfl_mode == o.cfl_mode && rf == o.rf && closure == o.closure && band == o.band && hook == o.hook &&
             every == o.every && overlap == o.overlap && fuse == o.fuse;
    }
  };
  int hook_every_ = 1;
  bool hook_overlap_ = false;
  bool fuse_ca_on_ = true;  // R2D3C_FUSE_CA
  bool ov_capture_ = false;  // the hook is being captured on ov_stream_
  bool ov_wait_ = false;     // the step being captured waits for the hook's inputs kernel
  static bool batched(int p) { return p <= P_C4; }  // ps, vz, fp, fz, c1 .. c4

 public:
  void set_step_hook(std::function<void(cudaStream_t)> hook, unsigned long long id) override {
    hook_ = id ? std::move(hook) : nullptr;
    hook_id_ = id;
  }
  // scratch of the closure's batched transforms: 8 spectral planes, 8 mixed
  // planes, 8 real planes (allocated once, outside any stream capture)
  void closure_scratch() {
    if (cl_t8_) return;
    cl_t8_ = alloc<cpx<T>>(8 * S_);
    cl_r8_ = alloc<T>((size_t)8 * n_ * n_);
    // the overlapped LES step: its own stream, fork / inputs / join events
    // and the next step's two tendency planes
    cl_tn_ = alloc<cpx<T>>(2 * S_);
    cuda_check(cudaStreamCreateWithFlags(&ov_stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    for (cudaEvent_t* e : {&ov_fork_, &ov_in_, &ov_join_})
      cuda_check(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
  }
  void closure_inputs(float* d_x, bool wait) override {
    // omega = -lap psi = k^2 psi, vz, d/dx and d/dy of psi, omega, vz: the 8
    // spectral fields formed as the column transforms load them, one batched
    // row C2R, one interleave into the FP32 NHWC tensor scaled by 1/n^2
    if (wait) closure_scratch();
    if (!cl_t8_) throw Error(kESTATE, "closure scratch not allocated (call before any capture)");
    const size_t cnt = (size_t)n_ * n_;
    const double s = 1.0 / ((double)n_ * n_);
    launch_closure_cols();
    launch_rowc2r(cl_t8_, cl_r8_, nullptr, 8);
    const Scale8 sc{{-s, s, s, s, -s, -s, s, s}};
    k_to_channels8<T><<<elem_blocks(cnt), 256, 0, st_>>>(cl_r8_, cnt, sc, d_x);
    post("k_to_channels8");
    if (wait) sync();
  }
  // pass C carries the next substep's pass A inside advance(): FP32 grids up
  // to 512, one run, no const_inj, one CTA (or team) per column pair;
  // R2D3C_FUSE_CA=0 keeps the separate pass A
  bool fuse_ca() const {
    bool ok = false;
    dispatch_n(n_, [&](auto NC) { ok = kFuseCA<T, decltype(NC)::value>; });
    return ok && fuse_ca_on_ && nb_ == 1 && !ci_on_ && passc_mode_ == 0;
  }
  bool closure_fused() const override {
    bool ok = false;
    dispatch_n(n_, [&](auto NC) { ok = RowsCnn<T, decltype(NC)::value>::OK; });
    return ok && nb_ == 1;
  }
  void closure_inputs_cnn(void* act0, const float* in_mean, const float* in_sd) override {
    if (!cl_t8_) throw Error(kESTATE, "closure scratch not allocated (call before any capture)");
    const double s = 1.0 / ((double)n_ * n_);
    launch_closure_cols();
    // overlapped step: the state has been read, the step may overwrite it
    if (ov_capture_) cuda_check(cudaEventRecord(ov_in_, st_), "event inputs");
    const Scale8 sc{{-s, s, s, s, -s, -s, s, s}};
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      if constexpr (RowsCnn<T, N>::OK) {
        k_rows_to_cnn8<T, N><<<N / 2, RowsCnn<T, N>::THREADS, RowsCnn<T, N>::SMEM, st_>>>(
            cl_t8_, sc, in_mean, in_sd, static_cast<__nv_bfloat16*>(act0), tw_);
        post("k_rows_to_cnn8");
      } else {
        throw Error(kEINVAL, "fused closure path: n too large");
      }
    });
  }
  void set_closure_cnn(const float* y, const float* out_mean, const float* out_sd) override {
    if (!cl_t8_) throw Error(kESTATE, "closure scratch not allocated (call before any capture)");
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      using C = Cfg<T, N>;
      const int g = fft_groups((long long)(N / 2) * 2, C::G);
      k_cnn2_to_rows<T, N><<<dim3((N / 2 + g - 1) / g, 2), C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(
          y, out_mean, out_sd, cl_t8_, tw_);
      post("k_cnn2_to_rows");
    });
    if (ov_capture_) {  // the next step's planes; weighted into the live ones after the join
      launch_colfft<-1>(cl_t8_, cl_tn_, 2 * gd_.nh, cl_tn_ + S_, gd_.nh);
      return;
    }
    if (band_nw_ > 0) {  // both tendency planes, transformed and band-weighted in one launch
      dispatch_n(n_, [&](auto NC) {
        constexpr int N = decltype(NC)::value;
        using C = Cfg<T, N>;
        const int ncols = 2 * gd_.nh, g = fft_groups(ncols, C::G);
        k_colfft_band2<T, N><<<(ncols + g - 1) / g, C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(
            cl_t8_, planes_[P_T5], planes_[P_T6], gd_.nh, tw_, band_w_, band_nw_);
        post("k_colfft_band2");
      });
    } else {
      launch_colfft<-1>(cl_t8_, planes_[P_T5], 2 * gd_.nh, planes_[P_T6], gd_.nh);  // both tendency planes
    }
    closure_on_ = true;
  }
  void set_closure_band(const float* w, int nw) override {
    if (nw < 0 || nw > gd_.nh) throw Error(kEINVAL, "closure band: 0 <= nshells <= n/2+1");
    if (nw > 0 && !w) throw Error(kEINVAL, "closure band: NULL weights");
    if (nw > 0) {
      if (!band_w_) band_w_ = alloc<float>(2 * (size_t)gd_.nh);
      cuda_check(cudaMemcpyAsync(band_w_, w, sizeof(float) * 2 * nw, cudaMemcpyHostToDevice, st_), "band upload");
      sync();
    }
    band_nw_ = nw;
  }
  void brackets() override { brackets_full(); }
  void coarsen_from(IEngine* fine, int fine_plane, int dst_plane) override {
    if (fine->precision() != precision() || fine->n() <= n_) throw Error(kEINVAL, "coarsen: finer grid of the same precision");
    const double r = (double)n_ / (double)fine->n();
    k_coarsen<T><<<elem_blocks(S_), 256, 0, st_>>>(static_cast<const cpx<T>*>(fine->plane_ptr(fine_plane)), fine->n(),
                                                   planes_[dst_plane], gd_, r * r);
    post("k_coarsen");
  }
  void refine_from(IEngine* coarse, int coarse_plane, int dst_plane) override {
    if (coarse->precision() != precision() || coarse->n() >= n_)
      throw Error(kEINVAL, "refine: coarser grid of the same precision");
    const double r = (double)n_ / (double)coarse->n();
    k_refine<T><<<elem_blocks(S_), 256, 0, st_>>>(static_cast<const cpx<T>*>(coarse->plane_ptr(coarse_plane)),
                                                  coarse->n(), planes_[dst_plane], gd_, r * r);
    post("k_refine");
  }
  void closure_targets(IEngine* fine, float* d_y) override {
    // tau = P_c([.,.]_fine) - [.,.]_coarse for both brackets, in physical space
    fine->brackets();
    fine->sync();
    brackets();
    const size_t cnt = (size_t)n_ * n_;
    const double s = 1.0 / ((double)n_ * n_);
    for (int c = 0; c < 2; ++c) {
      coarsen_from(fine, c == 0 ? P_B5 : P_B6, P_W1);
      k_spec_sub<T><<<elem_blocks(S_), 256, 0, st_>>>(planes_[P_W1], planes_[c == 0 ? P_B5 : P_B6], planes_[P_W1], S_);
      post("k_spec_sub");
      c2r(P_W1, R_1, nullptr, nullptr);
      k_to_channel<T><<<elem_blocks(cnt), 256, 0, st_>>>(rplanes_[R_1], cnt, s, d_y, 2, c);
      post("k_to_channel");
    }
    sync();
  }
  void set_closure(const float* d_t, bool wait) override {
    if (!d_t) {
      closure_on_ = false;
      return;
    }
    if (nb_ != 1) throw Error(kEINVAL, "the closure is a single-run feature");
    if (wait) closure_scratch();
    if (!cl_t8_) throw Error(kESTATE, "closure scratch not allocated (call before any capture)");
    // the two channels as two real planes, one batched row R2C, the column
    // transforms into the tendency planes
    const size_t cnt = (size_t)n_ * n_;
    k_from_channels2<T><<<elem_blocks(cnt), 256, 0, st_>>>(d_t, cnt, cl_r8_);
    post("k_from_channels2");
    launch_rowr2c(cl_r8_, cl_t8_, 2);
    launch_colfft<-1>(cl_t8_, planes_[P_T5], 2 * gd_.nh, planes_[P_T6], gd_.nh);  // both tendency planes
    band_weight();
    // the tendency planes are fixed buffers: a captured step keyed on
    // closure_on_ stays valid across calls
    closure_on_ = true;
    if (wait) sync();
  }

 private:
  // the per-shell weights of set_closure_band on both tendency planes
  void band_weight() {
    if (band_nw_ <= 0) return;
    k_shell_weight2<T><<<elem_blocks(S_), 256, 0, st_>>>(planes_[P_T5], planes_[P_T6], planes_[P_T5], planes_[P_T6],
                                                         gd_, band_w_, band_nw_);
    post("k_shell_weight2");
  }
  // per-run coefficient arrays: nb == 1 takes mc, a batch its run coefficients
  // (skipped when the device already holds the same coefficients: a caller
  // that advances one step per call pays no copy and no synchronisation)
  void upload_coefs(const ModelCoef& mc, double cfl) {
    if (nb_ == 1) coefs_.assign(1, mc);
    if ((int)coefs_.size() != nb_) throw Error(kESTATE, "run coefficients not set");
    std::vector<StepCoef> sc(nb_);
    std::vector<CflCoef> cc(nb_);
    for (int r = 0; r < nb_; ++r) {
      const ModelCoef& m = coefs_[r];
      sc[r] = StepCoef{m.nu, m.hnu, m.nuv, m.hnuv, 2 * m.omega, m.nn, m.mm, m.nnv, m.mmv};
      cc[r] = cfl_coef(cfl, m);
    }
    const size_t bs = sizeof(StepCoef) * nb_, bc = sizeof(CflCoef) * nb_;
    if (coefs_valid_ && up_sc_.size() == bs && up_cc_.size() == bc && std::memcmp(up_sc_.data(), sc.data(), bs) == 0 &&
        std::memcmp(up_cc_.data(), cc.data(), bc) == 0)
      return;
    cuda_check(cudaMemcpyAsync(d_sc_, sc.data(), bs, cudaMemcpyHostToDevice, st_), "H2D step coefs");
    cuda_check(cudaMemcpyAsync(d_cfl_, cc.data(), bc, cudaMemcpyHostToDevice, st_), "H2D cfl coefs");
    sync();
    up_sc_.assign(reinterpret_cast<const char*>(sc.data()), reinterpret_cast<const char*>(sc.data()) + bs);
    up_cc_.assign(reinterpret_cast<const char*>(cc.data()), reinterpret_cast<const char*>(cc.data()) + bc);
    coefs_valid_ = true;
  }

  template <typename U>
  U* alloc(size_t count) {
    void* p = nullptr;
    const cudaError_t e = cudaMalloc(&p, count * sizeof(U));
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw Error(kENOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    owned_.push_back(p);
    bytes_ += count * sizeof(U);
    return reinterpret_cast<U*>(p);
  }
  void release() {
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
    for (void* p : owned_) cudaFree(p);
    owned_.clear();
    if (d_rf_) cudaFree(d_rf_);
    if (d_ctr_) cudaFree(d_ctr_);
    for (void* p : {(void*)ci_idx_, (void*)ci_mir_, (void*)ci_rnd_})
      if (p) cudaFree(p);
    ci_idx_ = nullptr;
    ci_mir_ = nullptr;
    ci_rnd_ = nullptr;
    d_rf_ = nullptr;
    d_ctr_ = nullptr;
    if (hsmall_) cudaFreeHost(hsmall_);
    hsmall_ = nullptr;
    for (cudaEvent_t* e : {&ov_fork_, &ov_in_, &ov_join_}) {
      if (*e) cudaEventDestroy(*e);
      *e = nullptr;
    }
    if (ov_stream_) cudaStreamDestroy(ov_stream_);
    ov_stream_ = nullptr;
    if (st_) cudaStreamDestroy(st_);
    st_ = nullptr;
  }
  static unsigned elem_blocks(size_t count) {
    const size_t b = (count + 255) / 256;
    return (unsigned)std::min<size_t>(b, 152 * 16);
  }
  void post(const char* what) {
    ++launches_;
    cuda_check(cudaGetLastError(), what);
  }
  struct ProfEv {
    int kind;
    cudaEvent_t a, b;
  };
  // brackets one launch with events when profiling (kind: 0 A, 1 B, 2 C, 3 other)
  template <typename F>
  void timed(int kind, F&& launch) {
    if (!profiling_) {
      launch();
      return;
    }
    ProfEv e{kind, nullptr, nullptr};
    cuda_check(cudaEventCreate(&e.a), "cudaEventCreate");
    cuda_check(cudaEventCreate(&e.b), "cudaEventCreate");
    prof_.push_back(e);
    cuda_check(cudaEventRecord(e.a, st_), "cudaEventRecord");
    launch();
    cuda_check(cudaEventRecord(e.b, st_), "cudaEventRecord");
  }
  template <typename S, typename D>
  void convert(const S* src, D* dst, size_t count) {
    k_convert<S, D><<<elem_blocks(count), 256, 0, st_>>>(src, dst, count);
    post("k_convert");
  }
  static double dec_host(unsigned long long e) {
    const unsigned long long b = (e & 0x8000000000000000ULL) ? (e & 0x7fffffffffffffffULL) : ~e;
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
  }
  static double ipow(double x, int k) {  // REAL**INTEGER by repeated squaring
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
  void set_scal(int i, double v) {
    k_set_scalar<<<1, 1, 0, st_>>>(scal_ + i, v);
    post("k_set_scalar");
  }
  double get_scal(int i) {
    cuda_check(cudaMemcpyAsync(hsmall_, scal_ + i, sizeof(double), cudaMemcpyDeviceToHost, st_), "D2H scal");
    sync();
    return hsmall_[0];
  }
  void truncate_if_dirty() {
    const int keep = run_;
    for (int r = 0; r < nb_; ++r) {
      if (!dirty_[r]) continue;
      select_run(r);
      specop(P_PS, P_PS, OP_TRUNC_RECT, 0.0);
      specop(P_VZ, P_VZ, OP_TRUNC_RECT, 0.0);
      dirty_[r] = 0;
    }
    select_run(keep);
  }
  RandForceArgs make_rf_args(const RandForceHost* f) {
    RandForceArgs a;
    std::memset(&a, 0, sizeof(a));
    a.nsq = (double)n_ * (double)n_;
    for (int fi = 0; fi < 2; ++fi) {
      RandForceField& d = a.f[fi];
      d.nclear = prev_n_[fi];
      for (int c = 0; c < prev_n_[fi]; ++c) d.clear[c] = prev_[fi][c];
      d.nset = f[fi].nset;
      for (int c = 0; c < f[fi].nset; ++c) {
        d.set[c] = f[fi].set[c];
        d.conj[c] = f[fi].conj[c];
        prev_[fi][c] = f[fi].set[c];
      }
      prev_n_[fi] = f[fi].nset;
      d.c0 = f[fi].c0;
      d.kpow = f[fi].kpow;
      d.cph = f[fi].cph;
      d.sph = f[fi].sph;
    }
    return a;
  }

  // rf_mode: 0 none, 1 single args (rf), -1 sequence from the device array.
  // All nb_ runs advance together (blockIdx.y = run); forcing draws and
  // const_inj are single-run features.
  // fuse: pass A of every substep was queued before (by the previous
  // substep's pass C, or by advance() for the first), and every pass C
  // carries the next substep's pass A (fuse_ca())
  void enqueue_step(bool cfl_mode, bool add_time, int rf_mode, const RandForceHost* rf, bool fuse = false) {
    if (nb_ > 1 && (rf_mode != 0 || ci_on_)) throw Error(kEINVAL, "batched runs take constant forcing");
    cpx<T>* ps = pbase_[P_PS];
    cpx<T>* vz = pbase_[P_VZ];
    const unsigned rb = (unsigned)((nb_ + 31) / 32);
    // The substep state moves ps -> C1 -> C3 -> C1 -> ps (and vz -> C2 -> C4
    // -> C2 -> vz): no substep updates its own input in place, so pass C may
    // split a column pair's C1 and C2 updates over two CTAs (the last
    // substep writes ps, vz, which only the element's own thread reads).
    for (int o = 4; o >= 1; --o) {
      const int pin1 = o == 4 ? P_PS : o == 2 ? P_C3 : P_C1;
      const int pin2 = o == 4 ? P_VZ : o == 2 ? P_C4 : P_C2;
      const int pout1 = o == 1 ? P_PS : o == 3 ? P_C3 : P_C1;
      const int pout2 = o == 1 ? P_VZ : o == 3 ? P_C4 : P_C2;
      const cpx<T>* in1 = pbase_[pin1];
      const cpx<T>* in2 = pbase_[pin2];
      cpx<T>* out1 = pbase_[pout1];
      cpx<T>* out2 = pbase_[pout2];
      if (ci_on_) {  // const_inj every substep (Rot2D3C.para.f90:565-569)
        enqueue_const_inj(in1, pin1, P_FP, 1, ci_fp0_);
        enqueue_const_inj(in2, pin2, P_FZ, 0, ci_fz0_);
      }
      if (!fuse) timed(0, [&] { launch_passA(in1, in2, tf_, nb_); });
      if (o == 4 && cfl_mode) {
        cuda_check(cudaMemsetAsync(enc_base_, 0, sizeof(unsigned long long) * kScalStride * nb_, st_),
                   "memset cfl");
        launch_passB<true>(gd_.M, tf_, pb_, nb_);
        k_cfl_dt<<<rb, 32, 0, st_>>>(enc_base_, d_cfl_, scal_base_, add_time ? 1 : 0, nb_);
        post("k_cfl_dt");
      } else {
        timed(1, [&] { launch_passB<false>(gd_.M, tf_, pb_, nb_); });
        if (o == 4 && add_time) {
          k_add_time<<<rb, 32, 0, st_>>>(scal_base_, nb_);
          post("k_add_time");
        }
      }
      if (o == 4 && rf_mode == 1) {
        RandForceArgs a = make_rf_args(rf);
        k_randforce<T><<<1, 1, 0, st_>>>(pbase_[P_FP], pbase_[P_FZ], scal_base_, a);
        post("k_randforce");
      } else if (o == 4 && rf_mode == -1) {
        k_randforce_seq<T><<<1, 1, 0, st_>>>(pbase_[P_FP], pbase_[P_FZ], scal_base_, d_rf_, d_ctr_);
        post("k_randforce_seq");
      }
      if (o == 1 && ov_wait_) cuda_check(cudaStreamWaitEvent(st_, ov_in_, 0), "wait inputs");
      timed(2, [&] { launch_passC(in1, in2, out1, out2, o, nb_, fuse); });
    }
  }

  // ---------------------------------------------------------------- launchers
  // Groups per CTA of a generic transform launch over `units` transforms:
  // the config's G, halved while the grid would have fewer than two CTAs per
  // SM (on small grids more, smaller CTAs spread the transforms over the SMs;
  // the results are the same)
  int fft_groups(long long units, int G) const {
    int g = G;
    while (g > 1 && (units + g - 1) / g < 2LL * sms_) g /= 2;
    return g;
  }
  // the 8 closure-input fields of the state, y-transformed, into cl_t8_
  void launch_closure_cols() {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      using C = Cfg<T, N>;
      const int ncols = 8 * gd_.nh;
      const int g = fft_groups(ncols, C::G);
      k_closure_cols<T, N><<<(ncols + g - 1) / g, C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(
          planes_[P_PS], planes_[P_VZ], gd_, cl_t8_, tw_);
      post("k_closure_cols");
    });
  }
  // (out2, split: columns from split on go to out2)
  template <int DIR>
  void launch_colfft(const cpx<T>* in, cpx<T>* out, int ncols, cpx<T>* out2 = nullptr, int split = 0x7fffffff) {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      using C = Cfg<T, N>;
      auto k = k_colfft<T, N, DIR>;
      const int g = fft_groups(ncols, C::G);
      k<<<(ncols + g - 1) / g, C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(in, out, ncols, tw_, 0, out2, split);
      post("k_colfft");
    });
  }
  // forward y-FFT of the nh columns of a product plane in the passes' mixed
  // layout (pair-tiled in the FP32 tiled mode)
  void launch_colfft_mixed(const cpx<T>* in, cpx<T>* out) {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr int PY = PassNT<T, N>::value;
      using C = Cfg<T, N>;
      auto k = k_colfft<T, N, -1, PY>;
      const int g = fft_groups(gd_.nh, C::G);
      k<<<(gd_.nh + g - 1) / g, C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(in, out, gd_.nh, tw_, gd_.nh, nullptr,
                                                                                   0x7fffffff);
      post("k_colfft");
    });
  }
  // nplanes consecutive planes at once (blockIdx.y = plane)
  void launch_rowc2r(const cpx<T>* tin, T* rout, unsigned long long* mm, int nplanes = 1) {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      using C = Cfg<T, N>;
      auto k = k_rowc2r<T, N>;
      const int g = fft_groups((long long)(N / 2) * nplanes, C::G);
      k<<<dim3((N / 2 + g - 1) / g, nplanes), C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(tin, rout, mm, tw_);
      post("k_rowc2r");
    });
  }
  void launch_rowr2c(const T* rin, cpx<T>* tout, int nplanes = 1) {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      using C = Cfg<T, N>;
      auto k = k_rowr2c<T, N>;
      const int g = fft_groups((long long)(N / 2) * nplanes, C::G);
      k<<<dim3((N / 2 + g - 1) / g, nplanes), C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(rin, tout, tw_);
      post("k_rowr2c");
    });
  }
  Batch batch() const { return Batch{S_, (size_t)6 * gd_.M * n_, 2 * S_}; }
  void launch_passA(const cpx<T>* a, const cpx<T>* b, cpx<T>* tf, int nb) {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr int NT = PassNT<T, N>::value;
      auto go = [&](auto EC) {
        constexpr int EA = decltype(EC)::value;
        using C = CfgAE<T, N, EA>;
        auto k = k_passA<T, N, EA>;
        const int groups = (gd_.M + NT - 1) / NT;
        const int g = ga_ ? ga_ : C::G;  // groups per CTA, field chunks: autotuned
        const dim3 grid((groups + g - 1) / g, nb, fa_);
        // each radix has the twiddle table of its own stage schedule
        const tw_t<T>* tw = EA == PassAE<T, N>::value ? tw_a_ : tw_;
        k<<<grid, C::TPF * g, g * C::FFT::SMEM_BYTES, st_>>>(a, b, tf, gd_, tw, batch());
        post("k_passA");
      };
      if constexpr (kAltRadixA<T, N>) {
        if (radix_a_ == Cfg<T, N>::E) {
          go(std::integral_constant<int, Cfg<T, N>::E>{});
          return;
        }
      }
      go(std::integral_constant<int, PassAE<T, N>::value>{});
    });
  }
  template <bool CFL>
  void launch_passB(int kxo, const cpx<T>* tf, cpx<T>* pb, int nb) {
    const T inv4 = (T)(1.0 / ((double)n_ * n_ * n_ * n_));
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr int NR = PassNT<T, N>::value;
      using C = Cfg<T, N, NR>;
      bool persistent = false;
      if constexpr (kPipeB<T, N>) {
        if (passb_mode_ == 1) {
          // persistent: the autotuned CTA count (about as many as fit at once)
          persistent = true;
          constexpr int EP = PipeB<N>::E;
          static_assert(EP == PassAE<T, N>::value || EP == Cfg<T, N>::E, "pass B radix has a twiddle table");
          const tw_t<T>* twp = EP == PassAE<T, N>::value ? tw_a_ : tw_;
          const int per_run = std::max(1, std::min(N / 2, (pipeb_grid_ + nb - 1) / nb));
          auto k = k_passB_pipe<N, CFL>;
          k<<<dim3(per_run, nb), PipeB<N>::THREADS, PipeB<N>::smem(gd_.M), st_>>>(tf, pb, kxo, gd_, inv4, twp,
                                                                                    enc_base_, batch());
          post("k_passB_pipe");
        }
      }
      if constexpr (SplitB<T, N>::OK) {
        if (passb_mode_ == 2) {  // three CTA groups per row pair (small grids)
          persistent = true;
          k_passB_split<T, N, CFL><<<dim3(N / NR, nb), SplitB<T, N>::THREADS, SplitB<T, N>::SMEM, st_>>>(
              tf, pb, kxo, gd_, inv4, tw_, enc_base_, batch());
          post("k_passB_split");
        }
      }
      if (!persistent) {  // one CTA (group) per row pair; the only form below n = 2048
        auto k = k_passB<T, N, CFL>;
        const int g = gb_ ? gb_ : C::G;  // groups per CTA: autotuned
        const dim3 grid((N / NR + g - 1) / g, nb);
        // (the rolled form keeps each group's first bracket in shared memory too)
        const size_t smem = g * (PassSmem<T, N>::GROUP_ELEMS * sizeof(cpx<T>) + (RolledB<T, N>::OK ? N * sizeof(T) : 0));
        k<<<grid, C::TPF * g, smem, st_>>>(tf, pb, kxo, gd_, inv4, tw_, enc_base_, batch());
        post("k_passB");
      }
    });
  }
  void launch_passC(const cpx<T>* c1in, const cpx<T>* c2in, cpx<T>* c1out, cpx<T>* c2out, int o, int nb,
                    bool fuse = false) {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr int NT = PassNT<T, N>::value;
      using C = Cfg<T, N, NT>;
      const cpx<T>* t5 = closure_on_ ? pbase_[P_T5] : nullptr;
      const cpx<T>* t6 = closure_on_ ? pbase_[P_T6] : nullptr;
      bool persistent = false;
      if constexpr (kPipeC<T, N>) {
        if (passc_mode_ == 1) {
          // persistent: the autotuned CTA count
          persistent = true;
          const int pairs = (gd_.M + 1) / 2;
          const int per_run = std::max(1, std::min(pairs, (pipec_grid_ + nb - 1) / nb));
          k_passC_pipe<N><<<dim3(per_run, nb), PipeC<N>::THREADS, PipeC<N>::SMEM, st_>>>(
              pb_, c1in, c2in, pbase_[P_PS], pbase_[P_VZ], pbase_[P_FP], pbase_[P_FZ], c1out, c2out, gd_, d_sc_,
              scal_base_, o, tw_, batch(), t5, t6);
          post("k_passC_pipe");
        }
      }
      if (!persistent) {  // one CTA (group) per column pair
        auto k = k_passC<T, N>;
        if constexpr (kFuseCA<T, N>) {
          if (fuse) k = k_passC<T, N, true>;
        }
        if (fuse && !kFuseCA<T, N>) throw Error(kESTATE, "pass C carries pass A only for FP32 n <= 512");
        const int groups = (gd_.M + NT - 1) / NT;
        const int g = gc_ ? gc_ : C::G;  // groups per CTA: autotuned
        // the C1 and C2 updates of a column pair in one CTA or two, and
        // teams of wc_ groups per column pair (autotuned)
        const int w = kChunkC<T, N> ? wc_ : 1;
        const int teams = std::max(1, g / w);
        const dim3 grid((groups + teams - 1) / teams, nb, kChunkC<T, N> ? fc_ : 1);
        k<<<grid, C::TPF * g, g * PassSmem<T, N>::GROUP_ELEMS * sizeof(cpx<T>), st_>>>(pb_, c1in, c2in, pbase_[P_PS], pbase_[P_VZ],
                                                           pbase_[P_FP], pbase_[P_FZ], c1out, c2out, gd_, d_sc_,
                                                           scal_base_, o, tw_, batch(), t5, t6, w,
                                                           fuse ? tf_ : nullptr, fuse ? tw_a_ : nullptr);
        post("k_passC");
      }
    });
  }

  // Dynamic shared memory above 48 KB has to be enabled per kernel before the
  // first launch (and before any stream capture).
  void set_kernel_attrs() {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr size_t sm = Cfg<T, N>::SMEM;
      set_smem_attr(k_colfft<T, N, -1>, sm);
      set_smem_attr(k_colfft<T, N, +1>, sm);
      set_smem_attr(k_colfft<T, N, -1, PassNT<T, N>::value>, sm);
      set_smem_attr(k_rowc2r<T, N>, sm);
      set_smem_attr(k_rowr2c<T, N>, sm);
      set_smem_attr(k_cnn2_to_rows<T, N>, sm);
      set_smem_attr(k_closure_cols<T, N>, sm);
      set_smem_attr(k_colfft_band2<T, N>, sm);
      if constexpr (RowsCnn<T, N>::OK) set_smem_attr(k_rows_to_cnn8<T, N>, RowsCnn<T, N>::SMEM);
      constexpr size_t smh = PassSmem<T, N>::SMEM;
      set_smem_attr(k_passA<T, N>, CfgA<T, N>::SMEM);
      if constexpr (kAltRadixA<T, N>) set_smem_attr(k_passA<T, N, Cfg<T, N>::E>, CfgAE<T, N, Cfg<T, N>::E>::SMEM);
      set_smem_attr(k_passB<T, N, true>, RolledB<T, N>::SMEM);
      set_smem_attr(k_passB<T, N, false>, RolledB<T, N>::SMEM);
      if constexpr (SplitB<T, N>::OK) {
        set_smem_attr(k_passB_split<T, N, true>, SplitB<T, N>::SMEM);
        set_smem_attr(k_passB_split<T, N, false>, SplitB<T, N>::SMEM);
      }
      set_smem_attr(k_passC<T, N>, smh);
      if constexpr (kFuseCA<T, N>) set_smem_attr(k_passC<T, N, true>, smh);
      if constexpr (kPipeC<T, N>) {
        set_smem_attr(k_passC_pipe<N>, PipeC<N>::SMEM);
        cuda_check(cudaFuncSetAttribute(k_passC_pipe<N>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                        (int)cudaSharedmemCarveoutMaxShared),
                   "cudaFuncSetAttribute(carveout)");
        int per_sm = 0, sms = 0, dev = 0;
        cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_passC_pipe<N>, PipeC<N>::THREADS,
                                                                 PipeC<N>::SMEM),
                   "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
        if (per_sm < 1) throw Error(kEINVAL, "pass C pipeline does not fit on this device");
        pipec_ctas_ = per_sm * sms;
      }
      if constexpr (kPipeB<T, N>) {
        const size_t smp = PipeB<N>::smem(gd_.M);
        set_smem_attr(k_passB_pipe<N, true>, smp);
        set_smem_attr(k_passB_pipe<N, false>, smp);
        // all of the unified L1/shared array as shared memory: as many
        // persistent CTAs per SM as their shared memory allows
        for (auto k : {k_passB_pipe<N, true>, k_passB_pipe<N, false>})
          cuda_check(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                          (int)cudaSharedmemCarveoutMaxShared),
                     "cudaFuncSetAttribute(carveout)");
        int per_sm = 0, sms = 0, dev = 0;
        cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_passB_pipe<N, true>,
                                                                 PipeB<N>::THREADS, smp),
                   "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
        if (per_sm < 1) throw Error(kEINVAL, "pass B pipeline does not fit on this device");
        pipeb_ctas_ = per_sm * sms;
      }
    });
  }

  // Launch-schedule autotuner, run once when a full engine is created.  The
  // launch shapes of passes A, B and C that compute bit-identical results
  // are timed with CUDA events on this engine's own buffers (time_candidates)
  // and the fastest of each pass is kept:
  //   A: transform groups per CTA (the config's G down to 1) x field chunks
  //      (the six fields in 1, 2, 3 or 6 CTAs);
  //   B: one group per row pair, G down to 1 groups per CTA, or (n = 512 ..
  //      4096 FP32) persistent cp.async-staged CTAs, as many as are resident
  //      or half of that;
  //   C: the same with column pairs.
  // Small grids gain from spreading the work over more SMs (256^2: the
  // config's groups fill 6 CTAs in pass A); large ones from full CTAs.
  // Pass A's radix (FP32, n = 1024 .. 4096) is chosen as FFTW's measured
  // plans choose their algorithms: it changes the rounding (both radices
  // stay within the FP32 path's error bound against FP64), so the choice is
  // made once per process for each precision and n (choose_plan).
  // Time per launch (us) of each of nc candidates: one untimed launch of
  // every candidate, then three rounds over all of them (interleaved, so that
  // clock or cache drift affects them alike), each round three launches of a
  // candidate between two events; a candidate's fastest round counts.
  std::vector<float> time_candidates(size_t nc, const std::function<void(size_t)>& launch) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
    cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
    std::vector<float> best(nc, 0.f);
    for (size_t c = 0; c < nc; ++c) launch(c);
    for (int round = 0; round < 3; ++round)
      for (size_t c = 0; c < nc; ++c) {
        cuda_check(cudaEventRecord(e0, st_), "cudaEventRecord");
        for (int i = 0; i < 3; ++i) launch(c);
        cuda_check(cudaEventRecord(e1, st_), "cudaEventRecord");
        cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        const float us = 1e3f * ms / 3.f;
        if (round == 0 || us < best[c]) best[c] = us;
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
  }
  // R2D3C_GROUPS="ga,fa,gb,gc" fixes the groups per CTA of passes A, B, C
  // and pass A's field chunks (0 for a group count: the config's G)
  static void forced_groups(int G_A, int G_B, int G_C, int out[6]) {
    out[0] = out[2] = out[3] = -1;
    out[1] = -1;
    out[4] = out[5] = -1;
    const char* e = std::getenv("R2D3C_GROUPS");
    if (!e) return;
    int v[6] = {0, 0, 0, 0, -1, -1};
    const int got = std::sscanf(e, "%d,%d,%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]);
    if (got < 4) throw Error(kEINVAL, "R2D3C_GROUPS must be ga,fa,gb,gc[,cc[,cw]]");
    if (got >= 5 && v[4] != 1 && v[4] != 2) throw Error(kEINVAL, "R2D3C_GROUPS: pass C chunks must be 1 or 2");
    if (got == 6 && v[5] != 1 && v[5] != 2 && v[5] != 4)
      throw Error(kEINVAL, "R2D3C_GROUPS: pass C team must be 1, 2 or 4 groups");
    out[4] = got >= 5 ? v[4] : -1;
    out[5] = got == 6 ? v[5] : -1;
    auto group_ok = [](int g, int G) { return g == 0 || (g >= 1 && g <= G && (g & (g - 1)) == 0); };
    if (!group_ok(v[0], G_A) || !group_ok(v[2], G_B) || !group_ok(v[3], G_C) ||
        !(v[1] == 1 || v[1] == 2 || v[1] == 3 || v[1] == 6))
      throw Error(kEINVAL, "R2D3C_GROUPS: group counts must be 0 or a power of two up to G, field chunks 1, 2, 3 or 6");
    for (int i = 0; i < 4; ++i) out[i] = v[i];
  }
  void autotune() {
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr int GA = CfgA<T, N>::G;
      constexpr int GB = Cfg<T, N, PassNT<T, N>::value>::G;
      const int saved = launches_;
      int sms = 0;
      cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_), "cudaDeviceGetAttribute");
      // ---- pass A (reads the state, writes the derivative planes): every
      // radix it has (FP32 n = 1024 .. 4096: 16 and 8) x groups per CTA x
      // field chunks
      cuda_check(cudaMemsetAsync(tf_, 0, sizeof(cpx<T>) * 6 * (size_t)gd_.M * n_ * nb_, st_), "memset");
      {
        struct CandA {
          int radix, g, f;
        };
        std::vector<CandA> cands;
        std::vector<std::pair<int, int>> radices = {{PassAE<T, N>::value, GA}};
        if constexpr (kAltRadixA<T, N>) radices.push_back({Cfg<T, N>::E, CfgAE<T, N, Cfg<T, N>::E>::G});
        for (auto [r, G] : radices)
          for (int g = G; g >= 1; g /= 2)
            for (int f : {1, 2, 3, 6}) cands.push_back({r, g, f});
        const std::vector<float> us = time_candidates(cands.size(), [&](size_t i) {
          radix_a_ = cands[i].radix;
          ga_ = cands[i].g;
          fa_ = cands[i].f;
          launch_passA(pbase_[P_PS], pbase_[P_VZ], tf_, nb_);
        });
        tune_a_.clear();
        for (size_t i = 0; i < cands.size(); ++i)
          tune_a_.push_back({cands[i].g, cands[i].f, us[i], cands[i].radix});
      }
      // (mode, grid): mode 0 one CTA per row / column pair with `grid` groups
      // per CTA; mode 1 persistent with `grid` CTAs
      // ---- pass B (derivative planes -> bracket planes)
      {
        std::vector<std::pair<int, int>> cands;
        for (int g = GB; g >= 1; g /= 2) cands.push_back({0, g});
        if constexpr (kPipeB<T, N>) {
          cands.push_back({1, pipeb_ctas_});
          if (pipeb_ctas_ >= 2 * sms) cands.push_back({1, pipeb_ctas_ / 2});
        }
        if constexpr (SplitB<T, N>::OK) cands.push_back({2, 1});
        const std::vector<float> us = time_candidates(cands.size(), [&](size_t i) {
          passb_mode_ = cands[i].first;
          pipeb_grid_ = cands[i].first == 1 ? cands[i].second : 0;
          gb_ = cands[i].first ? GB : cands[i].second;
          launch_passB<false>(gd_.M, tf_, pb_, nb_);
        });
        tune_.clear();
        for (size_t i = 0; i < cands.size(); ++i) tune_.push_back({cands[i].first, cands[i].second, us[i]});
      }
      // ---- pass C on the engine's scratch planes (C1, C2 in and out), zero
      // coefficients
      {
        cuda_check(cudaMemsetAsync(pb_, 0, sizeof(cpx<T>) * 2 * S_ * nb_, st_), "memset");
        cuda_check(cudaMemsetAsync(d_sc_, 0, sizeof(StepCoef) * nb_, st_), "memset");
        coefs_valid_ = false;
        struct CandC {
          int mode, grid, chunks, wide;
        };
        std::vector<CandC> cands;
        for (int g = GB; g >= 1; g /= 2) {
          cands.push_back({0, g, 1, 1});
          if constexpr (kChunkC<T, N>) {
            cands.push_back({0, g, 2, 1});
            // teams of 2 or 4 groups per column pair share its update
            for (int w : {2, 4})
              if (w <= g) cands.push_back({0, g, 2, w});
          }
        }
        if constexpr (kPipeC<T, N>) {
          cands.push_back({1, pipec_ctas_, 1, 1});
          if (pipec_ctas_ >= 2 * sms) cands.push_back({1, pipec_ctas_ / 2, 1, 1});
        }
        cpx<T>* c1 = planes_[P_C1];
        cpx<T>* c2 = planes_[P_C2];
        cpx<T>* c3 = planes_[P_C3];
        cpx<T>* c4 = planes_[P_C4];
        const std::vector<float> us = time_candidates(cands.size(), [&](size_t i) {
          passc_mode_ = cands[i].mode;
          pipec_grid_ = cands[i].mode ? cands[i].grid : 0;
          gc_ = cands[i].mode ? GB : cands[i].grid;
          fc_ = cands[i].chunks;
          wc_ = cands[i].wide;
          launch_passC(c1, c2, c3, c4, 4, nb_);
        });
        tune_c_.clear();
        for (size_t i = 0; i < cands.size(); ++i) {
          TuneRec r{cands[i].mode, cands[i].grid, us[i]};
          r.chunks = cands[i].chunks;
          r.wide = cands[i].wide;
          tune_c_.push_back(r);
        }
        for (int p : {P_C1, P_C2, P_C3, P_C4})
          cuda_check(cudaMemsetAsync(planes_[p], 0, sizeof(cpx<T>) * S_ * nb_, st_), "memset");
      }
      launches_ = saved;
    });
    choose_plan();
  }

  // The launch choices from the autotuner's timings.  Policy 0: the fastest
  // candidate of each pass.  Policy 1 (ensembles of several size groups,
  // whose graphs run the groups side by side, where a flood of small CTAs
  // from one group measured slower than full ones): pass A with the
  // config's groups per CTA and all six fields in one CTA, passes B and C
  // with the config's groups per CTA or persistent.  Policy 2: as policy 1,
  // with passes B and C persistent wherever that form exists (a pass C
  // that is faster alone with one CTA per column pair measured slower side
  // by side with the other groups).  The environment overrides
  // (R2D3C_PASSB, R2D3C_PASSC, R2D3C_GROUPS) apply to all three.
  void choose_plan() {
    if (const char* e = std::getenv("R2D3C_FUSE_CA")) {
      if (std::strcmp(e, "0") != 0 && std::strcmp(e, "1") != 0) throw Error(kEINVAL, "R2D3C_FUSE_CA must be 0 or 1");
      fuse_ca_on_ = e[0] == '1';
    }
    if (tune_a_.empty()) return;
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr int GA = CfgA<T, N>::G;
      constexpr int GB = Cfg<T, N, PassNT<T, N>::value>::G;
      int forced[6];
      forced_groups(GA, GB, GB, forced);
      auto argmin = [](const std::vector<TuneRec>& t, const std::function<bool(const TuneRec&)>& ok) {
        size_t k = t.size();
        for (size_t i = 0; i < t.size(); ++i)
          if (ok(t[i]) && (k == t.size() || t[i].us < t[k].us)) k = i;
        return k;
      };
      const int pol = policy_;
      // pass A's radix: R2D3C_RADIX_A, else the choice already made in this
      // process for this precision and n, else the default radix unless the
      // other one's best candidate is more than 3% faster (then remembered
      // for the process, so that every engine of this precision and n --
      // single runs and batched ones alike -- rounds the same way)
      const int r0 = PassAE<T, N>::value;
      int ra = r0;
      if constexpr (kAltRadixA<T, N>) {
        const int r1 = Cfg<T, N>::E;
        if (const char* e = std::getenv("R2D3C_RADIX_A")) {
          ra = std::atoi(e);
          if (ra != r0 && ra != r1)
            throw Error(kEINVAL, "R2D3C_RADIX_A must be " + std::to_string(r0) + " or " + std::to_string(r1));
        } else {
          std::lock_guard<std::mutex> lk(radix_mu());
          auto& cache = radix_cache();
          const int key = (int)sizeof(T) * 1000000 + N;
          auto it = cache.find(key);
          if (it != cache.end()) {
            ra = it->second;
          } else {
            const size_t b0 = argmin(tune_a_, [&](const TuneRec& r) { return r.radix == r0; });
            const size_t b1 = argmin(tune_a_, [&](const TuneRec& r) { return r.radix == r1; });
            if (b1 < tune_a_.size() && tune_a_[b1].us < 0.97f * tune_a_[b0].us) ra = r1;
            cache[key] = ra;
          }
        }
      }
      radix_a_ = ra;
      const int GAr = ra == r0 ? GA : CfgAE<T, N, Cfg<T, N>::E>::G;
      const size_t ka = argmin(tune_a_, [&](const TuneRec& r) {
        return r.radix == ra && (pol == 0 || (r.mode == GAr && r.grid == 1));
      });
      if (forced[0] > GAr) throw Error(kEINVAL, "R2D3C_GROUPS: more pass-A groups per CTA than its radix allows");
      ga_ = forced[0] >= 0 ? (forced[0] ? forced[0] : GAr) : tune_a_[ka].mode;
      fa_ = forced[1] >= 0 ? forced[1] : tune_a_[ka].grid;
      auto pick_bc = [&](const std::vector<TuneRec>& t, const char* env, const char* pair_name, int forced_g,
                         int& mode, int& grid, int& groups) {
        auto ok = [&](const TuneRec& r) { return pol == 0 || r.mode == 1 || (r.mode == 0 && r.grid == GB); };
        const size_t pick0 = argmin(t, [&](const TuneRec& r) { return r.mode == 0 && ok(r); });
        size_t pick = argmin(t, ok);
        if (pol == 2) {  // the persistent form wherever it exists
          const size_t pp = argmin(t, [](const TuneRec& r) { return r.mode == 1; });
          if (pp < t.size()) pick = pp;
        }
        // env=<pair_name>|persistent overrides the measured choice
        // (persistent where it exists: FP32, n = 512 .. 4096)
        if (const char* force = std::getenv(env)) {
          if (std::strcmp(force, pair_name) == 0) {
            pick = pick0;
          } else if (std::strcmp(force, "split") == 0) {
            // three groups per row pair, where it exists (pass B of small grids)
            size_t k = t.size();
            for (size_t i = 0; i < t.size(); ++i)
              if (t[i].mode == 2) k = i;
            pick = k < t.size() ? k : pick0;
          } else if (std::strcmp(force, "persistent") == 0) {
            // the first persistent candidate: all resident CTAs
            size_t k = t.size();
            for (size_t i = t.size(); i-- > 0;)
              if (t[i].mode == 1) k = i;
            pick = k < t.size() ? k : pick0;
          } else {
            throw Error(kEINVAL, std::string(env) + " must be " + pair_name + ", persistent or split");
          }
        }
        mode = t[pick].mode;
        grid = mode == 1 ? t[pick].grid : 0;
        groups = forced_g >= 0 ? (forced_g ? forced_g : GB) : t[pick0].grid;
        return pick0;
      };
      pick_bc(tune_, "R2D3C_PASSB", "per_row_pair", forced[2], passb_mode_, pipeb_grid_, gb_);
      const size_t c0 = pick_bc(tune_c_, "R2D3C_PASSC", "per_column_pair", forced[3], passc_mode_, pipec_grid_, gc_);
      fc_ = forced[4] > 0 ? forced[4] : (c0 < tune_c_.size() ? tune_c_[c0].chunks : 1);
      // a forced pass-C group count without a forced team width runs one group per column pair
      wc_ = forced[5] > 0 ? forced[5] : forced[3] >= 0 ? 1 : (c0 < tune_c_.size() ? tune_c_[c0].wide : 1);
      if (!kChunkC<T, N>) fc_ = wc_ = 1;
      if (wc_ > gc_) throw Error(kEINVAL, "R2D3C_GROUPS: pass C team wider than its groups per CTA");
    });
  }
  void set_plan_policy(int policy) override {
    if (policy < 0 || policy > 2) throw Error(kEINVAL, "plan policy must be 0, 1 or 2");
    policy_ = policy;
    choose_plan();
  }

 public:
  std::string plan_report() const override {
    std::string r = "{\"policy\": " + std::to_string(policy_) + ", \"pass_a\": [";
    char b[200];
    for (size_t i = 0; i < tune_a_.size(); ++i) {
      snprintf(b, sizeof b, "%s{\"radix\": %d, \"groups\": %d, \"field_chunks\": %d, \"us\": %.2f}",
               i ? ", " : "", tune_a_[i].radix, tune_a_[i].mode, tune_a_[i].grid, (double)tune_a_[i].us);
      r += b;
    }
    snprintf(b, sizeof b, "], \"radix_a\": %d, \"groups_a\": %d, \"field_chunks_a\": %d, \"pass_b\": [",
             radix_a_, ga_, fa_);
    r += b;
    for (size_t i = 0; i < tune_.size(); ++i) {
      if (tune_[i].mode == 2)
        snprintf(b, sizeof b, "%s{\"variant\": \"split\", \"us\": %.2f}", i ? ", " : "", (double)tune_[i].us);
      else if (tune_[i].mode)
        snprintf(b, sizeof b, "%s{\"variant\": \"persistent\", \"ctas\": %d, \"us\": %.2f}", i ? ", " : "",
                 tune_[i].grid, (double)tune_[i].us);
      else
        snprintf(b, sizeof b, "%s{\"variant\": \"per_row_pair\", \"groups\": %d, \"us\": %.2f}", i ? ", " : "",
                 tune_[i].grid, (double)tune_[i].us);
      r += b;
    }
    snprintf(b, sizeof b, "], \"chosen\": \"%s\", \"ctas\": %d, \"groups_b\": %d",
             passb_mode_ == 2 ? "split" : passb_mode_ ? "persistent" : "per_row_pair", passb_mode_ == 1 ? pipeb_grid_ : 0,
             gb_);
    r += b;
    r += ", \"pass_c\": [";
    for (size_t i = 0; i < tune_c_.size(); ++i) {
      if (tune_c_[i].mode)
        snprintf(b, sizeof b, "%s{\"variant\": \"persistent\", \"ctas\": %d, \"us\": %.2f}", i ? ", " : "",
                 tune_c_[i].grid, (double)tune_c_[i].us);
      else
        snprintf(b, sizeof b,
                 "%s{\"variant\": \"per_column_pair\", \"groups\": %d, \"chunks\": %d, \"team\": %d, \"us\": %.2f}",
                 i ? ", " : "", tune_c_[i].grid, tune_c_[i].chunks, tune_c_[i].wide, (double)tune_c_[i].us);
      r += b;
    }
    snprintf(b, sizeof b,
             "], \"chosen_c\": \"%s\", \"ctas_c\": %d, \"groups_c\": %d, \"chunks_c\": %d, \"team_c\": %d, "
             "\"fused_ca\": %s}",
             passc_mode_ ? "persistent" : "per_column_pair", passc_mode_ ? pipec_grid_ : 0, gc_, fc_, wc_,
             fuse_ca() ? "true" : "false");
    return r + b;
  }

 private:
  void build_twiddles() {
    std::vector<double> c(n_), s(n_);
    host_unit_roots(n_, c.data(), s.data());
    std::vector<tw_t<T>> h(n_), ha(n_);
    dispatch_n(n_, [&](auto NC) {
      constexpr int N = decltype(NC)::value;
      constexpr int EA = PassAE<T, N>::value;
      static_assert(BlockFFT<T, N, Cfg<T, N>::E>::TW_ELEMS <= N, "twiddle table fits in n entries");
      static_assert(BlockFFT<T, N, EA>::TW_ELEMS <= N, "twiddle table fits in n entries");
      build_stage_twiddles<T, N, Cfg<T, N>::E>(h.data(), c.data(), s.data());
      build_stage_twiddles<T, N, EA>(ha.data(), c.data(), s.data());
    });
    cuda_check(cudaMemcpyAsync(tw_, h.data(), sizeof(tw_t<T>) * n_, cudaMemcpyHostToDevice, st_), "H2D twiddles");
    cuda_check(cudaMemcpyAsync(tw_a_, ha.data(), sizeof(tw_t<T>) * n_, cudaMemcpyHostToDevice, st_),
               "H2D twiddles");
    sync();
  }

  int n_, dev_;
  bool full_;
  int nb_ = 1, run_ = 0;
  bool closure_on_ = false;
  cpx<T>* cl_t8_ = nullptr;  // closure scratch (closure_scratch)
  float* band_w_ = nullptr;  // per-shell tendency weights (set_closure_band)
  int band_nw_ = 0;
  T* cl_r8_ = nullptr;
  cpx<T>* cl_tn_ = nullptr;  // the overlapped LES step's next tendencies (2 planes)
  cudaStream_t ov_stream_ = nullptr;
  cudaEvent_t ov_fork_ = nullptr, ov_in_ = nullptr, ov_join_ = nullptr;
  std::function<void(cudaStream_t)> hook_;
  unsigned long long hook_id_ = 0;
  int pipeb_ctas_ = 0;  // resident CTAs of the pipelined pass B (whole device)
  int passb_mode_ = 0;  // 0: one CTA per row pair, 1: persistent (autotuned)
  int pipeb_grid_ = 0;  // CTAs of the persistent pass B (autotuned)
  int pipec_ctas_ = 0;  // resident CTAs of the persistent pass C (whole device)
  int passc_mode_ = 0;  // 0: one CTA per column pair, 1: persistent (autotuned)
  int pipec_grid_ = 0;  // CTAs of the persistent pass C (autotuned)
  int sms_ = 0;         // SMs of the device
  int policy_ = 0;      // plan policy (choose_plan)
  int ga_ = 0, fa_ = 1;  // pass A: groups per CTA (0: the config's G), field chunks (autotuned)
  int fc_ = 1;           // pass C: CTAs per column pair (1 or 2, autotuned)
  int wc_ = 1;           // pass C: groups per column pair sharing its update (autotuned)
  int gb_ = 0, gc_ = 0;  // passes B, C one CTA per row / column pair: groups per CTA (autotuned)
  struct TuneRec {
    int mode, grid;  // pass A: groups, field chunks; B, C: variant, CTAs or groups
    float us;
    int radix = 0;   // pass A: the transform radix
    int chunks = 1;  // pass C: CTAs per column pair
    int wide = 1;    // pass C: groups per column pair
  };
  // pass A radix chosen per (precision, n), shared by the engines of a process
  static std::map<int, int>& radix_cache() {
    static std::map<int, int> m;
    return m;
  }
  static std::mutex& radix_mu() {
    static std::mutex m;
    return m;
  }
  int radix_a_ = 0;  // pass A radix (0 before the plan: the default)
  std::vector<TuneRec> tune_a_, tune_, tune_c_;
  cpx<T>* pbase_[P_COUNT] = {};
  double* scal_base_ = nullptr;
  unsigned long long* enc_base_ = nullptr;
  StepCoef* d_sc_ = nullptr;
  CflCoef* d_cfl_ = nullptr;
  std::vector<char> dirty_;
  std::vector<ModelCoef> coefs_;
  std::vector<char> up_sc_, up_cc_;  // the coefficients on the device (upload_coefs)
  bool coefs_valid_ = false;
  cudaStream_t st_ = nullptr;
  bool ci_on_ = false;
  int ci_n_ = 0;
  double ci_lo_ = 0, ci_hi_ = 0, ci_fp0_ = 0, ci_fz0_ = 0;
  int* ci_idx_ = nullptr;
  int* ci_mir_ = nullptr;
  float* ci_rnd_ = nullptr;
  DevGrid gd_{};
  size_t S_ = 0, stage_count_ = 0, bytes_ = 0;
  std::vector<void*> owned_;
  cpx<T>* planes_[P_COUNT] = {};
  T* rplanes_[R_COUNT] = {};
  cpx<T>* tf_ = nullptr;
  cpx<T>* pb_ = nullptr;
  cpx<T>* tg_ = nullptr;
  tw_t<T>* tw_ = nullptr;
  tw_t<T>* tw_a_ = nullptr;
  double* stage64_ = nullptr;
  double* scal_ = nullptr;
  unsigned long long* enc_ = nullptr;
  double* partials_ = nullptr;
  double* small_ = nullptr;
  double* hsmall_ = nullptr;
  RandForceArgs* d_rf_ = nullptr;
  int rf_cap_ = 0;
  int* d_ctr_ = nullptr;
  int prev_[2][4] = {};
  int prev_n_[2] = {0, 0};
  int launches_ = 0;
  cudaGraphExec_t graph_ = nullptr;
  int graph_launches_ = 0;
  bool profiling_ = false;
  std::vector<ProfEv> prof_;
  GraphKey gkey_;
};

}  // namespace r2d3c

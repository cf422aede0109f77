// Elementwise spectral operators, FP64 diagnostic reductions, forcing and
// initial-condition kernels of the Rot2D3C hot path (sm_103a).
#pragma once

#include <cuda_bf16.h>

#include "r2d3c_kernels.cuh"

namespace r2d3c {

// ---------------------------------------------------------------------------
// spectral elementwise operators (pseudospec2D_Rot2D3C.f90:6-127)
// ---------------------------------------------------------------------------
enum SpecOp : int {
  OP_COPY_MASK = 0,   // derivk2 dir 0
  OP_DERIV_X = 1,     // derivk2 dir 1: i*ka(i)*a, ka2 <= kmax
  OP_DERIV_Y = 2,     // derivk2 dir 2: i*ka(j)*a, ka2 <= kmax
  OP_LAPLA = 3,       // laplak2: -ka2*a
  OP_INVLAPLA = 4,    // inv_laplak2: -a/ka2 where ka2 > tiny
  OP_SCALE = 5,       // a*s          (field output, Rot2D3C.para.f90:476-491)
  OP_SCALE_KA2 = 6,   // a*ka2*s      (vorticity output, :497-501)
  OP_TRUNC_RECT = 7,  // zero outside the retained rectangle kx < M, |ky| <= L
};

// kx value of spectral column i (ka(i), Rot2D3C.para.f90:220-223)
__device__ __forceinline__ int kx_of(int i, int n) { return i < (n >> 1) ? i : i - n; }

struct Scale8 {
  double v[8];
};

// Row i (kx index) and column j (ky index) of element idx of a spectral
// plane [kx][ky] of n columns: n is a power of two in every engine, so a
// shift and a mask take the place of a 64-bit division (an emulated
// instruction sequence per element)
__device__ __forceinline__ void plane_ij(size_t idx, int n, int& i, int& j) {
  i = (int)(idx >> (__ffs(n) - 1));
  j = (int)(idx & (size_t)(n - 1));
}

template <typename T>
__global__ void k_specop(const cpx<T>* __restrict__ a, cpx<T>* __restrict__ b, DevGrid gd, int op,
                         double s) {
  const size_t total = (size_t)gd.nh * gd.n;
  const T sc = (T)s;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    plane_ij(idx, gd.n, i, j);
    const int kx = kx_of(i, gd.n), ky = ky_of(j, gd.n);
    const int k2 = kx * kx + ky * ky;
    const cpx<T> x = a[idx];
    cpx<T> y;
    switch (op) {
      case OP_DERIV_X:
        y = k2 <= gd.kmaxi ? mkc<T>(-(T)kx * x.y, (T)kx * x.x) : czero<T>();
        break;
      case OP_DERIV_Y:
        y = k2 <= gd.kmaxi ? mkc<T>(-(T)ky * x.y, (T)ky * x.x) : czero<T>();
        break;
      case OP_LAPLA: {
        const T m = -(T)k2;
        y = mkc<T>(m * x.x, m * x.y);
        break;
      }
      case OP_INVLAPLA:
        y = k2 >= 1 ? mkc<T>(-x.x / (T)k2, -x.y / (T)k2) : czero<T>();
        break;
      case OP_SCALE:
        y = mkc<T>(x.x * sc, x.y * sc);
        break;
      case OP_SCALE_KA2:
        y = mkc<T>(x.x * (T)k2 * sc, x.y * (T)k2 * sc);
        break;
      case OP_TRUNC_RECT:
        y = (i < gd.M && ky <= gd.L && -ky <= gd.L) ? x : czero<T>();
        break;
      default:  // OP_COPY_MASK
        y = k2 <= gd.kmaxi ? x : czero<T>();
        break;
    }
    b[idx] = y;
  }
}

// r3 = r1*r2 (mode 0) or r3 = (r3 - r1*r2)*s (mode 1): poisson products
// (pseudospec2D_Rot2D3C.f90:199-216); s = 1/n^4 is a power of two, so the
// multiply equals the reference's division exactly.
template <typename T>
__global__ void k_realprod(T* __restrict__ r3, const T* __restrict__ r1, const T* __restrict__ r2,
                           size_t count, int mode, double s) {
  const T sc = (T)s;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
       i += (size_t)gridDim.x * blockDim.x) {
    const T p = r1[i] * r2[i];
    r3[i] = mode == 0 ? p : (r3[i] - p) * sc;
  }
}

template <typename Src, typename Dst>
__global__ void k_convert(const Src* __restrict__ src, Dst* __restrict__ dst, size_t count) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
       i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (Dst)src[i];
}

// ---------------------------------------------------------------------------
// half-plane sums (energy :336-396, inerprod :400-451, cond_check :455-568)
// Every term sums two*w(k)*v over the half plane with two = 1 on the kx = 0
// column; the 1/n^4 factor of the reference (a power of two) is applied once
// to the total, which is exact.  Per-thread sequential sums, a fixed-shape
// tree per CTA and a fixed-order pass over the CTA partials make every sum
// reproducible run to run.
// ---------------------------------------------------------------------------
enum SumKind : int {
  S_ENERGY = 0,      // |a|^2 ka2^kin; kin >= 0 all k, kin < 0 ka2 >= tiny
  S_INERPROD = 1,    // ka2^kin Re(b conj a); ka2 <= kmax (kin >= 0), tiny <= ka2 <= kmax (kin < 0)
  S_INERPROD_DY = 2, // inerprod(a, derivk2(b,2), 0)
  S_BAND_KA2 = 3,    // ka2 |a|^2 for lo <= ka2 <= hi (energy in the kup band, :559-561)
  S_BAND = 4,        // |a|^2 for lo <= ka2 <= hi
};

constexpr int kMaxTerms = 24;
struct SumTerm {
  int kind, ia, ib, kin;
};
struct SumList {
  int nterms;
  SumTerm t[kMaxTerms];
  double band_lo, band_hi;
};

constexpr int kSumThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kSumThreads)
k_halfplane_sums(const cpx<T>* __restrict__ p0, const cpx<T>* __restrict__ p1,
                 const cpx<T>* __restrict__ p2, const cpx<T>* __restrict__ p3, DevGrid gd,
                 SumList sl, double* __restrict__ partials) {
  double acc[kMaxTerms];
#pragma unroll
  for (int t = 0; t < kMaxTerms; ++t) acc[t] = 0.0;
  const cpx<T>* planes[4] = {p0, p1, p2, p3};
  const size_t total = (size_t)gd.nh * gd.n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    plane_ij(idx, gd.n, i, j);
    const int kx = kx_of(i, gd.n), ky = ky_of(j, gd.n);
    const int k2 = kx * kx + ky * ky;
    const double ka2 = (double)k2;
    const double two = i == 0 ? 1.0 : 2.0;
    cpx<double> v[4];
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      if (planes[p]) {
        const cpx<T> x = planes[p][idx];
        v[p] = mkc<double>((double)x.x, (double)x.y);
      } else {
        v[p] = mkc<double>(0.0, 0.0);
      }
    }
#pragma unroll
    for (int t = 0; t < kMaxTerms; ++t) {
      if (t >= sl.nterms) break;
      const SumTerm tm = sl.t[t];
      const cpx<double> a = v[tm.ia], b = v[tm.ib];
      double val = 0.0;
      switch (tm.kind) {
        case S_ENERGY:
          if (tm.kin >= 0 || k2 >= 1) val = two * (a.x * a.x + a.y * a.y) * powi(ka2, tm.kin);
          break;
        case S_INERPROD:
          if (k2 <= gd.kmaxi && (tm.kin >= 0 || k2 >= 1))
            val = two * powi(ka2, tm.kin) * (b.x * a.x + b.y * a.y);
          break;
        case S_INERPROD_DY:
          if (k2 <= gd.kmaxi) {
            const double dx = -(double)ky * b.y, dy = (double)ky * b.x;
            val = two * (dx * a.x + dy * a.y);
          }
          break;
        case S_BAND_KA2:
          if (ka2 <= sl.band_hi && ka2 >= sl.band_lo) val = two * ka2 * (a.x * a.x + a.y * a.y);
          break;
        default:  // S_BAND
          if (ka2 <= sl.band_hi && ka2 >= sl.band_lo) val = two * (a.x * a.x + a.y * a.y);
          break;
      }
      acc[t] += val;
    }
  }
  __shared__ double red[kSumThreads];
  for (int t = 0; t < sl.nterms; ++t) {
    red[threadIdx.x] = acc[t];
    __syncthreads();
    for (int s = kSumThreads / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kMaxTerms + t] = red[0];
    __syncthreads();
  }
}

// out[t] = scale * sum_b partials[b][t], sequential over b (fixed order).
static __global__ void k_finalize_sums(const double* __restrict__ partials, int nblocks, int nterms,
                                double scale, double* __restrict__ out) {
  const int t = threadIdx.x;
  if (t >= nterms) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partials[(size_t)b * kMaxTerms + t];
  out[t] = s * scale;
}

// ---------------------------------------------------------------------------
// shell sums (spectrum :615-712, transfers :715-837): one CTA per shell b,
// kmn = int(sqrt(ka2)+.5) == b  <=>  (2b-1)^2 < 4 ka2 < (2b+1)^2.
// out[(b-1)*5 + {0..4}] = Ek, Ezk, Fl0, Fl1, Fl2 (times 1/n^4).
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long isqrt_ll(long long v) {
  if (v <= 0) return 0;
  long long r = (long long)sqrt((double)v);
  while (r * r > v) --r;
  while ((r + 1) * (r + 1) <= v) ++r;
  return r;
}

constexpr int kShellThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kShellThreads)
k_shells(const cpx<T>* __restrict__ ps, const cpx<T>* __restrict__ vz,
         const cpx<T>* __restrict__ c2, const cpx<T>* __restrict__ c1, DevGrid gd, double scale,
         double* __restrict__ out) {
  const int b = blockIdx.x + 1;
  const int n = gd.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int NW = kShellThreads / 32;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const long long lo = (long long)(2 * b - 1) * (2 * b - 1);
  const long long hi = (long long)(2 * b + 1) * (2 * b + 1);
  const int kxmax = min(b, n / 2);
  for (int kx = warp; kx <= kxmax; kx += NW) {
    const long long l2 = lo - 4LL * kx * kx;  // need 4 ky^2 > l2
    const long long h2 = hi - 4LL * kx * kx;  // need 4 ky^2 < h2
    if (h2 <= 0) continue;
    long long kmin = 0;
    if (l2 >= 0) {
      kmin = isqrt_ll(l2 / 4);
      while (4 * kmin * kmin <= l2) ++kmin;
    }
    long long kmaxk = isqrt_ll(h2 / 4) + 1;
    while (kmaxk >= 0 && 4 * kmaxk * kmaxk >= h2) --kmaxk;
    if (kmaxk < kmin) continue;
    const double two = kx == 0 ? 1.0 : 2.0;
    const double ka2c = (double)kx * kx;
    // positive ky in [kmin, min(kmaxk, n/2-1)], negative ky in
    // [-min(kmaxk, n/2), -max(kmin,1)]
    for (int side = 0; side < 2; ++side) {
      long long a0, a1;
      if (side == 0) {
        a0 = kmin;
        a1 = min(kmaxk, (long long)(n / 2 - 1));
      } else {
        a0 = max(kmin, 1LL);
        a1 = min(kmaxk, (long long)(n / 2));
      }
      for (long long k = a0 + lane; k <= a1; k += 32) {
        const int j = side == 0 ? (int)k : (int)(n - k);
        const size_t idx = (size_t)kx * n + j;
        const double ka2 = ka2c + (double)(k * k);
        const cpx<T> p = ps[idx], z = vz[idx];
        const double pe = (double)p.x * p.x + (double)p.y * p.y;
        acc[0] += two * ka2 * pe;
        acc[1] += two * ((double)z.x * z.x + (double)z.y * z.y);
        if (c2) {
          const cpx<T> q2 = c2[idx], q1 = c1[idx];
          const double r2 = (double)p.x * q2.x + (double)p.y * q2.y;
          acc[2] += two * ka2 * r2;
          acc[3] += two * r2;
          acc[4] -= two * ((double)z.x * q1.x + (double)z.y * q1.y);
        }
      }
    }
  }
  __shared__ double red[kShellThreads];
  for (int t = 0; t < 5; ++t) {
    red[threadIdx.x] = acc[t];
    __syncthreads();
    for (int s = kShellThreads / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)(b - 1) * 5 + t] = red[0] * scale;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// CFL time step from the encoded max |grad psi|^2 (CFL_condition :892-895).
// No FMA contraction, so the result equals the host FP64 formula bit for bit.
// ---------------------------------------------------------------------------
struct CflCoef {
  double cfl, kcut, nrm, nuk, nuvk, w2;  // nuk = nu*kcut**(2nn), w2 = 2*omega
};

__device__ __forceinline__ double dec_ordered(unsigned long long e) {
  const unsigned long long b = (e & 0x8000000000000000ULL) ? (e & 0x7fffffffffffffffULL) : ~e;
  return __longlong_as_double((long long)b);
}

// one thread per run r: enc, scal at r * kScalStride, coefficients c[r]
static __global__ void k_cfl_dt(const unsigned long long* __restrict__ enc, const CflCoef* __restrict__ cc,
                                double* scal, int add_time, int nruns) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nruns) return;
  enc += r * kScalStride;
  scal += r * kScalStride;
  const CflCoef c = cc[r];
  const double m = dec_ordered(enc[0]);
  const double tmp = __ddiv_rn(sqrt(m), c.nrm);
  const double den = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(c.kcut, tmp), c.nuk), c.nuvk), c.w2);
  const double dt = __ddiv_rn(c.cfl, den);
  scal[0] = dt;
  if (add_time) scal[1] = __dadd_rn(scal[1], dt);
}

// one device scalar set from a kernel parameter (no host buffer to keep
// alive, so no host synchronisation)
static __global__ void k_set_scalar(double* p, double v) { *p = v; }

static __global__ void k_add_time(double* scal, int nruns) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nruns) scal[r * kScalStride + 1] = __dadd_rn(scal[r * kScalStride + 1], scal[r * kScalStride]);
}

// ---------------------------------------------------------------------------
// rand_force (pseudospec2D_Rot2D3C.f90:1063-1126): the plane is zero except
// at the chosen mode and, on the kx = 0 column, its conjugate mirror.  The
// host draws the mode and phase; the amplitude sqrt(2 fp0)/(sqrt(dt) kup^kin)
// is formed here from the device dt so a CFL step needs no host round trip.
// ---------------------------------------------------------------------------
struct RandForceField {
  int nclear, clear[4];  // entries set by the previous call
  int nset, set[4], conj[4];
  double c0, kpow, cph, sph;  // sqrt(2 fp0), kup**kin, cos(phase), sin(phase)
};
struct RandForceArgs {
  RandForceField f[2];
  double nsq;  // dble(n)**2
};

template <typename T>
__global__ void k_randforce(cpx<T>* fp, cpx<T>* fz, const double* __restrict__ scal, RandForceArgs a) {
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
}

// ---------------------------------------------------------------------------
// physical-space initial condition (Rot2D3C.para.f90:255-279) and the
// deterministic iflow = 1 forcing fields (:345-352)
// ---------------------------------------------------------------------------
struct IcMode {
  double kr, ph1, ph2, ph3, ph4;
  int ir, jr;
};

template <typename T>
__global__ void k_ic_phys(const IcMode* __restrict__ modes, int nmodes, int n, double pi,
                          T* __restrict__ r1, T* __restrict__ r2) {
  const size_t total = (size_t)n * n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(idx / n), x = (int)(idx % n);
    double a1 = 0.0, a2 = 0.0;
    const double xi = (double)x, yj = (double)y, dn = (double)n;
    for (int m = 0; m < nmodes; ++m) {
      const IcMode md = modes[m];
      const double ax = 2.0 * (md.ir - 1) * pi * xi / dn;
      const double ay = 2.0 * (md.jr - 1) * pi * yj / dn;
      a1 = a1 + cos(ax + md.ph1) * cos(ay + md.ph2) / md.kr;
      a2 = a2 + sin(ax + md.ph3) * cos(ay + md.ph4);
    }
    r1[idx] = (T)a1;
    r2[idx] = (T)a2;
  }
}

template <typename T>
__global__ void k_iflow1_phys(int n, double kup, double pi, T* __restrict__ r1, T* __restrict__ r2) {
  const size_t total = (size_t)n * n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(idx / n), x = (int)(idx % n);
    const double ax = 2 * kup * pi * (double)x / (double)n;
    const double ay = 2 * kup * pi * (double)y / (double)n;
    r1[idx] = (T)(sin(ax) + sin(ay));
    r2[idx] = (T)(cos(ax) + sin(ay));
  }
}

// Rescale inside the dealiasing mask tiny <= ka2 <= kmax, zero elsewhere
// (Rot2D3C.para.f90:288-298 and :361-371).
template <typename T>
__global__ void k_scale_mask2(cpx<T>* a, cpx<T>* b, DevGrid gd, double sa, double sb) {
  const size_t total = (size_t)gd.nh * gd.n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    plane_ij(idx, gd.n, i, j);
    const int kx = kx_of(i, gd.n), ky = ky_of(j, gd.n);
    const int k2 = kx * kx + ky * ky;
    const bool in = k2 <= gd.kmaxi && k2 >= 1;
    const cpx<T> x = a[idx], y = b[idx];
    a[idx] = in ? mkc<T>((T)(sa * (double)x.x), (T)(sa * (double)x.y)) : czero<T>();
    b[idx] = in ? mkc<T>((T)(sb * (double)y.x), (T)(sb * (double)y.y)) : czero<T>();
  }
}

// ---------------------------------------------------------------------------
// const_inj (pseudospec2D_Rot2D3C.f90:977-1060), iflow = 2.  The reference
// reseeds randu with myrank before the rescaling loop (:1032), so the random
// factors of the band elements form one fixed sequence in loop order; the
// host precomputes it together with the band element list.
// ---------------------------------------------------------------------------
// fp = ps/(|ps|^2+1) in kdn^2 <= ka2 <= kup^2, Hermitian fill on kx = 0
// (:1005-1028)
template <typename T>
__global__ void k_ci_base(const cpx<T>* __restrict__ src, cpx<T>* __restrict__ dst, DevGrid gd,
                          double lo, double hi) {
  const size_t total = (size_t)gd.nh * gd.n;
  const int n = gd.n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    plane_ij(idx, n, i, j);
    const int kx = kx_of(i, n), ky = ky_of(j, n);
    const double ka2 = (double)(kx * kx + ky * ky);
    const bool band = ka2 <= hi && ka2 >= lo;
    cpx<T> out = czero<T>();
    if (i != 0) {
      if (band) {
        const cpx<T> p = src[idx];
        const double d = (double)p.x * p.x + (double)p.y * p.y + 1.0;
        out = mkc<T>((T)((double)p.x / d), (T)((double)p.y / d));
      }
    } else if (j != 0 && j != n / 2 && band) {
      const int js = j < n / 2 ? j : n - j;
      const cpx<T> p = src[js];
      const double d = (double)p.x * p.x + (double)p.y * p.y + 1.0;
      out = mkc<T>((T)((double)p.x / d), (T)(j < n / 2 ? (double)p.y / d : -((double)p.y / d)));
    }
    dst[idx] = out;
  }
}

// fp = fp*fp0/Efp + i*randu*|k|*ps on the band (:1033-1057)
template <typename T>
__global__ void k_ci_rescale(const cpx<T>* __restrict__ src, cpx<T>* __restrict__ dst,
                             const int* __restrict__ band_idx, const int* __restrict__ mirror,
                             const float* __restrict__ rnd, int nband, double f0,
                             const double* __restrict__ efp, int n) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nband) return;
  const int idx = band_idx[e];
  const int i = idx / n, j = idx % n;
  const int kx = kx_of(i, n), ky = ky_of(j, n);
  const double t3 = (double)rnd[e] * sqrt((double)(kx * kx + ky * ky));
  const double E = *efp;
  const cpx<T> f = dst[idx], p = src[idx];
  const double vx = ((double)f.x * f0) / E + (-t3 * (double)p.y);
  const double vy = ((double)f.y * f0) / E + (t3 * (double)p.x);
  dst[idx] = mkc<T>((T)vx, (T)vy);
  if (mirror[e] >= 0) dst[mirror[e]] = mkc<T>((T)vx, (T)(-vy));
}

// ---------------------------------------------------------------------------
// learned-closure plumbing
// ---------------------------------------------------------------------------
// sharp spectral filter: coarse[kx][ky] = fine[kx][ky] * (nc/nf)^2 for
// kx^2 + ky^2 <= kmaxi of the coarse grid, else 0
template <typename T>
__global__ void k_coarsen(const cpx<T>* __restrict__ fine, int nf, cpx<T>* __restrict__ coarse, DevGrid gc,
                          double scale) {
  const size_t total = (size_t)gc.nh * gc.n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    plane_ij(idx, gc.n, i, j);
    const int ky = ky_of(j, gc.n);
    const int k2 = i * i + ky * ky;
    cpx<T> v = czero<T>();
    if (i < gc.n / 2 && k2 <= gc.kmaxi) {
      const cpx<T> f = fine[(size_t)i * nf + (ky >= 0 ? ky : nf + ky)];
      v = mkc<T>((T)(f.x * scale), (T)(f.y * scale));
    }
    coarse[idx] = v;
  }
}

// Spectral zero-padding onto a finer grid (the inverse of k_coarsen): every
// mode |kx|, |ky| < nc/2 of the coarse plane lands at the same wavenumber of
// the fine plane, times scale = (nf/nc)^2 (unnormalised transforms keep the
// physical amplitude); all other fine modes are zero.
template <typename T>
__global__ void k_refine(const cpx<T>* __restrict__ coarse, int nc, cpx<T>* __restrict__ fine, DevGrid gf,
                         double scale) {
  const size_t total = (size_t)gf.nh * gf.n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i, j;
    plane_ij(idx, gf.n, i, j);
    const int ky = ky_of(j, gf.n);
    cpx<T> v = czero<T>();
    if (i < nc / 2 && ky < nc / 2 && -ky < nc / 2) {
      const cpx<T> c = coarse[(size_t)i * nc + (ky >= 0 ? ky : nc + ky)];
      v = mkc<T>((T)(c.x * scale), (T)(c.y * scale));
    }
    fine[idx] = v;
  }
}

// c = a - b on spectral planes
template <typename T>
__global__ void k_spec_sub(const cpx<T>* __restrict__ a, const cpx<T>* __restrict__ b, cpx<T>* __restrict__ c,
                           size_t total) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    c[i] = mkc<T>(a[i].x - b[i].x, a[i].y - b[i].y);
}

// Per-shell weights of the learned tendencies: spectral plane a (S = nh * n
// elements) times w[b], plane b times w[nw + b], b the shell of (kx, ky) by
// the rule of k_shells (kmn = int(sqrt(ka2) + .5)); shells beyond nw get 0.
// In place when a_in == a and b_in == b; nw = 0 is a plain copy.
template <typename T>
__global__ void k_shell_weight2(const cpx<T>* a_in, const cpx<T>* b_in, cpx<T>* a, cpx<T>* b, DevGrid gd,
                                const float* __restrict__ w, int nw) {
  const size_t total = (size_t)gd.nh * gd.n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const cpx<T> u = a_in[i], v = b_in[i];
    if (nw <= 0) {
      a[i] = u;
      b[i] = v;
      continue;
    }
    int kx, j;
    plane_ij(i, gd.n, kx, j);
    const int ky = ky_of(j, gd.n);
    // (2b-1)^2 < 4 ka2 < (2b+1)^2  <=>  b = (isqrt(4 ka2) + 1) / 2
    const int bsh = (int)((isqrt_ll(4LL * ((long long)kx * kx + (long long)ky * ky)) + 1) / 2);
    const T fa = bsh < nw ? (T)w[bsh] : (T)0;
    const T fb = bsh < nw ? (T)w[nw + bsh] : (T)0;
    a[i] = mkc<T>(u.x * fa, u.y * fa);
    b[i] = mkc<T>(v.x * fb, v.y * fb);
  }
}

// The forward y-transform of the two tendency planes (columns 0 .. nh-1 of
// `in` into a, nh .. 2nh-1 into b, as k_colfft with a split output), each
// element times the band weight of its shell (the rule and the multiply of
// k_shell_weight2): the transform and the weighting of the captured LES
// step in one launch, the same bits as the two launches.
template <typename T, int N>
__global__ void __launch_bounds__(Cfg<T, N>::THREADS)
k_colfft_band2(const cpx<T>* __restrict__ in, cpx<T>* __restrict__ a, cpx<T>* __restrict__ b, int nh,
               const tw_t<T>* __restrict__ tw, const float* __restrict__ w, int nw) {
  using C = Cfg<T, N>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * F::SMEM_ELEMS;
  const int col = blockIdx.x * (blockDim.x / C::TPF) + g;  // groups per CTA: a launch-time choice
  const bool ok = col < 2 * nh;
  cpx<T> v[1][C::E];
#pragma unroll
  for (int q = 0; q < C::E; ++q) v[0][q] = ok ? in[(size_t)col * N + lane + q * C::TPF] : czero<T>();
  F::template run<-1>(v, lane, sm, tw);
  if (ok) {
    const bool second = col >= nh;
    const int kx = second ? col - nh : col;
    cpx<T>* dst = (second ? b : a) + (size_t)kx * N;
    const float* wp = w + (second ? nw : 0);
#pragma unroll
    for (int q = 0; q < C::E; ++q) {
      const int j = lane + q * C::TPF, ky = ky_of(j, N);
      const int bsh = (int)((isqrt_ll(4LL * ((long long)kx * kx + (long long)ky * ky)) + 1) / 2);
      const T f = bsh < nw ? (T)wp[bsh] : (T)0;
      dst[j] = mkc<T>(v[0][q].x * f, v[0][q].y * f);
    }
  }
}

// (float)(v * s) for the closure's scales s = +-1/n^2, powers of two (n is
// one): the FP32 product is exact (or the same correctly rounded subnormal)
// and equal to the FP64 product rounded to FP32, so the FP32 path keeps its
// conversions off the FP64 pipe
template <typename T>
__device__ __forceinline__ float scale_to_float(T v, double s) {
  if constexpr (sizeof(T) == 4) {
    return v * (float)s;
  } else {
    return (float)(v * s);
  }
}

// out[p*nch + ch] = r[p] * s  (real plane -> one channel of an FP32 NHWC tensor)
template <typename T>
__global__ void k_to_channel(const T* __restrict__ r, size_t count, double s, float* __restrict__ out, int nch,
                             int ch) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < count; p += (size_t)gridDim.x * blockDim.x)
    out[p * nch + ch] = scale_to_float(r[p], s);
}

// Spectral field c (0..7) of the closure's inputs at (kx, ky) from psi (x)
// and vz (z) (the specop chain of closure_inputs, same arithmetic):
// -k^2 psi, vz, d_x psi, d_y psi, d_x(-k^2 psi), d_y(-k^2 psi), d_x vz,
// d_y vz; every field but the first masked to k^2 <= kmax (the first is
// psi's own truncation).
template <typename T>
__device__ __forceinline__ cpx<T> closure_field(int c, cpx<T> x, cpx<T> z, int kx, int ky, int kmaxi) {
  const int k2 = kx * kx + ky * ky;
  const bool in = k2 <= kmaxi;
  const T m = -(T)k2;
  const cpx<T> L = mkc<T>(m * x.x, m * x.y);
  const T fx = (T)kx, fy = (T)ky;
  const cpx<T> zero = czero<T>();
  switch (c) {
    case 0: return L;
    case 1: return in ? z : zero;
    case 2: return in ? mkc<T>(-fx * x.y, fx * x.x) : zero;
    case 3: return in ? mkc<T>(-fy * x.y, fy * x.x) : zero;
    case 4: return in ? mkc<T>(-fx * L.y, fx * L.x) : zero;
    case 5: return in ? mkc<T>(-fy * L.y, fy * L.x) : zero;
    case 6: return in ? mkc<T>(-fx * z.y, fx * z.x) : zero;
    default: return in ? mkc<T>(-fy * z.y, fy * z.x) : zero;
  }
}

// The 8 closure-input fields and their inverse y-transforms in one kernel:
// column col of the 8 * nh output columns (field col / nh, kx index
// col % nh) is formed from psi and vz as it is loaded and transformed as
// k_colfft does (out: 8 mixed planes [kx][y], one after the other).
template <typename T, int N>
__global__ void __launch_bounds__(Cfg<T, N>::THREADS)
k_closure_cols(const cpx<T>* __restrict__ ps, const cpx<T>* __restrict__ vz, DevGrid gd, cpx<T>* __restrict__ out,
               const tw_t<T>* __restrict__ tw) {
  using C = Cfg<T, N>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * F::SMEM_ELEMS;
  const int col = blockIdx.x * (blockDim.x / C::TPF) + g;  // groups per CTA: a launch-time choice
  const bool ok = col < 8 * gd.nh;
  const int c = ok ? col / gd.nh : 0, i = ok ? col % gd.nh : 0;
  const int kx = kx_of(i, N);
  cpx<T> v[1][C::E];
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    const int j = lane + q * C::TPF;
    const size_t idx = (size_t)i * N + j;
    v[0][q] = ok ? closure_field<T>(c, ps[idx], vz[idx], kx, ky_of(j, N), gd.kmaxi) : czero<T>();
  }
  F::template run<+1>(v, lane, sm, tw);
  if (ok) {
    cpx<T>* dst = out + (size_t)col * N;
#pragma unroll
    for (int q = 0; q < C::E; ++q) dst[lane + q * C::TPF] = v[0][q];
  }
}

// out[p*8 + c] = r8[c*count + p] * s[c]  (8 real planes -> FP32 NHWC)
template <typename T>
__global__ void k_to_channels8(const T* __restrict__ r8, size_t count, Scale8 s, float* __restrict__ out) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < count; p += (size_t)gridDim.x * blockDim.x) {
    float o[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) o[c] = scale_to_float(r8[c * count + p], s.v[c]);
    reinterpret_cast<float4*>(out + p * 8)[0] = make_float4(o[0], o[1], o[2], o[3]);
    reinterpret_cast<float4*>(out + p * 8)[1] = make_float4(o[4], o[5], o[6], o[7]);
  }
}

// r2[c*count + p] = in[p*2 + c], c = 0, 1  (FP32 NHWC, 2 channels -> 2 real planes)
template <typename T>
__global__ void k_from_channels2(const float* __restrict__ in, size_t count, T* __restrict__ r2) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < count; p += (size_t)gridDim.x * blockDim.x) {
    const float2 v = reinterpret_cast<const float2*>(in)[p];
    r2[p] = (T)v.x;
    r2[count + p] = (T)v.y;
  }
}

// Fused closure path of the LES step (n <= 512).
//
// k_rows_to_cnn8: the row C2R of the 8 closure-input planes of row pair y0
// (one transform group per plane, as k_rowc2r), then per pixel of the two
// rows the 8 channel values scaled by s (k_to_channels8) and standardised
// and rounded to bf16 (the network's input conversion), written as the 16
// bf16 channels (8 zero) of the network's first activation: 32 bytes per
// pixel.  Same arithmetic, in the same order, as the three separate kernels.
template <typename T, int N>
struct RowsCnn {
  using C = Cfg<T, N>;
  static constexpr int THREADS = 8 * C::TPF;
  static constexpr size_t SMEM = 8 * C::FFT::SMEM_BYTES;
  static constexpr bool OK = N <= 512 && THREADS <= 1024 && (size_t)C::FFT::SMEM_ELEMS * 2 >= (size_t)2 * N;
};
template <typename T, int N>
__global__ void __launch_bounds__(RowsCnn<T, N>::THREADS)
k_rows_to_cnn8(const cpx<T>* __restrict__ tin, Scale8 s, const float* __restrict__ mean,
               const float* __restrict__ sd, __nv_bfloat16* __restrict__ act, const tw_t<T>* __restrict__ tw) {
  using C = Cfg<T, N>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;  // g: channel plane
  cpx<T>* sm = smbase_ + (size_t)g * F::SMEM_ELEMS;
  const cpx<T>* in = tin + (size_t)g * (N / 2 + 1) * N;
  const int y0 = 2 * blockIdx.x;
  cpx<T> v[1][C::E];
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    const int k = lane + q * C::TPF;
    const int kk = k <= N / 2 ? k : N - k;
    const cpx<T> a = in[(size_t)kk * N + y0];
    const cpx<T> b = in[(size_t)kk * N + y0 + 1];
    if (k == 0 || k == N / 2) {
      v[0][q] = mkc<T>(a.x, b.x);
    } else if (k < N / 2) {
      v[0][q] = mkc<T>(a.x - b.y, a.y + b.x);
    } else {
      v[0][q] = mkc<T>(a.x + b.y, b.x - a.y);
    }
  }
  F::template run<+1>(v, lane, sm, tw);
  __syncthreads();  // every group's transform is done with its buffer
  T* rows = reinterpret_cast<T*>(sm);  // this plane's rows y0, y0 + 1: [2][N]
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    rows[lane + q * C::TPF] = v[0][q].x;
    rows[N + lane + q * C::TPF] = v[0][q].y;
  }
  __syncthreads();
  for (int p = threadIdx.x; p < 2 * N; p += blockDim.x) {
    unsigned u[8];
#pragma unroll
    for (int c = 0; c < 8; c += 2) {
      float o[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const T val = reinterpret_cast<const T*>(smbase_ + (size_t)(c + h) * F::SMEM_ELEMS)[p];
        const float x = scale_to_float(val, s.v[c + h]);
        o[h] = (x - mean[c + h]) / sd[c + h];
      }
      const __nv_bfloat162 b2 = __floats2bfloat162_rn(o[0], o[1]);
      u[c / 2] = *reinterpret_cast<const unsigned*>(&b2);
    }
    u[4] = u[5] = u[6] = u[7] = 0u;  // channels 8-15: padding
    uint4* dst = reinterpret_cast<uint4*>(act + ((size_t)(y0 + p / N) * N + p % N) * 16);
    dst[0] = make_uint4(u[0], u[1], u[2], u[3]);
    dst[1] = make_uint4(u[4], u[5], u[6], u[7]);
  }
}

// k_cnn2_to_rows: the network's output (standardised, FP32 NHWC, 2
// channels; blockIdx.y = channel) de-standardised as the network's own
// output conversion does (y * sd + mean, one fused multiply-add), as the two
// rows of row pair y0 of that channel's tendency plane, then the row R2C of
// k_rowr2c: k_denorm + k_from_channels2 + k_rowr2c in one kernel.
template <typename T, int N>
__global__ void __launch_bounds__(Cfg<T, N>::THREADS)
k_cnn2_to_rows(const float* __restrict__ y, const float* __restrict__ mean, const float* __restrict__ sd,
               cpx<T>* __restrict__ tout, const tw_t<T>* __restrict__ tw) {
  using C = Cfg<T, N>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int ch = blockIdx.y;
  tout += ch * (size_t)(N / 2 + 1) * N;
  const float m = mean[ch], d = sd[ch];
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * F::SMEM_ELEMS;
  int pair = blockIdx.x * (blockDim.x / C::TPF) + g;  // groups per CTA: a launch-time choice
  const bool ok = pair < N / 2;
  if (!ok) pair = 0;
  const int y0 = 2 * pair;
  cpx<T> v[1][C::E];
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    const int x = lane + q * C::TPF;
    const T a = (T)fmaf(y[((size_t)y0 * N + x) * 2 + ch], d, m);
    const T b = (T)fmaf(y[((size_t)(y0 + 1) * N + x) * 2 + ch], d, m);
    v[0][q] = mkc<T>(a, b);
  }
  F::template run<-1>(v, lane, sm, tw);
  F::to_smem(v, lane, sm);
  fft_sync<C::TPF>();
  const T h = (T)0.5;
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    const int k = lane + q * C::TPF;
    if (ok && k <= N / 2) {
      const cpx<T> w = F::from_smem(0, k, sm);
      const cpx<T> u = F::from_smem(0, (N - k) & (N - 1), sm);
      tout[(size_t)k * N + y0] = mkc<T>((w.x + u.x) * h, (w.y - u.y) * h);
      tout[(size_t)k * N + y0 + 1] = mkc<T>((w.y + u.y) * h, (u.x - w.x) * h);
    }
  }
}

// r[p] = in[p*nch + ch]
template <typename T>
__global__ void k_from_channel(const float* __restrict__ in, int nch, int ch, size_t count, T* __restrict__ r) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < count; p += (size_t)gridDim.x * blockDim.x)
    r[p] = (T)in[p * nch + ch];
}

}  // namespace r2d3c

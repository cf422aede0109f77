// Device kernels of the Rot2D3C time-step hot path (sm_103a).
//
// Data layout in HBM (identical to the reference's Fortran arrays):
//   spectral plane  C[kx][ky]  kx in [0, n/2], ky index j in [0, n), ky fastest
//                   (Fortran C(n, n/2+1), fftp2D.f90:153)
//   physical plane  R[y][x]    x fastest (Fortran R(n, n), fftp2D.f90:157)
//   mixed plane     T[kx][y]   result of the y-direction transform of one kx
//                   column, y fastest; used between the column and row passes
//
// Hot path of one RK substep (Rot2D3C.para.f90:571-599), three passes:
//   A  per kx column (kx <= n/3): the six masked spectral derivatives
//      d_x psi, d_y psi, d_x(-k^2 psi), d_y(-k^2 psi), d_x vz, d_y vz
//      (derivk2/laplak2, pseudospec2D_Rot2D3C.f90:6-95) and their inverse
//      y-FFTs -> 6 mixed planes.  Only |ky| <= n/3 is read (2/3 truncation).
//   B  per physical row y: three packed complex x-IFFTs give the six real
//      derivative rows (two real C2R per complex transform), the brackets
//      [psi,-k^2 psi] and [psi,vz] (poisson, :169-226) are formed in
//      registers, scaled by 1/n^4, and one packed forward x-FFT returns both
//      to mixed space; only kx <= n/3 is written.  Substep 1 also takes the
//      CFL maximum of |grad psi|^2 (CFL_condition, :862-876).
//   C  per kx column: forward y-FFT of both brackets and the semi-implicit
//      RK update with Coriolis coupling and forcing (Rot2D3C.para.f90:578-599).
#pragma once

#include <type_traits>

#include "r2d3c_fft.cuh"

namespace r2d3c {

struct DevGrid {
  int n;      // grid points per direction (power of two)
  int nh;     // n/2 + 1 spectral columns
  int L;      // floor(n/3): largest retained |kx|, |ky|
  int M;      // L + 1 retained kx columns
  int kmaxi;  // floor((n/3)^2): ka2 <= kmax  <=>  kx^2+ky^2 <= kmaxi
};

struct StepCoef {
  double nu, hnu, nuv, hnuv, w2;  // w2 = 2*omega
  int nn, mm, nnv, mmv;
};

// Element strides between the runs of a batched launch (blockIdx.y = run):
// spectral planes, the six derivative planes, the two product planes.  A
// single run uses gridDim.y = 1.  Per-run scalars (dt, time, CFL maximum)
// sit 8 entries apart.
struct Batch {
  size_t spec, tf, pb;
};
constexpr int kScalStride = 8;

// Launch shape of a kernel carrying NT transforms per thread group: E
// elements per thread, TPF = N/E threads per transform group, G groups per CTA.
template <typename T, int N, int NT = 1, int EOVR = 0, bool ILV_OK = true>
struct Cfg {
  static constexpr int E = EOVR ? EOVR : (N >= 8192 ? 16 : 8);
  using FFT = BlockFFT<T, N, E, NT, ILV_OK>;
  static constexpr int TPF = N / E;
  static constexpr int G = TPF >= 256 ? 1 : 256 / TPF;  // transform groups per CTA
  static constexpr int THREADS = TPF * G;
  static constexpr size_t SMEM = (size_t)G * FFT::SMEM_BYTES;
};

// Transforms carried at once by one group in passes A, B and C.  Two in the
// FP32 path up to n = 4096 ("tiled" mode): pass A and C transform two
// adjacent kx columns, pass B two adjacent rows, and the mixed planes use the
// pair-tiled layout below so that every access moves whole 32-byte sectors.
// One in the FP64 path (its FP64 arithmetic is the bound and its register
// budget is full) and at n = 8192: plain column layout T[kx][y].
template <typename T, int N> struct PassNT {
  static constexpr int value = (sizeof(T) == 4 && N <= 4096) ? 2 : 1;
};

// Elements per thread of pass A: radix-16 (up to 255 registers, fewer
// exchanges per transform) for the FP32 grids 1024-4096, where it measured
// faster; the default radix elsewhere.  Pass A then needs the twiddle table
// of its own stage schedule.
template <typename T, int N> struct PassAE {
  static constexpr int value = (sizeof(T) == 4 && N >= 1024 && N <= 4096) ? 16 : Cfg<T, N>::E;
};
// (pass A keeps the two transforms' exchange buffers separate: with its 255
// registers the interleaved float4 exchange measured slower)
template <typename T, int N>
using CfgA = Cfg<T, N, PassNT<T, N>::value, PassAE<T, N>::value, PassAE<T, N>::value != 16>;
// Pass A with radix EA (the plan autotuner may pick the other radix where
// two exist: FP32, n = 1024 .. 4096, radix 16 or 8)
template <typename T, int N, int EA>
using CfgAE = Cfg<T, N, PassNT<T, N>::value, EA, EA != 16>;
template <typename T, int N>
constexpr bool kAltRadixA = PassAE<T, N>::value != Cfg<T, N>::E;

// Shared memory of passes B and C: NT transform buffers per group, plus (when
// it fits) a store for the first transform's result, which is held across the
// later transforms (pass B: dx psi + i dy psi; pass C: the [psi,-k^2 psi]
// column) -- keeping it out of registers avoids spills.
template <typename T, int N>
struct PassSmem {
  static constexpr int NT = PassNT<T, N>::value;
  using C = Cfg<T, N, NT>;
  static constexpr size_t HOLD_BYTES = (size_t)NT * N * sizeof(cpx<T>);
  static constexpr bool HOLD = C::FFT::SMEM_BYTES + HOLD_BYTES <= 200 * 1024;
  static constexpr size_t GROUP_ELEMS = (size_t)NT * C::FFT::SMEM_ELEMS + (HOLD ? (size_t)NT * N : 0);
  static constexpr size_t SMEM = (size_t)C::G * GROUP_ELEMS * sizeof(cpx<T>);
};

// Mixed-plane element (kx, y) of a plane holding MX columns.  Column layout
// (PY = 1 transform per group): kx*N + y.  Pair-tiled layout (PY = 2): rows
// y = 2p, 2p+1 of all MX columns form one contiguous tile, each column's two
// rows adjacent: ((y/2)*MX + kx)*2 + y%2.  Both layouts hold N*MX elements.
template <int N, int PY>
__host__ __device__ __forceinline__ size_t mix_idx(int kx, int y, int MX) {
  if constexpr (PY == 2) {
    return ((size_t)(y >> 1) * MX + kx) * 2 + (y & 1);
  } else {
    return (size_t)kx * N + y;
  }
}

// ky value of row index j (Rot2D3C.para.f90:220-223)
__device__ __forceinline__ int ky_of(int j, int n) { return j < (n >> 1) ? j : j - n; }

// x through an opaque move: the compiler cannot treat the result as equal
// to x, so values derived from it are not hoisted out of a loop
__device__ __forceinline__ int opaque(int x) {
  int r;
  asm volatile("mov.b32 %0, %1;" : "=r"(r) : "r"(x));
  return r;
}

template <typename T>
__device__ __forceinline__ cpx<T> czero() {
  return mkc<T>((T)0, (T)0);
}

// Non-negative double -> order-preserving 64-bit key for atomicMax (CFL max);
// signed doubles use the sign-flip encoding below.
__device__ __forceinline__ unsigned long long enc_ordered(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}

template <typename T>
__device__ __forceinline__ T powi(T x, int k) {
  if (k == 0) return (T)1;
  unsigned e = k < 0 ? (unsigned)(-k) : (unsigned)k;
  T r = (T)1, b = x;
  while (true) {
    if (e & 1u) r = r * b;
    e >>= 1;
    if (!e) break;
    b = b * b;
  }
  return k < 0 ? (T)1 / r : r;
}

#define R2D3C_SMEM_DECL                                     \
  extern __shared__ __align__(16) unsigned char smraw_[]; \
  cpx<T>* smbase_ = reinterpret_cast<cpx<T>*>(smraw_);

// --------------------------------------------------------------------------
// generic y-direction transform of `ncols` contiguous columns of length N
// (fftp2D.f90:208 forward, :251 inverse), in place allowed; columns from
// `split` on go to out2 (two output planes of one launch)
// --------------------------------------------------------------------------
template <typename T, int N, int DIR, int PY = 1>
__global__ void __launch_bounds__(Cfg<T, N>::THREADS)
k_colfft(const cpx<T>* __restrict__ in, cpx<T>* out, int ncols, const tw_t<T>* __restrict__ tw,
         int mx_in = 0, cpx<T>* out2 = nullptr, int split = 0x7fffffff) {
  using C = Cfg<T, N>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * F::SMEM_ELEMS;
  const int col = blockIdx.x * (blockDim.x / C::TPF) + g;  // groups per CTA: a launch-time choice
  const bool ok = col < ncols;
  cpx<T> v[1][C::E];
#pragma unroll
  for (int q = 0; q < C::E; ++q)
    v[0][q] = ok ? in[mix_idx<N, PY>(col, lane + q * C::TPF, mx_in)] : czero<T>();
  F::template run<DIR>(v, lane, sm, tw);
  if (ok) {
    cpx<T>* dst = col < split ? out + (size_t)col * N : out2 + (size_t)(col - split) * N;
#pragma unroll
    for (int q = 0; q < C::E; ++q) dst[lane + q * C::TPF] = v[0][q];
  }
}

// --------------------------------------------------------------------------
// generic x-direction C2R of two rows (y0, y0+1) per transform: the two
// Hermitian spectra are packed as Z = Xa + i Xb so one complex IFFT returns
// row y0 in the real and row y0+1 in the imaginary part.  Im at kx = 0 and
// kx = n/2 is ignored, as FFTW's complex-to-real does (fftp2D.f90:286).
// Optionally stores the rows and/or folds them into a max/min.
// --------------------------------------------------------------------------
template <typename T, int N>
__global__ void __launch_bounds__(Cfg<T, N>::THREADS)
k_rowc2r(const cpx<T>* __restrict__ tin, T* __restrict__ rout,
         unsigned long long* __restrict__ mm_enc, const tw_t<T>* __restrict__ tw) {
  using C = Cfg<T, N>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  // blockIdx.y: plane of a batch of consecutive mixed / real planes
  tin += blockIdx.y * (size_t)(N / 2 + 1) * N;
  if (rout) rout += blockIdx.y * (size_t)N * N;
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * F::SMEM_ELEMS;
  int pair = blockIdx.x * (blockDim.x / C::TPF) + g;  // groups per CTA: a launch-time choice
  const bool ok = pair < N / 2;
  if (!ok) pair = 0;  // surplus groups recompute pair 0 and store nothing
  const int y0 = 2 * pair;
  cpx<T> v[1][C::E];
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    const int k = lane + q * C::TPF;
    const int kk = k <= N / 2 ? k : N - k;
    const cpx<T> a = tin[(size_t)kk * N + y0];
    const cpx<T> b = tin[(size_t)kk * N + y0 + 1];
    if (k == 0 || k == N / 2) {
      v[0][q] = mkc<T>(a.x, b.x);
    } else if (k < N / 2) {
      v[0][q] = mkc<T>(a.x - b.y, a.y + b.x);
    } else {
      v[0][q] = mkc<T>(a.x + b.y, b.x - a.y);
    }
  }
  F::template run<+1>(v, lane, sm, tw);
  if (rout && ok) {
#pragma unroll
    for (int q = 0; q < C::E; ++q) {
      const int x = lane + q * C::TPF;
      rout[(size_t)y0 * N + x] = v[0][q].x;
      rout[(size_t)(y0 + 1) * N + x] = v[0][q].y;
    }
  }
  if (mm_enc) {
    double mx = (double)v[0][0].x, mn = (double)v[0][0].x;
#pragma unroll
    for (int q = 0; q < C::E; ++q) {
      mx = fmax(mx, fmax((double)v[0][q].x, (double)v[0][q].y));
      mn = fmin(mn, fmin((double)v[0][q].x, (double)v[0][q].y));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&mm_enc[0], enc_ordered(mx));
      atomicMax(&mm_enc[1], enc_ordered(-mn));
    }
  }
}

// --------------------------------------------------------------------------
// generic x-direction R2C of two rows per transform (fftp2D.f90:171):
// z = r[y0] + i r[y0+1]; Xa = (W[k] + conj W[N-k])/2, Xb = (W[k] - conj W[N-k])/2i
// written to the mixed plane T[kx][y] for kx in [0, N/2].
// --------------------------------------------------------------------------
template <typename T, int N>
__global__ void __launch_bounds__(Cfg<T, N>::THREADS)
k_rowr2c(const T* __restrict__ rin, cpx<T>* __restrict__ tout, const tw_t<T>* __restrict__ tw) {
  using C = Cfg<T, N>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  // blockIdx.y: plane of a batch of consecutive real / mixed planes
  rin += blockIdx.y * (size_t)N * N;
  tout += blockIdx.y * (size_t)(N / 2 + 1) * N;
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
    v[0][q] = mkc<T>(rin[(size_t)y0 * N + x], rin[(size_t)(y0 + 1) * N + x]);
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

// --------------------------------------------------------------------------
// pass A: masked derivatives + inverse y-FFT, 6 fields per kx column.  In
// tiled mode each group transforms two adjacent columns at once and writes
// both as 16-byte column pairs of the pair-tiled plane.
// --------------------------------------------------------------------------
template <typename T, int N, int EA = PassAE<T, N>::value>
__global__ void __launch_bounds__(CfgAE<T, N, EA>::THREADS, (sizeof(T) == 4 && CfgAE<T, N, EA>::THREADS == 256) ? 2 : 1)
k_passA(const cpx<T>* __restrict__ ps, const cpx<T>* __restrict__ vz, cpx<T>* __restrict__ tf,
        DevGrid gd, const tw_t<T>* __restrict__ tw, Batch bs) {
  constexpr int NT = PassNT<T, N>::value;
  ps += blockIdx.y * bs.spec;
  vz += blockIdx.y * bs.spec;
  tf += blockIdx.y * bs.tf;
  using C = CfgAE<T, N, EA>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * NT * F::SMEM_ELEMS;
  // groups per CTA and field chunks are launch-time choices (blockDim.x =
  // groups * TPF, gridDim.z chunks of the six fields): small grids spread
  // one column pair's fields over several CTAs; the arithmetic per field is
  // the same whatever the split
  const int kx0 = (blockIdx.x * (blockDim.x / C::TPF) + g) * NT;
  const int fpc = 6 / gridDim.z, f0 = blockIdx.z * fpc;
  const size_t plane = (size_t)gd.M * N;
  int kyi[C::E];
#pragma unroll
  for (int q = 0; q < C::E; ++q) kyi[q] = ky_of(lane + q * C::TPF, N);
  // The source column (pair) is re-read for every field, from L2, rather
  // than held in registers across the fields: the registers freed let FP32
  // run two 256-thread CTAs per SM (and keep FP64 from spilling)
  cpx<T> v[NT][C::E];
  auto src_at = [&](const cpx<T>* sp, int t, int q) -> cpx<T> {
    const int col = kx0 + t, ky = kyi[q];
    const bool in = col < gd.M && (ky <= gd.L && -ky <= gd.L) && col * col + ky * ky <= gd.kmaxi;
    return in ? sp[(size_t)col * N + lane + q * C::TPF] : czero<T>();
  };
#pragma unroll 1
  for (int f = f0; f < f0 + fpc; ++f) {
    const cpx<T>* sp = f < 4 ? ps : vz;  // psi for fields 0-3, vz for fields 4-5
    {
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        const int col = kx0 + t;
#pragma unroll
        for (int q = 0; q < C::E; ++q) {
          // (0,k)*(x,y) = (-k*y, k*x): derivk2 dir 1 (k = kx) / dir 2 (k = ky)
          const T k = (f & 1) ? (T)kyi[q] : (T)col;
          cpx<T> x = src_at(sp, t, q);
          if (f == 2 || f == 3) {
            const T m = -(T)(col * col + kyi[q] * kyi[q]);  // laplak2: -ka2*a
            x = mkc<T>(m * x.x, m * x.y);
          }
          v[t][q] = mkc<T>(-k * x.y, k * x.x);
        }
      }
      F::template run<+1>(v, lane, sm, tw);
      cpx<T>* dst = tf + (size_t)f * plane;
      if constexpr (NT == 2) {
        // lanes (2p, 2p+1) hold rows y = 2p, 2p+1 of columns kx0, kx0+1: swap
        // one value so each lane writes one column's row pair (16 bytes)
        const bool odd = lane & 1;
        const int kx = kx0 + (odd ? 1 : 0);
#pragma unroll
        for (int q = 0; q < C::E; ++q) {
          const cpx<T> give = odd ? v[0][q] : v[1][q];
          cpx<T> got;
          got.x = __shfl_xor_sync(0xffffffffu, give.x, 1);
          got.y = __shfl_xor_sync(0xffffffffu, give.y, 1);
          const int y = (lane + q * C::TPF) & ~1;
          if (kx < gd.M) {
            const cpx<T> lo = odd ? got : v[0][q];
            const cpx<T> hi = odd ? v[1][q] : got;
            *reinterpret_cast<float4*>(dst + mix_idx<N, 2>(kx, y, gd.M)) = make_float4(lo.x, lo.y, hi.x, hi.y);
          }
        }
      } else {
        if (kx0 < gd.M) {
#pragma unroll
          for (int q = 0; q < C::E; ++q) dst[(size_t)kx0 * N + lane + q * C::TPF] = v[0][q];
        }
      }
    }
  }
}

// NR consecutive rows y0.. of a mixed plane at column kx: one 16-byte load
// for two FP32 rows.
template <typename T, int NR>
__device__ __forceinline__ void load_rows(const cpx<T>* __restrict__ p, size_t off, cpx<T> (&o)[NR]) {
  if constexpr (NR == 2 && sizeof(T) == 4) {
    const float4 w = __ldg(reinterpret_cast<const float4*>(p + off));
    o[0] = mkc<T>(w.x, w.y);
    o[1] = mkc<T>(w.z, w.w);
  } else {
#pragma unroll
    for (int t = 0; t < NR; ++t) o[t] = p[off + t];
  }
}

template <typename T, int NR>
__device__ __forceinline__ void store_rows(cpx<T>* __restrict__ p, size_t off, const cpx<T> (&o)[NR]) {
  if constexpr (NR == 2 && sizeof(T) == 4) {
    *reinterpret_cast<float4*>(p + off) = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
  } else {
#pragma unroll
    for (int t = 0; t < NR; ++t) p[off + t] = o[t];
  }
}

// Packed spectrum of a pair of mixed planes (A, B) at rows y0.. for x-position
// k: Z[k] = A[k] + i B[k] on the retained kx < M, conj-extended for k > N - M.
template <typename T, int N, int NR>
__device__ __forceinline__ void packed_pair(const cpx<T>* __restrict__ pa, const cpx<T>* __restrict__ pb,
                                            int k, int y0, int M, cpx<T> (&z)[NR]) {
  if (k < M || k > N - M) {
    const int kk = k < M ? k : N - k;
    cpx<T> a[NR], b[NR];
    const size_t off = mix_idx<N, NR>(kk, y0, M);
    load_rows<T, NR>(pa, off, a);
    load_rows<T, NR>(pb, off, b);
#pragma unroll
    for (int t = 0; t < NR; ++t) {
      if (k == 0) {
        z[t] = mkc<T>(a[t].x, b[t].x);  // Im of the kx = 0 column is ignored
      } else if (k < M) {
        z[t] = mkc<T>(a[t].x - b[t].y, a[t].y + b[t].x);
      } else {
        z[t] = mkc<T>(a[t].x + b[t].y, b[t].x - a[t].y);
      }
    }
  } else {
#pragma unroll
    for (int t = 0; t < NR; ++t) z[t] = czero<T>();
  }
}

// --------------------------------------------------------------------------
// pass B: per group NR rows; the two brackets in physical space and back to
// mixed space
// --------------------------------------------------------------------------
// CFL maximum of |grad psi|^2 = x^2 + y^2 over a thread's values of
// z1 = d_x psi + i d_y psi (CFL_condition, pseudospec2D_Rot2D3C.f90:867-874),
// folded into the run's encoded maximum.  The squares are formed in the
// compute type (an FP64 square per value would double the FP32 pass's time
// on GB300's FP64 rate); the maximum is kept in FP64.
template <typename T, int NT, int E>
__device__ __forceinline__ void cfl_max_sq(const cpx<T> (&v)[NT][E], unsigned long long* enc) {
  T m = (T)0;
#pragma unroll
  for (int t = 0; t < NT; ++t)
#pragma unroll
    for (int q = 0; q < E; ++q) m = max(m, v[t][q].x * v[t][q].x + v[t][q].y * v[t][q].y);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(enc, enc_ordered((double)m));
}

// Pass B with one rolled copy of the transform code (a loop over the four
// transforms that is not unrolled) and the first bracket p1 in shared
// memory, for the FP32 grid with one row per group (n = 8192): unrolled,
// the compiler interleaves the four 8192-point transforms and spills
// hundreds of bytes per thread.  The forward transform is the inverse one
// of the conjugate, conjugated: bit-identical to the unrolled form.
template <typename T, int N>
struct RolledB {
  static constexpr bool OK = sizeof(T) == 4 && PassNT<T, N>::value == 1 && PassSmem<T, N>::HOLD;
  static constexpr size_t SMEM = PassSmem<T, N>::SMEM + (OK ? (size_t)Cfg<T, N, 1>::G * N * sizeof(T) : 0);
};

template <typename T, int N, bool CFL>
__global__ void __launch_bounds__(Cfg<T, N, PassNT<T, N>::value>::THREADS, 1)
k_passB(const cpx<T>* __restrict__ tf, cpx<T>* __restrict__ pb, int kxo, DevGrid gd, T inv_n4,
        const tw_t<T>* __restrict__ tw, unsigned long long* __restrict__ cfl_enc, Batch bs) {
  constexpr int NR = PassNT<T, N>::value;
  using PS = PassSmem<T, N>;
  constexpr bool HOLD = PS::HOLD;
  tf += blockIdx.y * bs.tf;
  pb += blockIdx.y * bs.pb;
  cfl_enc += blockIdx.y * kScalStride;
  using C = Cfg<T, N, NR>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / C::TPF, lane = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * PS::GROUP_ELEMS;
  cpx<T>* hold = sm + NR * F::SMEM_ELEMS;  // z1 store (HOLD)
  int rg = blockIdx.x * (blockDim.x / C::TPF) + g;  // groups per CTA: a launch-time choice
  const bool ok = rg < N / NR;
  if (!ok) rg = 0;  // surplus groups recompute rows 0.. and store nothing
  const int y0 = rg * NR;
  const int M = gd.M;
  const size_t plane = (size_t)M * N;
  cpx<T> v[NR][C::E];
  if constexpr (RolledB<T, N>::OK) {
    T* P1 = reinterpret_cast<T*>(smbase_ + (size_t)(blockDim.x / C::TPF) * PS::GROUP_ELEMS) + (size_t)g * N;
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
      if (f < 3) {
        const cpx<T>* pa = tf + (size_t)(2 * f) * plane;
#pragma unroll
        for (int q = 0; q < C::E; ++q) {
          cpx<T> z[1];
          packed_pair<T, N, 1>(pa, pa + plane, lane + q * C::TPF, y0, M, z);
          v[0][q] = z[0];
        }
      } else {
#pragma unroll
        for (int q = 0; q < C::E; ++q) v[0][q].y = -v[0][q].y;
      }
      F::template run<+1>(v, lane, sm, tw);
      // each thread reads back only the positions it wrote: no barrier needed
      if (f == 0) {
        if constexpr (CFL) cfl_max_sq<T, 1, C::E>(v, cfl_enc);
#pragma unroll
        for (int q = 0; q < C::E; ++q) hold[lane + q * C::TPF] = v[0][q];
      } else if (f == 1) {
#pragma unroll
        for (int q = 0; q < C::E; ++q) {
          const cpx<T> a = hold[lane + q * C::TPF];
          P1[lane + q * C::TPF] = (a.x * v[0][q].y - a.y * v[0][q].x) * inv_n4;
        }
      } else if (f == 2) {
#pragma unroll
        for (int q = 0; q < C::E; ++q) {
          const cpx<T> a = hold[lane + q * C::TPF];
          v[0][q] = mkc<T>(P1[lane + q * C::TPF], (a.x * v[0][q].y - a.y * v[0][q].x) * inv_n4);
        }
      } else {
#pragma unroll
        for (int q = 0; q < C::E; ++q) v[0][q].y = -v[0][q].y;
      }
    }
  } else {
  cpx<T> z1r[HOLD ? 1 : NR][C::E];
  T p1[NR][C::E];
  // pair (d_x psi, d_y psi)
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    cpx<T> z[NR];
    packed_pair<T, N, NR>(tf, tf + plane, lane + q * C::TPF, y0, M, z);
#pragma unroll
    for (int t = 0; t < NR; ++t) v[t][q] = z[t];
  }
  F::template run<+1>(v, lane, sm, tw);
  if constexpr (CFL) cfl_max_sq<T, NR, C::E>(v, cfl_enc);
  // each thread reads back only the positions it wrote: no barrier needed
  auto z1 = [&](int t, int q) -> cpx<T> {
    if constexpr (HOLD) return hold[t * N + lane + q * C::TPF];
    else return z1r[t][q];
  };
#pragma unroll
  for (int t = 0; t < NR; ++t)
#pragma unroll
    for (int q = 0; q < C::E; ++q) {
      if constexpr (HOLD) hold[t * N + lane + q * C::TPF] = v[t][q];
      else z1r[t][q] = v[t][q];
    }
  // pair (d_x(-k^2 psi), d_y(-k^2 psi)) -> [psi, -k^2 psi]
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    cpx<T> z[NR];
    packed_pair<T, N, NR>(tf + 2 * plane, tf + 3 * plane, lane + q * C::TPF, y0, M, z);
#pragma unroll
    for (int t = 0; t < NR; ++t) v[t][q] = z[t];
  }
  F::template run<+1>(v, lane, sm, tw);
#pragma unroll
  for (int t = 0; t < NR; ++t)
#pragma unroll
    for (int q = 0; q < C::E; ++q) {
      const cpx<T> a = z1(t, q);
      p1[t][q] = (a.x * v[t][q].y - a.y * v[t][q].x) * inv_n4;
    }
  // pair (d_x vz, d_y vz) -> [psi, vz]
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    cpx<T> z[NR];
    packed_pair<T, N, NR>(tf + 4 * plane, tf + 5 * plane, lane + q * C::TPF, y0, M, z);
#pragma unroll
    for (int t = 0; t < NR; ++t) v[t][q] = z[t];
  }
  F::template run<+1>(v, lane, sm, tw);
#pragma unroll
  for (int t = 0; t < NR; ++t)
#pragma unroll
    for (int q = 0; q < C::E; ++q) {
      const cpx<T> a = z1(t, q);
      v[t][q] = mkc<T>(p1[t][q], (a.x * v[t][q].y - a.y * v[t][q].x) * inv_n4);
    }
  // forward x-FFT of both real products at once
  F::template run<-1>(v, lane, sm, tw);
  }
  F::to_smem(v, lane, sm);
  fft_sync<C::TPF>();
  const size_t oplane = (size_t)gd.nh * N;
  const T h = (T)0.5;
#pragma unroll
  for (int q = 0; q < C::E; ++q) {
    const int k = lane + q * C::TPF;
    if (ok && k < kxo) {
      cpx<T> o1[NR], o2[NR];
#pragma unroll
      for (int t = 0; t < NR; ++t) {
        const cpx<T> w = F::from_smem(t, k, sm);
        const cpx<T> u = F::from_smem(t, (N - k) & (N - 1), sm);
        o1[t] = mkc<T>((w.x + u.x) * h, (w.y - u.y) * h);
        o2[t] = mkc<T>((w.y + u.y) * h, (u.x - w.x) * h);
      }
      const size_t off = mix_idx<N, NR>(k, y0, gd.nh);
      store_rows<T, NR>(pb, off, o1);
      store_rows<T, NR>(pb + oplane, off, o2);
    }
  }
}

// --------------------------------------------------------------------------
// Pass B for small grids, the three inverse transforms of a row pair side by
// side: a CTA of three groups per row pair, group j transforming the packed
// pair (planes 2j, 2j+1), so the serial chain is one inverse and one forward
// transform instead of four transforms (small grids are bound by that chain,
// not by throughput).  The three results meet in shared memory; every group
// then forms the two brackets and runs the forward transform (the same
// values: keeping all groups in step keeps every barrier uniform), and
// group 0 stores.  Same arithmetic, in the same order, as k_passB:
// bit-identical (the launch autotuner chooses).
// --------------------------------------------------------------------------
template <typename T, int N>
struct SplitB {
  static constexpr int NR = PassNT<T, N>::value;
  using C = Cfg<T, N, NR>;
  using F = typename C::FFT;
  static constexpr int TPF = C::TPF;
  static constexpr int THREADS = 3 * TPF;
  static constexpr bool OK = THREADS <= 384;
  static constexpr size_t SMEM = 3 * F::SMEM_BYTES + (size_t)3 * NR * N * sizeof(cpx<T>);
};

template <typename T, int N, bool CFL>
__global__ void __launch_bounds__(SplitB<T, N>::THREADS)
k_passB_split(const cpx<T>* __restrict__ tf, cpx<T>* __restrict__ pb, int kxo, DevGrid gd, T inv_n4,
              const tw_t<T>* __restrict__ tw, unsigned long long* __restrict__ cfl_enc, Batch bs) {
  using SB = SplitB<T, N>;
  constexpr int NR = SB::NR, E = SB::C::E, TPF = SB::TPF;
  using F = typename SB::F;
  tf += blockIdx.y * bs.tf;
  pb += blockIdx.y * bs.pb;
  cfl_enc += blockIdx.y * kScalStride;
  extern __shared__ __align__(16) unsigned char smraw_[];
  const int j = threadIdx.x / TPF, lane = threadIdx.x % TPF;
  cpx<T>* sm = reinterpret_cast<cpx<T>*>(smraw_ + (size_t)j * F::SMEM_BYTES);
  cpx<T>* res = reinterpret_cast<cpx<T>*>(smraw_ + 3 * F::SMEM_BYTES);  // [pair j][row t][x]
  const int y0 = blockIdx.x * NR;
  const int M = gd.M;
  const size_t plane = (size_t)M * N;
  cpx<T> v[NR][E];
#pragma unroll
  for (int q = 0; q < E; ++q) {
    cpx<T> z[NR];
    packed_pair<T, N, NR>(tf + (size_t)(2 * j) * plane, tf + (size_t)(2 * j + 1) * plane, lane + q * TPF, y0, M,
                          z);
#pragma unroll
    for (int t = 0; t < NR; ++t) v[t][q] = z[t];
  }
  F::template run<+1>(v, lane, sm, tw);
  if constexpr (CFL) {  // CFL maximum of |grad psi|^2 from z1 (cfl_max_sq; every lane joins the shuffles)
    T m = (T)0;
    if (j == 0) {
#pragma unroll
      for (int t = 0; t < NR; ++t)
#pragma unroll
        for (int q = 0; q < E; ++q) m = max(m, v[t][q].x * v[t][q].x + v[t][q].y * v[t][q].y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(cfl_enc, enc_ordered((double)m));
  }
#pragma unroll
  for (int t = 0; t < NR; ++t)
#pragma unroll
    for (int q = 0; q < E; ++q) res[((size_t)j * NR + t) * N + lane + q * TPF] = v[t][q];
  __syncthreads();
  // [psi, -k^2 psi] and [psi, vz] from z1 (pair 0) with z2, z3 (pairs 1, 2)
#pragma unroll
  for (int t = 0; t < NR; ++t)
#pragma unroll
    for (int q = 0; q < E; ++q) {
      const int x = lane + q * TPF;
      const cpx<T> a = res[(size_t)t * N + x];
      const cpx<T> b = res[((size_t)NR + t) * N + x];
      const cpx<T> c = res[((size_t)2 * NR + t) * N + x];
      const T p1 = (a.x * b.y - a.y * b.x) * inv_n4;
      v[t][q] = mkc<T>(p1, (a.x * c.y - a.y * c.x) * inv_n4);
    }
  F::template run<-1>(v, lane, sm, tw);
  F::to_smem(v, lane, sm);
  fft_sync<TPF>();
  if (j != 0) return;  // (no barrier follows)
  const size_t oplane = (size_t)gd.nh * N;
  const T h = (T)0.5;
#pragma unroll
  for (int q = 0; q < E; ++q) {
    const int k = lane + q * TPF;
    if (k < kxo) {
      cpx<T> o1[NR], o2[NR];
#pragma unroll
      for (int t = 0; t < NR; ++t) {
        const cpx<T> w = F::from_smem(t, k, sm);
        const cpx<T> u = F::from_smem(t, (N - k) & (N - 1), sm);
        o1[t] = mkc<T>((w.x + u.x) * h, (w.y - u.y) * h);
        o2[t] = mkc<T>((w.y + u.y) * h, (u.x - w.x) * h);
      }
      const size_t off = mix_idx<N, NR>(k, y0, gd.nh);
      store_rows<T, NR>(pb, off, o1);
      store_rows<T, NR>(pb + oplane, off, o2);
    }
  }
}

// --------------------------------------------------------------------------
// Pass B, FP32 pair-tiled grids (n = 512 .. 4096), one row pair per CTA at a
// time: persistent CTAs that stage each row pair's mixed-plane inputs in
// shared memory with asynchronous copies (cp.async, 16 bytes per thread and
// instruction) one plane pair ahead of the transform that needs it, so that
// the global loads of pairs 2 and 3 and of the next row pair's pair 1 overlap
// the x-transforms instead of stalling them.  The four transforms of a row
// pair run through one rolled copy of the transform code.  Same arithmetic,
// in the same order, as k_passB: results are bit-identical (the launch
// autotuner chooses between the two).
//
// Shared memory: the transform buffers (2 x SMEM_ELEMS), the held z1
// (2 x N) and two staging buffers S0, S1 of one plane pair each (2 x M
// float4: the retained kx < M of rows y0, y0+1 of two planes).  Pipeline of
// one row pair (S0: pairs 1 and 3, S1: pair 2, then the first bracket p1):
//   wait pair 1 -> read it (S0) -> copy pair 3 into S0 -> x-IFFT z1
//   wait pair 2 -> read it (S1) -> x-IFFT z2 -> p1 into S1
//   wait pair 3 -> read it (S0) -> copy the next row pair's pair 1 into S0
//   -> x-IFFT z3 -> products -> x-FFT -> copy the next row pair's pair 2
//   into S1 -> Hermitian split -> stores
// cp.async.wait_group is a hardware wait on the thread's own copies (no spin
// loop); a barrier after it makes every thread's copies visible to all.
// --------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory");
}

// One plane pair of row pair rp into dst (plane a at [0, M), plane b at
// [M, 2M)) as one commit group; `on` false commits an empty group so that the
// group count stays the same on every path.
template <int THREADS>
__device__ __forceinline__ void stage_plane_pair(float4* dst, const float4* __restrict__ pa,
                                                 const float4* __restrict__ pb, int M, bool on) {
  if (on) {
    for (int i = threadIdx.x; i < 2 * M; i += THREADS) cp_async16(dst + i, i < M ? pa + i : pb + (i - M));
  }
  cp_async_commit();
}

// Launch shape of the pipelined pass B: G groups of TPF = N/E threads, each
// group carrying NT of the row pair's two rows (G * NT == 2).  Radix 8 with
// both rows in one group measured fastest at n = 4096 (radix 16 with one row
// per group: 5% slower).
template <int N>
struct PipeB {
  static constexpr int E = 8;
  static constexpr int NT = 2;
  static constexpr int G = 2 / NT;
  using F = BlockFFT<float, N, E, NT>;
  static constexpr int TPF = N / E;
  static constexpr int THREADS = G * TPF;
  // CTAs per SM the registers are sized for: 16 warps per SM at 128 registers
  // (shared memory allows exactly one CTA at n = 4096)
  static constexpr int MINB = 512 / THREADS;
  // dynamic shared memory for M retained columns: transform buffers, held z1,
  // two staging buffers
  static size_t smem(int M) {
    return (size_t)G * NT * F::SMEM_ELEMS * sizeof(float2) + (size_t)2 * N * sizeof(float2) +
           (size_t)4 * M * sizeof(float4);
  }
};

// pass B runs as k_passB_pipe where it applies
template <typename T, int N>
constexpr bool kPipeB = sizeof(T) == 4 && PassNT<T, N>::value == 2 && PipeB<N>::THREADS >= 64 &&
                        PipeB<N>::THREADS <= 512;

// Row t (0/1) of the staged pair at column kk: S holds float4 (row 0, row 1).
__device__ __forceinline__ float2 staged_row(const float4* S, int idx, int t) {
  return reinterpret_cast<const float2*>(S)[2 * idx + t];
}

template <int N, bool CFL>
__global__ void __launch_bounds__(PipeB<N>::THREADS, PipeB<N>::MINB)
k_passB_pipe(const float2* __restrict__ tf, float2* __restrict__ pb, int kxo, DevGrid gd, float inv_n4,
             const float4* __restrict__ tw, unsigned long long* __restrict__ cfl_enc, Batch bs) {
  using T = float;
  using PB = PipeB<N>;
  constexpr int NT = PB::NT, E = PB::E, TPF = PB::TPF, THREADS = PB::THREADS;
  using F = typename PB::F;
  constexpr int NRP = N / 2;  // row pairs
  tf += blockIdx.y * bs.tf;
  pb += blockIdx.y * bs.pb;
  cfl_enc += blockIdx.y * kScalStride;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / TPF, lane = threadIdx.x % TPF;
  const int r0 = g * NT;  // first row of the pair carried by this group
  cpx<T>* sm = smbase_ + (size_t)g * NT * F::SMEM_ELEMS;
  cpx<T>* hold = smbase_ + (size_t)PB::G * NT * F::SMEM_ELEMS + (size_t)r0 * N;
  const int M = gd.M;
  float4* S0 = reinterpret_cast<float4*>(smbase_ + (size_t)PB::G * NT * F::SMEM_ELEMS + (size_t)2 * N);
  float4* S1 = S0 + 2 * M;
  float* P1 = reinterpret_cast<float*>(S1) + (size_t)r0 * N;  // p1 (after pair 2 is read)
  // plane p, row pair rp: P + p * pl4 + rp * M (float4 = two rows of one column)
  const float4* P = reinterpret_cast<const float4*>(tf);
  const size_t pl4 = (size_t)M * NRP;
  const size_t oplane = (size_t)gd.nh * N;
  const T h = (T)0.5;
  // packed spectrum Z[k] of the staged pair for this group's rows
  auto load_z = [&](const float4* S, cpx<T> (&v)[NT][E]) {
#pragma unroll
    for (int q = 0; q < E; ++q) {
      const int k = lane + q * TPF;
      if (k < M || k > N - M) {
        const int kk = k < M ? k : N - k;
#pragma unroll
        for (int t = 0; t < NT; ++t) {
          const float2 a = staged_row(S, kk, r0 + t), b = staged_row(S, M + kk, r0 + t);
          if (k == 0) v[t][q] = make_float2(a.x, b.x);
          else if (k < M) v[t][q] = make_float2(a.x - b.y, a.y + b.x);
          else v[t][q] = make_float2(a.x + b.y, b.x - a.y);
        }
      } else {
#pragma unroll
        for (int t = 0; t < NT; ++t) v[t][q] = make_float2(0.f, 0.f);
      }
    }
  };
  int rp = blockIdx.x;
  if (rp >= NRP) return;  // uniform for the whole CTA
  stage_plane_pair<THREADS>(S0, P + (size_t)rp * M, P + pl4 + (size_t)rp * M, M, true);
  stage_plane_pair<THREADS>(S1, P + 2 * pl4 + (size_t)rp * M, P + 3 * pl4 + (size_t)rp * M, M, true);
  for (; rp < NRP; rp += gridDim.x) {
    const int y0 = 2 * rp;
    const int nx = rp + gridDim.x;
    const bool more = nx < NRP;
    cpx<T> v[NT][E];
    // The four transforms of the row pair run through one copy of the
    // transform code (a loop that is not unrolled): unrolled, the compiler
    // interleaves them and runs out of registers.  The forward transform is
    // the inverse one of the conjugate, conjugated (bit-identical).
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
      if (f < 3) {
        // pending copy groups: f = 0: pairs 1, 2; f = 1: pairs 2, 3; f = 2: pair 3
        if (f == 2) cp_async_wait<0>();
        else cp_async_wait<1>();
        __syncthreads();  // the staged pair is visible; the previous users of sm are done
        load_z(f == 1 ? S1 : S0, v);
        __syncthreads();  // every read of the staging buffer is done
        if (f == 0) {
          stage_plane_pair<THREADS>(S0, P + 4 * pl4 + (size_t)rp * M, P + 5 * pl4 + (size_t)rp * M, M, true);
        } else if (f == 2) {
          stage_plane_pair<THREADS>(S0, P + (size_t)nx * M, P + pl4 + (size_t)nx * M, M, more);
        }
      } else {
#pragma unroll
        for (int t = 0; t < NT; ++t)
#pragma unroll
          for (int q = 0; q < E; ++q) v[t][q].y = -v[t][q].y;
      }
      F::template run<+1>(v, lane, sm, tw);
      if (f == 0) {
        if constexpr (CFL) cfl_max_sq<T, NT, E>(v, cfl_enc);
        // each thread reads back only the positions it wrote: no barrier needed
#pragma unroll
        for (int t = 0; t < NT; ++t)
#pragma unroll
          for (int q = 0; q < E; ++q) hold[t * N + lane + q * TPF] = v[t][q];
      } else if (f == 1) {
#pragma unroll
        for (int t = 0; t < NT; ++t)
#pragma unroll
          for (int q = 0; q < E; ++q) {
            const cpx<T> a = hold[t * N + lane + q * TPF];
            P1[t * N + lane + q * TPF] = (a.x * v[t][q].y - a.y * v[t][q].x) * inv_n4;
          }
      } else if (f == 2) {
#pragma unroll
        for (int t = 0; t < NT; ++t)
#pragma unroll
          for (int q = 0; q < E; ++q) {
            const cpx<T> a = hold[t * N + lane + q * TPF];
            v[t][q] = mkc<T>(P1[t * N + lane + q * TPF], (a.x * v[t][q].y - a.y * v[t][q].x) * inv_n4);
          }
      } else {
#pragma unroll
        for (int t = 0; t < NT; ++t)
#pragma unroll
          for (int q = 0; q < E; ++q) v[t][q].y = -v[t][q].y;
      }
    }
    F::to_smem(v, lane, sm);
    __syncthreads();  // also ends every read of p1 in S1
    stage_plane_pair<THREADS>(S1, P + 2 * pl4 + (size_t)nx * M, P + 3 * pl4 + (size_t)nx * M, M, more);
#pragma unroll
    for (int q = 0; q < E; ++q) {
      const int k = lane + q * TPF;
      if (k < kxo) {
        cpx<T> o1[NT], o2[NT];
#pragma unroll
        for (int t = 0; t < NT; ++t) {
          const cpx<T> w = F::from_smem(t, k, sm);
          const cpx<T> u = F::from_smem(t, (N - k) & (N - 1), sm);
          o1[t] = mkc<T>((w.x + u.x) * h, (w.y - u.y) * h);
          o2[t] = mkc<T>((w.y + u.y) * h, (u.x - w.x) * h);
        }
        const size_t off = mix_idx<N, 2>(k, y0 + r0, gd.nh);
        if constexpr (NT == 2) {
          store_rows<T, 2>(pb, off, o1);
          store_rows<T, 2>(pb + oplane, off, o2);
        } else {
          pb[off] = o1[0];
          pb[oplane + off] = o2[0];
        }
      }
    }
  }
  cp_async_wait<0>();  // no copy outlives the CTA
}

// --------------------------------------------------------------------------
// pass C: forward y-FFT of both brackets + RK substep update
// (Rot2D3C.para.f90:578-599).  c1in/c2in may alias c1out/c2out, and in the
// last substep c1out/c2out are ps/vz themselves: every element is read and
// written by the same thread.
// --------------------------------------------------------------------------
// The inputs of one element's update, loaded ahead of the arithmetic so that
// a batch of elements can have all its loads in flight before its first
// store (the output planes may alias the inputs, which keeps the compiler
// from reordering loads and stores itself).
template <typename T>
struct RkIn {
  cpx<T> a1, a2, p0, f0, v0, g0;
};

template <typename T>
__device__ __forceinline__ void rk_load(RkIn<T>& r, size_t idx, const cpx<T>* c1in, const cpx<T>* c2in,
                                        const cpx<T>* ps, const cpx<T>* vz, const cpx<T>* __restrict__ fp,
                                        const cpx<T>* __restrict__ fz) {
  r.a1 = c1in[idx];
  r.a2 = c2in[idx];
  r.p0 = ps[idx];
  r.f0 = fp[idx];
  r.v0 = vz[idx];
  r.g0 = fz[idx];
}

// New C1 (rk_apply1) and C2 (rk_apply2) of one element
// (Rot2D3C.para.f90:580-599); zero outside the retained disc and at k = 0.
// Both components are divided by the same implicit divisor: one reciprocal
// and two products (within an ulp of the two quotients; an FP64 division
// is a long sequence on the FP64 pipe, which binds the FP64 path).
// The two are independent: C1 needs C2's input (the Coriolis term 2 Omega
// d_y C2) and [psi, -k^2 psi], C2 needs C1's input and [psi, vz].
template <typename T>
__device__ __forceinline__ cpx<T> rk_apply1(const RkIn<T>& r, const cpx<T> c5, int kyi, int k2, const StepCoef& sc,
                                            T tmp1) {
  const T nu = (T)sc.nu, hnu = (T)sc.hnu, w2 = (T)sc.w2;
  const T kyf = (T)kyi, ka2 = (T)k2;
  const cpx<T> C4 = mkc<T>(-kyf * r.a2.y, kyf * r.a2.x);  // derivk2(C2,C4,2)
  const T tmp2 = (T)1 / ka2;
  const T tmp3 = (T)1 + (nu * powi(ka2, sc.nn) + hnu * powi(tmp2, sc.mm)) * tmp1;
  const T u1x = r.p0.x + ((-c5.x + w2 * C4.x) * tmp2 + r.f0.x) * tmp1;
  const T u1y = r.p0.y + ((-c5.y + w2 * C4.y) * tmp2 + r.f0.y) * tmp1;
  const T r3 = (T)1 / tmp3;
  return mkc<T>(u1x * r3, u1y * r3);
}
template <typename T>
__device__ __forceinline__ cpx<T> rk_apply2(const RkIn<T>& r, const cpx<T> c6, int kyi, int k2, const StepCoef& sc,
                                            T tmp1) {
  const T nuv = (T)sc.nuv, hnuv = (T)sc.hnuv, w2 = (T)sc.w2;
  const T kyf = (T)kyi, ka2 = (T)k2;
  const cpx<T> C3 = mkc<T>(-kyf * r.a1.y, kyf * r.a1.x);  // derivk2(C1,C3,2)
  const T tmp2 = (T)1 / ka2;
  const T tmp3v = (T)1 + (nuv * powi(ka2, sc.nnv) + hnuv * powi(tmp2, sc.mmv)) * tmp1;
  const T u2x = r.v0.x + (c6.x + w2 * C3.x + r.g0.x) * tmp1;
  const T u2y = r.v0.y + (c6.y + w2 * C3.y + r.g0.y) * tmp1;
  const T r3v = (T)1 / tmp3v;
  return mkc<T>(u2x * r3v, u2y * r3v);
}
template <typename T>
__device__ __forceinline__ void rk_apply(const RkIn<T>& r, const cpx<T> c5, const cpx<T> c6, int kyi, int k2,
                                         const StepCoef& sc, T tmp1, cpx<T>& n1, cpx<T>& n2) {
  n1 = rk_apply1<T>(r, c5, kyi, k2, sc, tmp1);
  n2 = rk_apply2<T>(r, c6, kyi, k2, sc, tmp1);
}

// L2 prefetch (cp.async.bulk.prefetch, no completion to wait for) of the
// retained rows |ky| <= L of ncol adjacent spectral columns starting at p:
// rows [0, L] of the first column, then each run [N - L, N + L] across a
// column boundary, then rows [N - L, N) of the last column.
// The range is widened to 16-byte boundaries (the instruction's alignment
// rule); every caller's range lies inside columns that start and end on
// 16-byte boundaries, so the widened range stays inside the same allocation.
template <typename T>
__device__ __forceinline__ void prefetch_l2(const T* p, size_t count) {
  const unsigned long long a0 = reinterpret_cast<unsigned long long>(p) & ~15ull;
  const unsigned long long a1 = (reinterpret_cast<unsigned long long>(p + count) + 15ull) & ~15ull;
  if (a1 > a0)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a0), "r"((unsigned)(a1 - a0)) : "memory");
}
template <typename T>
__device__ __forceinline__ void prefetch_columns_l2(const cpx<T>* p, int ncol, int N, int L) {
  prefetch_l2(p, (size_t)L + 1);
  for (int c = 1; c < ncol; ++c) prefetch_l2(p + (size_t)c * N - L, (size_t)2 * L + 1);
  prefetch_l2(p + (size_t)ncol * N - L, (size_t)L);
}

// The RK update of pass C for FP32 with the held c5 (FP32 grids up to 4096):
// c6 (this thread's transform output v) joins c5 in shared memory (the
// transform buffer sm is free after the last transform), then the threads
// update the retained rows two at a time (rows 2p, 2p+1 of one column:
// 16-byte loads and stores), two row pairs per iteration with all loads of
// an iteration issued before its stores.  Each element is loaded and stored
// by one thread.  Every thread of the CTA calls it (one barrier inside).
template <typename T, int N, int NT, int E, int TPF>
__device__ __forceinline__ void passC_update_pairs(cpx<T>* sm, const cpx<T>* hold, const cpx<T> (&v)[NT][E],
                                                   int lane, int kx0, const cpx<T>* c1in, const cpx<T>* c2in,
                                                   const cpx<T>* ps, const cpx<T>* vz, const cpx<T>* __restrict__ fp,
                                                   const cpx<T>* __restrict__ fz, cpx<T>* c1out, cpx<T>* c2out,
                                                   const DevGrid& gd, const StepCoef& sc, T tmp1,
                                                   const cpx<T>* __restrict__ tau5,
                                                   const cpx<T>* __restrict__ tau6, int chunk = -1,
                                                   int uidx = -1, int ustride = TPF, bool owner = true) {
  // chunk -1: both outputs; 0: C1 only (v and hold hold the [psi,-k^2 psi]
  // columns); 1: C2 only (v holds the [psi, vz] columns).  The update runs
  // over ustride threads (thread uidx; default: the group's own TPF), of
  // which the owner group's results are in sm / hold.
  if (uidx < 0) uidx = lane;
  const bool do1 = chunk != 1, do2 = chunk != 0;
  cpx<T>* c6s = sm;
  if (do2 && owner) {
#pragma unroll
    for (int t = 0; t < NT; ++t)
#pragma unroll
      for (int q = 0; q < E; ++q) c6s[t * N + lane + q * TPF] = v[t][q];
  }
  __syncthreads();
  const int L = gd.L;
  const int lo_pairs = L / 2 + 1;       // pairs p = 0 .. L/2 hold rows 0 .. L
  const int hi_first = (N - L) / 2;     // pairs hi_first .. N/2-1 hold rows N-L .. N-1
  const int npc = lo_pairs + (N / 2 - hi_first);
  const int total = NT * npc;
  using F4 = float4;
  constexpr int RB = 2;
  auto ld4 = [](const cpx<T>* base, size_t idx) { return *reinterpret_cast<const F4*>(base + idx); };
#pragma unroll 1
  for (int e0 = uidx; e0 < total; e0 += RB * ustride) {
    F4 a1[RB], a2[RB], p0[RB], f0[RB], v0[RB], g0[RB];
    int col[RB], j0[RB];
    bool keep[RB][2], in[RB][2];
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int e = e0 + b * ustride;
      const int t = e / npc, pi = e % npc;
      const int pr = pi < lo_pairs ? pi : hi_first + (pi - lo_pairs);
      col[b] = kx0 + t;
      j0[b] = 2 * pr;
      bool any = false;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int ky = ky_of(j0[b] + h, N), k2 = col[b] * col[b] + ky * ky;
        keep[b][h] = e < total && col[b] < gd.M && ky <= L && -ky <= L;
        in[b][h] = keep[b][h] && k2 <= gd.kmaxi && k2 >= 1;
        any |= in[b][h];
      }
      if (any) {
        const size_t idx = (size_t)col[b] * N + j0[b];
        if (do2) a1[b] = ld4(c1in, idx);
        if (do1) a2[b] = ld4(c2in, idx);
        if (do1) p0[b] = ld4(ps, idx);
        if (do1) f0[b] = ld4(fp, idx);
        if (do2) v0[b] = ld4(vz, idx);
        if (do2) g0[b] = ld4(fz, idx);
      }
    }
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      if (!keep[b][0] && !keep[b][1]) continue;
      const int t = col[b] - kx0;
      const size_t idx = (size_t)col[b] * N + j0[b];
      // the two rows of the pair: h = 0 (x, y halves of the float4s), h = 1 (z, w)
      auto row = [&](int h, cpx<T>& n1, cpx<T>& n2) {
        n1 = czero<T>();
        n2 = czero<T>();
        if (!in[b][h]) return;
        const int ky = ky_of(j0[b] + h, N), k2 = col[b] * col[b] + ky * ky;
        RkIn<T> r;
        if (do1) {
          r.a2 = h ? mkc<T>(a2[b].z, a2[b].w) : mkc<T>(a2[b].x, a2[b].y);
          r.p0 = h ? mkc<T>(p0[b].z, p0[b].w) : mkc<T>(p0[b].x, p0[b].y);
          r.f0 = h ? mkc<T>(f0[b].z, f0[b].w) : mkc<T>(f0[b].x, f0[b].y);
          cpx<T> c5 = hold[t * N + j0[b] + h];
          if (tau5) {  // learned subgrid tendency of the first bracket
            const cpx<T> u = tau5[idx + h];
            c5 = mkc<T>(c5.x + u.x, c5.y + u.y);
          }
          n1 = rk_apply1<T>(r, c5, ky, k2, sc, tmp1);
        }
        if (do2) {
          r.a1 = h ? mkc<T>(a1[b].z, a1[b].w) : mkc<T>(a1[b].x, a1[b].y);
          r.v0 = h ? mkc<T>(v0[b].z, v0[b].w) : mkc<T>(v0[b].x, v0[b].y);
          r.g0 = h ? mkc<T>(g0[b].z, g0[b].w) : mkc<T>(g0[b].x, g0[b].y);
          cpx<T> c6 = c6s[t * N + j0[b] + h];
          if (tau5) {  // learned subgrid tendency of the second bracket
            const cpx<T> w = tau6[idx + h];
            c6 = mkc<T>(c6.x + w.x, c6.y + w.y);
          }
          n2 = rk_apply2<T>(r, c6, ky, k2, sc, tmp1);
        }
      };
      cpx<T> n10, n20, n11, n21;
      row(0, n10, n20);
      row(1, n11, n21);
      if (keep[b][0] && keep[b][1]) {
        if (do1) *reinterpret_cast<F4*>(c1out + idx) = make_float4(n10.x, n10.y, n11.x, n11.y);
        if (do2) *reinterpret_cast<F4*>(c2out + idx) = make_float4(n20.x, n20.y, n21.x, n21.y);
      } else if (keep[b][0]) {
        if (do1) c1out[idx] = n10;
        if (do2) c2out[idx] = n20;
      } else {
        if (do1) c1out[idx + 1] = n11;
        if (do2) c2out[idx + 1] = n21;
      }
    }
  }
}

// Pass C with ATAIL: the next substep's pass A on the same column pairs, in
// the same launch (FP32, n <= 512): the team that updated a column pair
// reads back the state it has just written (c1out: psi, c2out: vz) and
// derivative-transforms it into the mixed planes atf, each team group
// taking other fields, with the per-field arithmetic of k_passA (the same
// transform configuration and twiddle table `twa`), so the results are
// bit-identical to the separate pass A.
template <typename T, int N, bool ATAIL = false>
__global__ void __launch_bounds__(Cfg<T, N, PassNT<T, N>::value>::THREADS, 1)
k_passC(const cpx<T>* __restrict__ pb, const cpx<T>* c1in, const cpx<T>* c2in,
        const cpx<T>* ps, const cpx<T>* vz, const cpx<T>* __restrict__ fp,
        const cpx<T>* __restrict__ fz, cpx<T>* c1out, cpx<T>* c2out, DevGrid gd,
        const StepCoef* __restrict__ scs, const double* __restrict__ scal, int o,
        const tw_t<T>* __restrict__ tw, Batch bs, const cpx<T>* __restrict__ tau5,
        const cpx<T>* __restrict__ tau6, int wide = 1, cpx<T>* __restrict__ atf = nullptr,
        const tw_t<T>* __restrict__ twa = nullptr) {
  constexpr int NT = PassNT<T, N>::value;
  using PS = PassSmem<T, N>;
  constexpr bool HOLD = PS::HOLD;
  const size_t rs = blockIdx.y * bs.spec;
  pb += blockIdx.y * bs.pb;
  c1in += rs;
  c2in += rs;
  ps += rs;
  vz += rs;
  fp += rs;
  fz += rs;
  c1out += rs;
  c2out += rs;
  using C = Cfg<T, N, NT>;
  using F = typename C::FFT;
  R2D3C_SMEM_DECL
  const int g = threadIdx.x / C::TPF, lane0 = threadIdx.x % C::TPF;
  cpx<T>* sm = smbase_ + (size_t)g * PS::GROUP_ELEMS;
  cpx<T>* hold = sm + NT * F::SMEM_ELEMS;  // transformed [psi,-k^2 psi] columns (HOLD)
  // wide > 1 (FP32 grids with the held c5): a team of `wide` groups per
  // column pair; each group transforms (the same values), and the team
  // shares the RK update, which is the longer part of small grids' chain
  const int W = (HOLD && sizeof(T) == 4) ? wide : 1;
  const int team = g / W, member = g % W;
  const int kx0 = (blockIdx.x * ((blockDim.x / C::TPF) / W) + team) * NT;  // groups per CTA: a launch-time choice
  const size_t oplane = (size_t)gd.nh * N;
  // The RK update at the end reads six spectral planes (eight with the
  // closure tendencies) on this group's columns; they are prefetched into L2
  // now, while the transforms run, so that those reads do not wait for DRAM.
  if (lane0 < 8 && member == 0) {
    const int lane = lane0;
    const cpx<T>* src = lane == 0 ? c1in : lane == 1 ? c2in : lane == 2 ? ps : lane == 3 ? vz
                      : lane == 4 ? fp : lane == 5 ? fz : lane == 6 ? tau5 : tau6;
    // with two chunks each CTA needs half of them: z = 0 the C1 update's
    // (c2in, ps, fp, tau5), z = 1 the C2 update's (c1in, vz, fz, tau6)
    const int user = lane < 2 ? 1 - lane : (lane & 1);  // the chunk that reads src
    const bool need = gridDim.z == 1 || !(sizeof(T) == 4 && HOLD) || (int)blockIdx.z == user;
    const int ncol = min(NT, gd.M - kx0);
    if (src && need && ncol > 0) prefetch_columns_l2<T>(src + (size_t)kx0 * N, ncol, N, gd.L);
  }
  cpx<T> v[NT][C::E];
  cpx<T> c5r[HOLD ? 1 : NT][C::E];
  // gridDim.z = 2 splits a column pair's work over two CTAs (FP32 grids with
  // the held c5): z = 0 transforms [psi,-k^2 psi] and updates C1, z = 1
  // transforms [psi, vz] and updates C2; the arithmetic per element is the
  // same as with one CTA (the launch autotuner chooses)
  const int chunk = (HOLD && sizeof(T) == 4 && gridDim.z > 1) ? (int)blockIdx.z : -1;
#pragma unroll 1
  for (int pl = 0; pl < 2; ++pl) {
    if (chunk >= 0 && pl != chunk) continue;
    // the loop-invariant addresses of the transform are recomputed per
    // iteration from an opaque copy of the lane index instead of being
    // hoisted out of the loop and held in registers across it
    const int lane = opaque(lane0);
    const cpx<T>* src = pb + pl * oplane;
    if constexpr (NT == 2) {
      // lane pair (2p, 2p+1): the even lane loads column kx0's rows (2p, 2p+1),
      // the odd lane column kx0+1's; one swap gives each lane its own row of
      // both columns
      const bool odd = lane & 1;
      const int kx = kx0 + (odd ? 1 : 0);
#pragma unroll
      for (int q = 0; q < C::E; ++q) {
        const int y = (lane + q * C::TPF) & ~1;
        const float4 w = __ldg(reinterpret_cast<const float4*>(src + mix_idx<N, 2>(kx, y, gd.nh)));
        const float gx = odd ? w.x : w.z, gy = odd ? w.y : w.w;  // value the partner needs
        const float rx = __shfl_xor_sync(0xffffffffu, gx, 1);
        const float ry = __shfl_xor_sync(0xffffffffu, gy, 1);
        if (odd) {
          v[0][q] = mkc<T>(rx, ry);
          v[1][q] = mkc<T>(w.z, w.w);
        } else {
          v[0][q] = mkc<T>(w.x, w.y);
          v[1][q] = mkc<T>(rx, ry);
        }
      }
    } else {
      const cpx<T>* s5 = src + (size_t)(kx0 < gd.M ? kx0 : 0) * N;
#pragma unroll
      for (int q = 0; q < C::E; ++q) v[0][q] = s5[lane + q * C::TPF];
    }
    F::template run<-1>(v, lane, sm, tw);
    if (pl == 0) {
#pragma unroll
      for (int t = 0; t < NT; ++t)
#pragma unroll
        for (int q = 0; q < C::E; ++q) {
          if constexpr (HOLD) hold[t * N + lane + q * C::TPF] = v[t][q];
          else c5r[t][q] = v[t][q];
        }
    }
  }
  const int lane = lane0;
  // v holds the transformed [psi, vz] columns (c6).  The coefficients are
  // read only now, not held in registers across the transforms.
  const StepCoef sc = scs[blockIdx.y];
  const T tmp1 = (T)(scal[blockIdx.y * kScalStride] / (double)o);  // :581
  if constexpr (HOLD && sizeof(T) == 4) {
    cpx<T>* lsm = smbase_ + (size_t)(team * W) * PS::GROUP_ELEMS;  // the team's first group
    passC_update_pairs<T, N, NT, C::E, C::TPF>(lsm, lsm + NT * F::SMEM_ELEMS, v, lane, kx0, c1in, c2in, ps, vz, fp,
                                                fz, c1out, c2out, gd, sc, tmp1, tau5, tau6, chunk, member * C::TPF + lane,
                                                W * C::TPF, member == 0);
    if constexpr (ATAIL) {
      using CA = CfgA<T, N>;
      static_assert(NT == 2 && std::is_same<typename CA::FFT, F>::value && CA::TPF == C::TPF,
                    "pass A's transform configuration is pass C's");
      // the team's update stores (and its reads of the shared staging) are
      // done: the state written is visible to the whole CTA
      __syncthreads();
      // fields 0-3 from the new psi (C1), 4-5 from the new vz (C2); a CTA of
      // a chunked launch takes its own update's fields.  Every group runs the
      // same number of transforms (their barriers are CTA-wide above 32
      // threads per transform); a group without a field transforms zeros and
      // stores nothing.
      const int fb = chunk == 1 ? 4 : 0, fe = chunk == 0 ? 4 : 6;
      const int rounds = (fe - fb + W - 1) / W;
      const size_t plane = (size_t)gd.M * N;
      cpx<T>* tsm = smbase_ + (size_t)g * PS::GROUP_ELEMS;  // this group's transform buffers
#pragma unroll 1
      for (int r = 0; r < rounds; ++r) {
        const int f = fb + member + r * W;
        const bool act = f < fe;
        const cpx<T>* sp = f < 4 ? c1out : c2out;
        cpx<T> a[NT][C::E];
#pragma unroll
        for (int t = 0; t < NT; ++t) {
          const int col = kx0 + t;
#pragma unroll
          for (int q = 0; q < C::E; ++q) {
            const int ky = ky_of(lane + q * C::TPF, N);
            const bool in = act && col < gd.M && (ky <= gd.L && -ky <= gd.L) && col * col + ky * ky <= gd.kmaxi;
            cpx<T> x = in ? sp[(size_t)col * N + lane + q * C::TPF] : czero<T>();
            // (0,k)*(x,y) = (-k*y, k*x): derivk2 dir 1 (k = kx) / dir 2 (k = ky)
            const T k = (f & 1) ? (T)ky : (T)col;
            if (f == 2 || f == 3) {
              const T m = -(T)(col * col + ky * ky);  // laplak2: -ka2*a
              x = mkc<T>(m * x.x, m * x.y);
            }
            a[t][q] = mkc<T>(-k * x.y, k * x.x);
          }
        }
        F::template run<+1>(a, lane, tsm, twa);
        // lanes (2p, 2p+1) hold rows y = 2p, 2p+1 of columns kx0, kx0+1: one
        // swap, then each lane writes one column's row pair (16 bytes)
        const bool odd = lane & 1;
        const int kx = kx0 + (odd ? 1 : 0);
        cpx<T>* dst = atf + (size_t)(act ? f : 0) * plane;
#pragma unroll
        for (int q = 0; q < C::E; ++q) {
          const cpx<T> give = odd ? a[0][q] : a[1][q];
          cpx<T> got;
          got.x = __shfl_xor_sync(0xffffffffu, give.x, 1);
          got.y = __shfl_xor_sync(0xffffffffu, give.y, 1);
          const int y = (lane + q * C::TPF) & ~1;
          if (act && kx < gd.M) {
            const cpx<T> lo = odd ? got : a[0][q];
            const cpx<T> hi = odd ? a[1][q] : got;
            *reinterpret_cast<float4*>(dst + mix_idx<N, 2>(kx, y, gd.M)) = make_float4(lo.x, lo.y, hi.x, hi.y);
          }
        }
      }
    }
  } else if constexpr (HOLD) {
    // c6 joins c5 in shared memory (the transform buffer is free after the
    // last transform; each thread reads back only what it wrote), and the
    // update runs over this thread's elements in batches of RB: all loads of
    // a batch, then its arithmetic and stores.
    cpx<T>* c6s = sm;
#pragma unroll
    for (int t = 0; t < NT; ++t)
#pragma unroll
      for (int q = 0; q < C::E; ++q) c6s[t * N + lane + q * C::TPF] = v[t][q];
    constexpr int NE = NT * C::E, RB = 2;
    static_assert(NE % RB == 0, "whole batches");
#pragma unroll 1
    for (int e0 = 0; e0 < NE; e0 += RB) {
      RkIn<T> in[RB];
      cpx<T> ta[RB], tb[RB];
#pragma unroll
      for (int b = 0; b < RB; ++b) {
        const int t = (e0 + b) / C::E, q = (e0 + b) % C::E;
        const int col = kx0 + t, j = lane + q * C::TPF, ky = ky_of(j, N), k2 = col * col + ky * ky;
        if (col < gd.M && k2 <= gd.kmaxi && k2 >= 1) {
          const size_t idx = (size_t)col * N + j;
          rk_load<T>(in[b], idx, c1in, c2in, ps, vz, fp, fz);
          if (tau5) {
            ta[b] = tau5[idx];
            tb[b] = tau6[idx];
          }
        }
      }
#pragma unroll
      for (int b = 0; b < RB; ++b) {
        const int t = (e0 + b) / C::E, q = (e0 + b) % C::E;
        const int col = kx0 + t, j = lane + q * C::TPF, ky = ky_of(j, N), k2 = col * col + ky * ky;
        if (col >= gd.M || ky > gd.L || -ky > gd.L) continue;
        cpx<T> n1 = czero<T>(), n2 = czero<T>();
        if (k2 <= gd.kmaxi && k2 >= 1) {  // ka2 <= kmax .and. ka2 > tiny (:580)
          cpx<T> c5 = hold[t * N + j], c6 = c6s[t * N + j];
          if (tau5) {  // learned subgrid tendencies of the two brackets
            c5 = mkc<T>(c5.x + ta[b].x, c5.y + ta[b].y);
            c6 = mkc<T>(c6.x + tb[b].x, c6.y + tb[b].y);
          }
          rk_apply<T>(in[b], c5, c6, ky, k2, sc, tmp1, n1, n2);
        }
        const size_t idx = (size_t)col * N + j;
        c1out[idx] = n1;
        c2out[idx] = n2;
      }
    }
  } else {
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const int col = kx0 + t;
      if (col >= gd.M) continue;
#pragma unroll
      for (int q = 0; q < C::E; ++q) {
        const int j = lane + q * C::TPF;
        const int ky = ky_of(j, N);
        if (ky > gd.L || -ky > gd.L) continue;
        const int k2 = col * col + ky * ky;
        cpx<T> n1 = czero<T>(), n2 = czero<T>();
        const size_t idx = (size_t)col * N + j;
        if (k2 <= gd.kmaxi && k2 >= 1) {
          cpx<T> c5 = c5r[t][q], c6 = v[t][q];
          if (tau5) {
            const cpx<T> a = tau5[idx], b = tau6[idx];
            c5 = mkc<T>(c5.x + a.x, c5.y + a.y);
            c6 = mkc<T>(c6.x + b.x, c6.y + b.y);
          }
          RkIn<T> in;
          rk_load<T>(in, idx, c1in, c2in, ps, vz, fp, fz);
          rk_apply<T>(in, c5, c6, ky, k2, sc, tmp1, n1, n2);
        }
        c1out[idx] = n1;
        c2out[idx] = n2;
      }
    }
  }
}

// --------------------------------------------------------------------------
// Pass C, FP32 pair-tiled grids (n = 512 .. 4096): persistent CTAs, one
// column pair at a time.  Each bracket plane's two columns are staged in
// shared memory by cp.async (32 contiguous bytes per row pair: rows 2p, 2p+1
// of both columns) while the previous transform runs: plane 1 during plane
// 0's transform, the next column pair's plane 0 during plane 1's transform
// and the RK update.  The RK inputs of the column pair are prefetched into
// L2 when its turn starts.  Same arithmetic as k_passC (bit-identical; the
// launch autotuner chooses between the two).
// --------------------------------------------------------------------------
template <int N>
struct PipeC {
  using C = Cfg<float, N, 2>;
  using F = typename C::FFT;
  static constexpr int TPF = C::TPF, THREADS = TPF;
  static constexpr int MINB = 512 / THREADS;  // 16 warps per SM at 128 registers
  // transform buffers, held c5 (2 columns), one staged plane (2 columns)
  static constexpr size_t SMEM = (size_t)2 * F::SMEM_ELEMS * sizeof(float2) + (size_t)4 * N * sizeof(float2);
};
// pass C may split a column pair's C1 and C2 updates over two CTAs (gridDim.z
// = 2) where it holds c5 in shared memory and updates row pairs (FP32)
template <typename T, int N>
constexpr bool kChunkC = sizeof(T) == 4 && PassSmem<T, N>::HOLD;
// pass C carries the next substep's pass A (k_passC<T, N, true>): FP32 grids
// whose pass A and pass C share one transform configuration
template <typename T, int N>
constexpr bool kFuseCA = sizeof(T) == 4 && N <= 512 && PassNT<T, N>::value == 2 && PassSmem<T, N>::HOLD &&
                         !kAltRadixA<T, N> && PassAE<T, N>::value == Cfg<T, N>::E;
template <typename T, int N>
constexpr bool kPipeC = sizeof(T) == 4 && PassNT<T, N>::value == 2 && PassSmem<T, N>::HOLD &&
                        PipeC<N>::THREADS >= 64 && PipeC<N>::THREADS <= 512;

template <int N>
__global__ void __launch_bounds__(PipeC<N>::THREADS, PipeC<N>::MINB)
k_passC_pipe(const float2* __restrict__ pb, const float2* c1in, const float2* c2in, const float2* ps,
             const float2* vz, const float2* __restrict__ fp, const float2* __restrict__ fz, float2* c1out,
             float2* c2out, DevGrid gd, const StepCoef* __restrict__ scs, const double* __restrict__ scal, int o,
             const float4* __restrict__ tw, Batch bs, const float2* __restrict__ tau5,
             const float2* __restrict__ tau6) {
  using T = float;
  constexpr int NT = 2;
  using PC = PipeC<N>;
  using F = typename PC::F;
  constexpr int TPF = PC::TPF, E = PC::C::E;
  const size_t rs = blockIdx.y * bs.spec;
  pb += blockIdx.y * bs.pb;
  c1in += rs;
  c2in += rs;
  ps += rs;
  vz += rs;
  fp += rs;
  fz += rs;
  c1out += rs;
  c2out += rs;
  R2D3C_SMEM_DECL
  const int lane0 = threadIdx.x;
  cpx<T>* sm = smbase_;
  cpx<T>* hold = sm + NT * F::SMEM_ELEMS;
  float4* S4 = reinterpret_cast<float4*>(hold + NT * N);  // [row pair][column] = rows 2p, 2p+1
  const size_t oplane = (size_t)gd.nh * N;
  const int npairs = (gd.M + 1) / 2;
  // plane pl of column pair cp into S4 (one commit group; empty when !on)
  auto stage = [&](int pl, int cp, bool on) {
    if (on) {
      const float4* src = reinterpret_cast<const float4*>(pb + pl * oplane) + 2 * cp;  // ((p*nh + kx0)*2) / 2
      for (int i = threadIdx.x; i < N; i += TPF) {
        const int p = i >> 1, h = i & 1;
        cp_async16(S4 + i, src + (size_t)p * gd.nh + h);
      }
    }
    cp_async_commit();
  };
  int cp = blockIdx.x;
  if (cp >= npairs) return;  // uniform for the whole CTA
  stage(0, cp, true);
  for (; cp < npairs; cp += gridDim.x) {
    const int kx0 = 2 * cp;
    const int nx = cp + gridDim.x;
    if (lane0 < 8) {  // the RK update's inputs into L2 while the transforms run
      const int lane = lane0;
      const cpx<T>* src = lane == 0 ? c1in : lane == 1 ? c2in : lane == 2 ? ps : lane == 3 ? vz
                        : lane == 4 ? fp : lane == 5 ? fz : lane == 6 ? tau5 : tau6;
      const int ncol = min(NT, gd.M - kx0);
      if (src && ncol > 0) prefetch_columns_l2<T>(src + (size_t)kx0 * N, ncol, N, gd.L);
    }
    cpx<T> v[NT][E];
#pragma unroll 1
    for (int pl = 0; pl < 2; ++pl) {
      // addresses derived from an opaque lane index: not hoisted out of the
      // loop into registers held across it
      const int lane = opaque(lane0);
      cp_async_wait<0>();
      __syncthreads();  // plane pl staged; previous users of sm and hold done
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int y = lane + q * TPF;
#pragma unroll
        for (int t = 0; t < NT; ++t) {
          const float4 w = S4[(y >> 1) * 2 + t];
          v[t][q] = (y & 1) ? mkc<T>(w.z, w.w) : mkc<T>(w.x, w.y);
        }
      }
      __syncthreads();  // every read of S4 done
      if (pl == 0) stage(1, cp, true);
      else stage(0, nx, nx < npairs);
      F::template run<-1>(v, lane, sm, tw);
      if (pl == 0) {
#pragma unroll
        for (int t = 0; t < NT; ++t)
#pragma unroll
          for (int q = 0; q < E; ++q) hold[t * N + lane + q * TPF] = v[t][q];
      }
    }
    const StepCoef sc = scs[blockIdx.y];
    const T tmp1 = (T)(scal[blockIdx.y * kScalStride] / (double)o);  // :581
    passC_update_pairs<T, N, NT, E, TPF>(sm, hold, v, lane0, kx0, c1in, c2in, ps, vz, fp, fz, c1out, c2out, gd,
                                         sc, tmp1, tau5, tau6);
  }
  cp_async_wait<0>();  // no copy outlives the CTA
}

}  // namespace r2d3c

// Shared-memory / register block FFT for sm_103a.
//
// One length-N complex transform is carried by TPF = N/E threads.  Thread
// `lane` holds v[q] = x[lane + q*TPF] (q < E) on entry and X[lane + q*TPF] on
// exit, for every N and radix schedule: the same thread always owns the same
// positions, which is what lets the bracket kernels form products of several
// transforms in registers without another exchange.
//
// The schedule is a Stockham auto-sort: radix-E stages (the last one may have
// a smaller radix), each an in-register DFT of R points followed by one padded
// shared-memory exchange.  NT transforms can be carried at once by the same
// threads; they share the twiddle loads and the barriers.  Twiddles come from a per-N table
// tw[k] = exp(-2*pi*i*k/N) built on the host in FP64; the FP32 path stores
// every twiddle as an (hi, lo) float pair and applies the low part with an
// extra FMA ("compensated twiddles"), which removes the twiddle rounding from
// the FP32 error budget.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace r2d3c {

template <typename T> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };
template <typename T> using cpx = typename V2<T>::t;

// Twiddle storage: FP64 -> (re, im); FP32 -> (re_hi, im_hi, re_lo, im_lo).
template <typename T> struct TwS;
template <> struct TwS<double> { using t = double2; };
template <> struct TwS<float> { using t = float4; };
template <typename T> using tw_t = typename TwS<T>::t;

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }

template <typename T>
__device__ __forceinline__ cpx<T> mkc(T x, T y) {
  cpx<T> r;
  r.x = x;
  r.y = y;
  return r;
}

// a * w with w from the table; DIR = -1 uses w, DIR = +1 uses conj(w).
template <int DIR>
__device__ __forceinline__ double2 twmul(double2 a, double2 w) {
  const double wy = DIR < 0 ? w.y : -w.y;
  return make_double2(fma(a.x, w.x, -a.y * wy), fma(a.x, wy, a.y * w.x));
}
template <int DIR>
__device__ __forceinline__ float2 twmul(float2 a, float4 w) {
  const float wy = DIR < 0 ? w.y : -w.y;
  const float ly = DIR < 0 ? w.w : -w.w;
  const float tr = fmaf(a.x, w.z, -a.y * ly);
  const float ti = fmaf(a.x, ly, a.y * w.z);
  return make_float2(fmaf(a.x, w.x, fmaf(-a.y, wy, tr)),
                     fmaf(a.x, wy, fmaf(a.y, w.x, ti)));
}

// Constant twiddle exp(DIR*2*pi*i*I16/16), I16 in [0,8).  The constants are
// cos/sin of multiples of pi/8; the FP32 variant carries a low-order part.
template <typename T, int I16, int DIR>
__device__ __forceinline__ cpx<T> kmul(cpx<T> a) {
  constexpr double C1 = 0.92387953251128675613;  // cos(pi/8)
  constexpr double S1 = 0.38268343236508977173;  // sin(pi/8)
  constexpr double R2 = 0.70710678118654752440;  // 1/sqrt(2)
  if constexpr (I16 == 0) {
    return a;
  } else if constexpr (I16 == 4) {  // DIR * i
    if constexpr (DIR > 0) return mkc<T>(-a.y, a.x);
    else return mkc<T>(a.y, -a.x);
  } else if constexpr (I16 == 2) {  // (1 + DIR i)/sqrt2
    constexpr T s = (T)R2;
    if constexpr (DIR > 0) return mkc<T>((a.x - a.y) * s, (a.y + a.x) * s);
    else return mkc<T>((a.x + a.y) * s, (a.y - a.x) * s);
  } else if constexpr (I16 == 6) {  // (-1 + DIR i)/sqrt2
    constexpr T s = (T)R2;
    if constexpr (DIR > 0) return mkc<T>((-a.x - a.y) * s, (a.x - a.y) * s);
    else return mkc<T>((a.y - a.x) * s, (-a.x - a.y) * s);
  } else {
    constexpr double c = (I16 == 1) ? C1 : (I16 == 3) ? S1 : (I16 == 5) ? -S1 : -C1;
    constexpr double s = (I16 == 1) ? S1 : (I16 == 3) ? C1 : (I16 == 5) ? C1 : S1;
    constexpr double sd = DIR * s;
    if constexpr (sizeof(T) == 8) {
      return mkc<T>(fma(a.x, c, -a.y * sd), fma(a.x, sd, a.y * c));
    } else {
      constexpr float ch = (float)c, cl = (float)(c - (double)(float)c);
      constexpr float sh = (float)sd, sl = (float)(sd - (double)(float)sd);
      const float tr = fmaf(a.x, cl, -a.y * sl);
      const float ti = fmaf(a.x, sl, a.y * cl);
      return mkc<T>(fmaf(a.x, ch, fmaf(-a.y, sh, tr)), fmaf(a.x, sh, fmaf(a.y, ch, ti)));
    }
  }
}

// In-register DFT of R points: X[k] = sum_r u[r] exp(DIR*2*pi*i*r*k/R),
// recursive radix-2 decimation in time, unrolled at compile time.
template <typename T, int R, int DIR> struct RegDFT {
  template <int K>
  static __device__ __forceinline__ void bfly(cpx<T>* u, const cpx<T>* e, const cpx<T>* o) {
    if constexpr (K < R / 2) {
      const cpx<T> t = kmul<T, (K * 16) / R, DIR>(o[K]);
      u[K] = mkc<T>(e[K].x + t.x, e[K].y + t.y);
      u[K + R / 2] = mkc<T>(e[K].x - t.x, e[K].y - t.y);
      bfly<K + 1>(u, e, o);
    }
  }
  static __device__ __forceinline__ void run(cpx<T>* u) {
    cpx<T> e[R / 2], o[R / 2];
#pragma unroll
    for (int i = 0; i < R / 2; ++i) {
      e[i] = u[2 * i];
      o[i] = u[2 * i + 1];
    }
    RegDFT<T, R / 2, DIR>::run(e);
    RegDFT<T, R / 2, DIR>::run(o);
    bfly<0>(u, e, o);
  }
};
template <typename T, int DIR> struct RegDFT<T, 1, DIR> {
  static __device__ __forceinline__ void run(cpx<T>*) {}
};
template <typename T, int DIR> struct RegDFT<T, 2, DIR> {
  static __device__ __forceinline__ void run(cpx<T>* u) {
    const cpx<T> a = u[0], b = u[1];
    u[0] = mkc<T>(a.x + b.x, a.y + b.y);
    u[1] = mkc<T>(a.x - b.x, a.y - b.y);
  }
};

template <int TPF>
__device__ __forceinline__ void fft_sync() {
  if constexpr (TPF <= 32) {
    __syncwarp();
  } else {
    __syncthreads();
  }
}

// NT independent length-N transforms carried by the same TPF = N/E threads
// (thread `lane` holds v[t][q] = x_t[lane + q*TPF]).  The NT transforms share
// every twiddle load and every barrier.  Shared memory: NT interleaved
// complex buffers of SMEM_ELEMS elements, padded by one element every
// 128 bytes so that the strided Stockham writes stay (nearly) bank-conflict
// free.
//
// Two FP32 transforms (NT = 2) are interleaved in shared memory instead
// (unless ILV_OK is false): one float4 per position holds both transforms'
// values, so every exchange moves 16 bytes per instruction (half the
// shared-memory instructions), padded by one float4 every 128 bytes.
template <typename T, int N, int E, int NT = 1, bool ILV_OK = true>
struct BlockFFT {
  static_assert((N & (N - 1)) == 0 && N >= E && E >= 2, "N, E powers of two");
  static constexpr int TPF = N / E;
  static constexpr int LOGN = ilog2(N);
  static constexpr int LOGE = ilog2(E);
  static constexpr int NST = (LOGN + LOGE - 1) / LOGE;
  static constexpr int LAST_R = 1 << (LOGN - LOGE * (NST - 1));
  static constexpr bool ILV = ILV_OK && sizeof(T) == 4 && NT == 2;  // interleaved float4 exchange
  static constexpr int PADSH = ilog2(128 / (int)(ILV ? 16 : sizeof(cpx<T>)));
  static constexpr int SMEM_ELEMS = N + (N >> PADSH);  // per transform (complex elements)
  static constexpr size_t SMEM_BYTES = (size_t)NT * SMEM_ELEMS * sizeof(cpx<T>);

  static __device__ __forceinline__ int pad(int i) { return i + (i >> PADSH); }
  // both transforms' values at (padded) position idx of the interleaved layout
  static __device__ __forceinline__ void st2(cpx<T>* sm, int idx, const cpx<T>& a, const cpx<T>& b) {
    reinterpret_cast<float4*>(sm)[idx] = make_float4(a.x, a.y, b.x, b.y);
  }
  static __device__ __forceinline__ void ld2(const cpx<T>* sm, int idx, cpx<T>& a, cpx<T>& b) {
    const float4 w = reinterpret_cast<const float4*>(sm)[idx];
    a = mkc<T>(w.x, w.y);
    b = mkc<T>(w.z, w.w);
  }

  // Radix of stage s, sub-transform size NS before stage s, and the offset of
  // stage s's block in the stage-major twiddle table.  Block s holds the
  // twiddles exp(-2 pi i r jm / (NS R)), r = 1..R-1, jm < NS(s), r-major:
  // entry (r-1)*NS + jm, so that the threads of a warp (consecutive jm) read
  // one contiguous run for each r.
  static __host__ __device__ constexpr int radix(int s) { return s == NST - 1 ? LAST_R : E; }
  static __host__ __device__ constexpr int ns_of(int s) {
    int ns = 1;
    for (int i = 0; i < s; ++i) ns *= radix(i);
    return ns;
  }
  static __host__ __device__ constexpr int tw_off(int s) {
    int off = 0;
    for (int i = 1; i < s; ++i) off += ns_of(i) * (radix(i) - 1);
    return off;
  }
  static constexpr int TW_ELEMS = tw_off(NST) > 0 ? tw_off(NST) : 1;

  template <int DIR, int S, int NS>
  static __device__ __forceinline__ void stage(cpx<T> (&v)[NT][E], int lane, cpx<T>* sm,
                                               const tw_t<T>* __restrict__ tw) {
    constexpr int R = (S == NST - 1) ? LAST_R : E;
    constexpr int B = E / R;
    constexpr int LOGNS = ilog2(NS);
#pragma unroll
    for (int m = 0; m < B; ++m) {
      const int j = lane + m * TPF;
      const int jm = j & (NS - 1);
      if constexpr (NS > 1) {
        const tw_t<T>* tb = tw + tw_off(S) + jm;
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const tw_t<T> w = __ldg(&tb[(r - 1) * NS]);
#pragma unroll
          for (int t = 0; t < NT; ++t) v[t][m + r * B] = twmul<DIR>(v[t][m + r * B], w);
        }
      }
#pragma unroll
      for (int t = 0; t < NT; ++t) {
        cpx<T> u[R];
#pragma unroll
        for (int r = 0; r < R; ++r) u[r] = v[t][m + r * B];
        RegDFT<T, R, DIR>::run(u);
#pragma unroll
        for (int r = 0; r < R; ++r) v[t][m + r * B] = u[r];
      }
    }
    if constexpr (S < NST - 1) {
#pragma unroll
      for (int m = 0; m < B; ++m) {
        const int j = lane + m * TPF;
        const int base = ((j >> LOGNS) << (LOGNS + ilog2(R))) + (j & (NS - 1));
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int idx = pad(base + r * NS);
          if constexpr (ILV) {
            st2(sm, idx, v[0][m + r * B], v[NT - 1][m + r * B]);
          } else {
#pragma unroll
            for (int t = 0; t < NT; ++t) sm[t * SMEM_ELEMS + idx] = v[t][m + r * B];
          }
        }
      }
      fft_sync<TPF>();
#pragma unroll
      for (int q = 0; q < E; ++q) {
        const int idx = pad(lane + q * TPF);
        if constexpr (ILV) {
          ld2(sm, idx, v[0][q], v[NT - 1][q]);
        } else {
#pragma unroll
          for (int t = 0; t < NT; ++t) v[t][q] = sm[t * SMEM_ELEMS + idx];
        }
      }
      fft_sync<TPF>();
      stage<DIR, S + 1, NS * R>(v, lane, sm, tw);
    }
  }

  // X_t[k] = sum_x x_t[x] exp(DIR*2*pi*i*x*k/N), unnormalised, t < NT.
  template <int DIR>
  static __device__ __forceinline__ void run(cpx<T> (&v)[NT][E], int lane, cpx<T>* sm,
                                             const tw_t<T>* __restrict__ tw) {
    stage<DIR, 0, 1>(v, lane, sm, tw);
  }

  // Natural-order result to shared memory so that any thread of the group can
  // read X[k] and X[N-k] (Hermitian split of packed pairs).
  static __device__ __forceinline__ void to_smem(const cpx<T> (&v)[NT][E], int lane, cpx<T>* sm) {
#pragma unroll
    for (int q = 0; q < E; ++q) {
      const int idx = pad(lane + q * TPF);
      if constexpr (ILV) {
        st2(sm, idx, v[0][q], v[NT - 1][q]);
      } else {
#pragma unroll
        for (int t = 0; t < NT; ++t) sm[t * SMEM_ELEMS + idx] = v[t][q];
      }
    }
  }
  static __device__ __forceinline__ cpx<T> from_smem(int t, int k, const cpx<T>* sm) {
    if constexpr (ILV) {
      const float4 w = reinterpret_cast<const float4*>(sm)[pad(k)];
      return t ? mkc<T>(w.z, w.w) : mkc<T>(w.x, w.y);
    } else {
      return sm[t * SMEM_ELEMS + pad(k)];
    }
  }
};

// Host: the N-th roots of unity c[k] + i s[k] = exp(2 pi i k/N) in FP64 from
// libm on the first octant and exact symmetries elsewhere.
inline void host_unit_roots(int n, double* c, double* s) {
  const double twopi = 2.0 * 3.1415926535897932384;
  for (int k = 0; k <= n / 8; ++k) {
    const double a = twopi * (double)k / (double)n;
    c[k] = std::cos(a);
    s[k] = std::sin(a);
  }
  for (int k = n / 8 + 1; k <= n / 4; ++k) {
    c[k] = s[n / 4 - k];
    s[k] = c[n / 4 - k];
  }
  for (int k = n / 4 + 1; k <= n / 2; ++k) {
    c[k] = -c[n / 2 - k];
    s[k] = s[n / 2 - k];
  }
  for (int k = n / 2 + 1; k < n; ++k) {
    c[k] = c[n - k];
    s[k] = -s[n - k];
  }
}

inline void fill_tw(double2& w, double re, double im) {
  w.x = re;
  w.y = im;
}
inline void fill_tw(float4& w, double re, double im) {
  w.x = (float)re;
  w.y = (float)im;
  w.z = (float)(re - (double)w.x);
  w.w = (float)(im - (double)w.y);
}

// Host: the stage-major twiddle table of BlockFFT<T, N, E> (forward roots;
// the inverse uses their conjugates).
template <typename T, int N, int E>
void build_stage_twiddles(tw_t<T>* out, const double* c, const double* s) {
  using F = BlockFFT<T, N, E, 1>;
  for (int st = 1; st < F::NST; ++st) {
    const int ns = F::ns_of(st), r = F::radix(st), stride = N / (ns * r);
    for (int jm = 0; jm < ns; ++jm)
      for (int q = 1; q < r; ++q) {
        const int k = q * jm * stride;
        fill_tw(out[F::tw_off(st) + (q - 1) * ns + jm], c[k], -s[k]);
      }
  }
}

}  // namespace r2d3c

// Learned subgrid closure: a small periodic CNN (6 layers of 3x3 convolution,
// 8 -> 32 -> 32 -> 32 -> 32 -> 32 -> 2 channels, GELU between layers) with
// BF16 operands and FP32 accumulation on the tensor cores, trained with Adam
// by the kernels of this file.  No counterpart in the reference.
//
// Activations are NHWC (channels fastest) on an H x W periodic grid, batch B.
// Every convolution is an implicit GEMM: out[p][co] = sum_{tap, ci}
// in[p + offset(tap)][ci] * w[tap*CIN + ci][co], tap = (dy, dx) in 3x3,
// computed by warp-level mma.sync m16n8k16 (bf16 x bf16 -> f32) from a
// shared-memory halo tile of the input and the weights.  Backward data is the
// same convolution of dY with the tap-flipped, channel-transposed weights;
// backward weights is the GEMM dW[k][co] = sum_p in_col[p][k] dY[p][co],
// split over persistent CTAs with a fixed-order reduction of the partials.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../include/r2d3c.h"
#include "r2d3c_engine.h"

namespace r2d3c {
std::string& last_error_slot();
}

namespace {

using namespace r2d3c;
using bf16 = __nv_bfloat16;

constexpr int kLayers = 6;
constexpr int kCinPad[kLayers] = {16, 32, 32, 32, 32, 32};   // input channels (layer 0 padded 8 -> 16)
constexpr int kCoutPad[kLayers] = {32, 32, 32, 32, 32, 16};  // output channels (last padded 2 -> 16)
constexpr int kCin[kLayers] = {8, 32, 32, 32, 32, 32};
constexpr int kCout[kLayers] = {32, 32, 32, 32, 32, 2};

// tile of the implicit GEMM: 8 rows x 16 columns of pixels, 8 warps, one
// 16-pixel row per warp
constexpr int TH = 8, TW = 16, kThreads = 256;

__device__ __forceinline__ unsigned pack_bf16(bf16 lo, bf16 hi) {
  return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// ---------------------------------------------------------------------------
// Shared-memory tiles hold rows of C bf16 values (a pixel's channels, or a
// weight row's output channels) as C/8 chunks of 16 bytes; chunk c of row r
// is stored at chunk position c ^ swz(r) so that the 8 rows an ldmatrix
// reads (8 consecutive pixels, or 8 consecutive weight rows) fall in 8
// different bank groups.
// ---------------------------------------------------------------------------
template <int C>
__device__ __forceinline__ int swz(int r) {
  constexpr int C8 = C / 8;
  static_assert(C8 == 2 || C8 == 4, "16 or 32 channels");
  return (r / (8 / C8)) % C8;
}
template <int C>
__device__ __forceinline__ int tile_off(int r, int chunk) {  // bf16 offset of (row, chunk)
  return r * C + ((chunk ^ swz<C>(r)) << 3);
}

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}
__device__ __forceinline__ void ldsm_x2_t(unsigned (&r)[2], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(a));
}

// Halo tile (TH+2) x (TW+2) pixels of CIN channels around tile (b, ty0, tx0),
// periodic wrap, into the swizzled layout.
template <int CIN>
__device__ __forceinline__ void stage_halo(bf16* s_in, const bf16* __restrict__ in, int b, int ty0, int tx0, int H,
                                           int W) {
  constexpr int VPP = CIN / 8;
  for (int i = threadIdx.x; i < (TH + 2) * (TW + 2) * VPP; i += kThreads) {
    const int v = i % VPP, q = i / VPP, px = q % (TW + 2), py = q / (TW + 2);
    const int gy = (ty0 + py - 1 + H) % H, gx = (tx0 + px - 1 + W) % W;
    *reinterpret_cast<uint4*>(s_in + tile_off<CIN>(q, v)) =
        reinterpret_cast<const uint4*>(in + (((size_t)b * H + gy) * W + gx) * CIN)[v];
  }
}

// ---------------------------------------------------------------------------
// out[p][co] = sum_k in_col[p][k] w[k][co] (+ bias), periodic 3x3 stencil.
// in: [B][H][W][CIN] bf16; w: [9*CIN][COUT] bf16; y: [B][H][W][cout_store] f32
// (pre-activation, may be null); a: [B][H][W][COUT] bf16 = act(y) (may be
// null); act: 0 identity, 1 GELU.  Requires H % TH == 0, W % TW == 0.
// Persistent CTAs: the weights are staged once, then the CTA loops over
// 8 x 16 pixel tiles; warp w computes tile row w (16 pixels x COUT).
// Fragments come from ldmatrix: A (pixels x k) directly, B (k x co) through
// the transposing form.
// ---------------------------------------------------------------------------
template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads)
k_conv(const bf16* __restrict__ in, const bf16* __restrict__ w, const float* __restrict__ bias, int H, int W,
       int ntiles, float* __restrict__ y, bf16* __restrict__ a, int act, int cout_store) {
  constexpr int NTN = COUT / 8;  // n-tiles
  static_assert(NTN % 2 == 0, "n-tiles in pairs");
  __shared__ __align__(128) bf16 s_in[(TH + 2) * (TW + 2) * CIN];
  __shared__ __align__(128) bf16 s_w[9 * CIN * COUT];
  for (int i = threadIdx.x; i < 9 * CIN * COUT / 8; i += kThreads) {
    const int r = i / (COUT / 8), c = i % (COUT / 8);
    *reinterpret_cast<uint4*>(s_w + tile_off<COUT>(r, c)) = reinterpret_cast<const uint4*>(w)[i];
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int lj = lane >> 3, lr = lane & 7;  // ldmatrix: matrix and row this lane addresses
  const int tiles_x = W / TW, tiles_y = H / TH;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int b = t / (tiles_x * tiles_y);
    const int ty0 = ((t / tiles_x) % tiles_y) * TH, tx0 = (t % tiles_x) * TW;
    __syncthreads();  // weights staged / previous tile's reads done
    stage_halo<CIN>(s_in, in, b, ty0, tx0, H, W);
    __syncthreads();
    float acc[NTN][4];
#pragma unroll
    for (int n = 0; n < NTN; ++n)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[n][r] = 0.f;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int dy = tap / 3, dx = tap % 3;
#pragma unroll
      for (int c0 = 0; c0 < CIN; c0 += 16) {
        // A: matrices (px 0-7 | 8-15) x (k c0..c0+7 | c0+8..c0+15)
        unsigned af[4];
        {
          const int q = (warp + dy) * (TW + 2) + lr + 8 * (lj & 1) + dx;
          ldsm_x4(af, s_in + tile_off<CIN>(q, (c0 >> 3) + (lj >> 1)));
        }
        const int k0 = tap * CIN + c0;
#pragma unroll
        for (int n = 0; n < NTN; n += 2) {
          // B: matrices (k0..k0+7 | k0+8..) x (co n*8.. | (n+1)*8..), transposed
          unsigned bq[4];
          ldsm_x4_t(bq, s_w + tile_off<COUT>(k0 + lr + 8 * (lj & 1), n + (lj >> 1)));
          const unsigned b0[2] = {bq[0], bq[1]}, b1[2] = {bq[2], bq[3]};
          mma_bf16(acc[n], af, b0);
          mma_bf16(acc[n + 1], af, b1);
        }
      }
    }
    // D: rows gid, gid+8 (pixels), cols n*8 + tig*2 (+1)
    const int gy = ty0 + warp;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int gx = tx0 + gid + half * 8;
      const size_t pix = ((size_t)b * H + gy) * W + gx;
#pragma unroll
      for (int n = 0; n < NTN; ++n) {
        const int co = n * 8 + tig * 2;
        if (co >= cout_store) continue;
        const float v0 = acc[n][half * 2] + (bias ? bias[co] : 0.f);
        const float v1 = acc[n][half * 2 + 1] + (bias ? bias[co + 1] : 0.f);
        if (y) *reinterpret_cast<float2*>(y + pix * cout_store + co) = make_float2(v0, v1);
        if (a)
          *reinterpret_cast<__nv_bfloat162*>(a + pix * COUT + co) =
              __halves2bfloat162(__float2bfloat16_rn(act ? gelu(v0) : v0), __float2bfloat16_rn(act ? gelu(v1) : v1));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The same convolution on the 5th-generation tensor cores (tcgen05), for
// W % 128 == 0.  A CTA of 128 threads owns 128 consecutive pixels of one
// image row per tile (persistent over tiles).  Shared memory holds, in the
// canonical no-swizzle K-major UMMA layout (core matrices of 8 rows x 16 bytes):
//   halo  unit (r, c, p) = 16 bytes = channels 8c..8c+7 of pixel p of halo
//         row r (r = dy, p = 0..129 <-> x0-1 .. x0+128, periodic), at
//         ((r*NCH + c)*130 + p)*16: the A operand of tap (dy, dx), channel
//         chunks c, c+1 is the descriptor starting at unit (dy, c, dx) with
//         leading (K) byte offset 130*16 and stride (M) byte offset 128 --
//         the shifted window needs no copy;
//   weights unit (kc, n) = k = 8kc..8kc+7 of output channel n, at
//         (kc*COUT + n)*16 (B operand, K-major: LBO = COUT*16, SBO = 128).
// One elected thread issues the 9 * CIN/16 MMAs (M = 128, N = COUT, K = 16,
// bf16 x bf16 -> f32) into a 32-column TMEM accumulator and commits them to
// an mbarrier; the 4 warps then read their 32 TMEM lanes (one pixel per
// thread, COUT columns) with tcgen05.ld for the epilogue.  Every wait is
// bounded: a wait that runs out sets *err, waits once more (bounded) for the
// MMAs in flight, frees the TMEM and ends the kernel.
// ---------------------------------------------------------------------------
constexpr int kTcPix = 128;          // pixels per tile (M)
constexpr int kTcThreads = 128;
constexpr unsigned kTcWaitLimit = 1u << 24;  // mbarrier polls before giving up

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle, K-major (version 1 for sm_100+)
__device__ __forceinline__ unsigned long long umma_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
  unsigned long long d = (unsigned long long)((saddr >> 4) & 0x3FFFu);
  d |= (unsigned long long)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (unsigned long long)((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;
  return d;
}
// instruction descriptor of kind::f16: D f32, A and B bf16, both K-major
__host__ __device__ constexpr unsigned umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(unsigned addr, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(addr), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned addr, unsigned parity) {
  for (unsigned i = 0; i < kTcWaitLimit; ++i) {
    if (mbar_try_wait(addr, parity)) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

template <int N>
__device__ __forceinline__ void tmem_ld32(unsigned taddr, unsigned (&r)[N]);
template <>
__device__ __forceinline__ void tmem_ld32<32>(unsigned taddr, unsigned (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld32<16>(unsigned taddr, unsigned (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tc_cp16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void tc_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void tc_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory");
}

template <int CIN, int COUT>
struct TcConv {
  static constexpr int NCH = CIN / 8;
  static constexpr int HALO_UNITS = 3 * NCH * (kTcPix + 2);
  static constexpr int W_UNITS = 9 * CIN * COUT / 8;
  // output staging of one tile: y [128][COUT] f32 and a [128][COUT] bf16,
  // 16-byte chunks XOR-swizzled within each pixel row.  It reuses the tile's
  // own halo buffer (free once the MMAs have completed) when it fits, else
  // it has its own region.
  static constexpr int Y_UNITS = kTcPix * COUT / 4, A_UNITS = kTcPix * COUT / 8;
  static constexpr bool STAGE_IN_HALO = Y_UNITS + A_UNITS <= HALO_UNITS;
  static constexpr int STAGE_UNITS = STAGE_IN_HALO ? 0 : Y_UNITS + A_UNITS;
  // two halo buffers (the next tile's is copied while this one's runs), the
  // weights, the output staging, the mbarrier, the TMEM address and the bias
  static constexpr size_t SMEM = (size_t)(2 * HALO_UNITS + W_UNITS + STAGE_UNITS) * 16 + 16 + 4 * 32;
};

// halo of tile t into buffer dst (one cp.async commit group; empty when
// t >= ntiles)
template <int CIN>
__device__ __forceinline__ void tc_stage_halo(uint4* dst, const bf16* __restrict__ in, int t, int ntiles, int H,
                                              int W) {
  constexpr int NCH = CIN / 8, HP = kTcPix + 2;
  if (t < ntiles) {
    const int tiles_x = W / kTcPix;
    const int b = t / (tiles_x * H), gy = (t / tiles_x) % H, x0 = (t % tiles_x) * kTcPix;
    for (int i = threadIdx.x; i < 3 * NCH * HP; i += kTcThreads) {
      const int c = i % NCH, p = (i / NCH) % HP, r = i / (NCH * HP);
      int sy = gy + r - 1, sx = x0 + p - 1;
      sy += sy < 0 ? H : (sy >= H ? -H : 0);
      sx += sx < 0 ? W : (sx >= W ? -W : 0);
      tc_cp16(dst + (r * NCH + c) * HP + p, in + (((size_t)b * H + sy) * W + sx) * CIN + c * 8);
    }
  }
  tc_commit();
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(kTcThreads)
k_conv_tc(const bf16* __restrict__ in, const bf16* __restrict__ wt, const float* __restrict__ bias, int H, int W,
          int ntiles, float* __restrict__ y, bf16* __restrict__ a, int act, int cout_store, int* __restrict__ err) {
  using TC = TcConv<CIN, COUT>;
  constexpr int NCH = TC::NCH, HP = kTcPix + 2;
  constexpr unsigned IDESC = umma_idesc_bf16(kTcPix, COUT);
  extern __shared__ __align__(128) unsigned char tc_smem[];
  uint4* s_halo = reinterpret_cast<uint4*>(tc_smem);  // two buffers
  uint4* s_w = s_halo + 2 * TC::HALO_UNITS;
  uint4* s_stage = s_w + TC::W_UNITS;  // own staging region (STAGE_UNITS)
  unsigned long long* s_bar = reinterpret_cast<unsigned long long*>(s_stage + TC::STAGE_UNITS);
  unsigned* s_tmem = reinterpret_cast<unsigned*>(s_bar + 1);
  float* s_bias = reinterpret_cast<float*>(s_bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // Launched with programmatic stream serialisation: the next convolution
  // may start its prologue (weights, bias, barrier, tensor memory) as this
  // one's CTAs leave; it reads this one's outputs only after
  // griddepcontrol.wait, which returns once this grid has completed and
  // its writes are visible.  Nothing before that wait reads what a
  // preceding kernel writes or writes what it reads.
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  // the bias (the last layer's has only its cout_store real channels)
  if (tid < COUT) s_bias[tid] = bias && tid < cout_store ? bias[tid] : 0.f;
  // weights, already in the K-major UMMA layout: unit (kc, n) = k 8kc..8kc+7 of column n
  for (int i = tid; i < TC::W_UNITS; i += kTcThreads) tc_cp16(s_w + i, wt + (size_t)i * 8);
  tc_commit();
  int t = blockIdx.x;
  const unsigned bar = smem_u32(s_bar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;\n" ::"r"(smem_u32(s_tmem))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = *s_tmem;
  asm volatile("griddepcontrol.wait;\n" ::: "memory");  // the input activations are complete
  tc_stage_halo<CIN>(s_halo, in, t, ntiles, H, W);
  const int tiles_x = W / kTcPix;
  unsigned phase = 0;
  for (int it = 0; t < ntiles; t += gridDim.x, ++it) {
    uint4* cur = s_halo + (it & 1) * TC::HALO_UNITS;
    // the next tile's halo into the other buffer (its last reader, the
    // previous tile's MMAs, has completed)
    tc_stage_halo<CIN>(s_halo + ((it + 1) & 1) * TC::HALO_UNITS, in, t + gridDim.x, ntiles, H, W);
    tc_wait<1>();  // weights and this tile's halo landed
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // visible to the tensor cores
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const unsigned hb = smem_u32(cur), wb = smem_u32(s_w);
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
#pragma unroll
        for (int kk = 0; kk < CIN / 16; ++kk) {
          const unsigned long long ad = umma_desc(hb + (unsigned)(((dy * NCH + 2 * kk) * HP + dx) * 16), HP * 16, 128);
          const int kc = (tap * CIN + 16 * kk) / 8;
          const unsigned long long bd = umma_desc(wb + (unsigned)(kc * COUT * 16), COUT * 16, 128);
          const unsigned accum = (tap | kk) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(IDESC), "r"(accum)
              : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                   : "memory");
    }
    const bool done = mbar_wait_bounded(bar, phase);
    if (__syncthreads_or(!done)) {  // the same decision in every thread
      if (tid == 0) atomicExch(err, 1);
      mbar_wait_bounded(bar, phase);  // one more bounded wait for the MMAs in flight
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    unsigned r[COUT];
    tmem_ld32<COUT>(tmem + ((unsigned)(warp * 32) << 16), r);
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    // epilogue: pixel m = 32*warp + lane of the tile, COUT accumulators
    uint4* s_y = TC::STAGE_IN_HALO ? cur : s_stage;
    uint4* s_a = s_y + TC::Y_UNITS;
    const int b = t / (tiles_x * H), gy = (t / tiles_x) % H, x0 = (t % tiles_x) * kTcPix;
    const size_t pix0 = ((size_t)b * H + gy) * W + x0;  // the tile's pixels are contiguous
    const int m = warp * 32 + lane;
    float v[COUT];
#pragma unroll
    for (int co = 0; co < COUT; ++co) v[co] = __uint_as_float(r[co]) + s_bias[co];
    if (y && cout_store < COUT) {
      // the network output (2 channels): 8 bytes per pixel straight from registers
#pragma unroll
      for (int co = 0; co < COUT; co += 2)
        if (co < cout_store) *reinterpret_cast<float2*>(y + (pix0 + m) * cout_store + co) = make_float2(v[co], v[co + 1]);
    }
    // full rows go through the swizzled staging so that the global stores of
    // the tile are contiguous 16-byte chunks
    constexpr int YC = COUT / 4, AC = COUT / 8;  // 16-byte chunks per pixel row
    if (y && cout_store == COUT) {
#pragma unroll
      for (int c = 0; c < YC; ++c)
        s_y[m * YC + (c ^ (m % YC))] = make_uint4(__float_as_uint(v[4 * c]), __float_as_uint(v[4 * c + 1]),
                                                  __float_as_uint(v[4 * c + 2]), __float_as_uint(v[4 * c + 3]));
    }
    if (a) {
#pragma unroll
      for (int c = 0; c < AC; ++c) {
        unsigned u[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float p0 = v[8 * c + 2 * e], p1 = v[8 * c + 2 * e + 1];
          u[e] = pack_bf16(__float2bfloat16_rn(act ? gelu(p0) : p0), __float2bfloat16_rn(act ? gelu(p1) : p1));
        }
        s_a[m * AC + (c ^ ((m / (8 / AC)) % AC))] = make_uint4(u[0], u[1], u[2], u[3]);
      }
    }
    __syncthreads();  // staging complete; TMEM read before the next tile's MMAs
    if (y && cout_store == COUT) {
      uint4* gy4 = reinterpret_cast<uint4*>(y + pix0 * COUT);
      for (int q = tid; q < TC::Y_UNITS; q += kTcThreads) {
        const int mm = q / YC, c = q % YC;
        gy4[q] = s_y[mm * YC + (c ^ (mm % YC))];
      }
    }
    if (a) {
      uint4* ga4 = reinterpret_cast<uint4*>(a + pix0 * COUT);
      for (int q = tid; q < TC::A_UNITS; q += kTcThreads) {
        const int mm = q / AC, c = q % AC;
        ga4[q] = s_a[mm * AC + (c ^ ((mm / (8 / AC)) % AC))];
      }
    }
    // the staging (possibly this tile's halo buffer, which the copy issued
    // at the top of the next-but-one iteration refills) is free only after
    // every thread's copy-out
    if constexpr (TC::STAGE_IN_HALO) __syncthreads();
  }
  tc_wait<0>();  // no copy outlives the CTA
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;\n" ::"r"(tmem) : "memory");
  }
}

// ---------------------------------------------------------------------------
// dW[k][co] and db[co] partials: CTA c accumulates over pixel tiles c,
// c + grid, ...  in: [B][H][W][CIN] bf16, dy: [B][H][W][COUT] bf16;
// part: [grid][9*CIN*COUT + COUT] (weights, then bias).  The GEMM is
// dW = in_col^T dY over the tile's 128 pixels (8 k-steps of one tile row);
// warp w owns the m-tiles (16 rows of k) w, w+8, w+16 and all n-tiles.
// Both fragments come from the transposing ldmatrix.
// ---------------------------------------------------------------------------
template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads)
k_conv_wgrad(const bf16* __restrict__ in, const bf16* __restrict__ dy, int H, int W, int ntiles,
             float* __restrict__ part) {
  constexpr int K = 9 * CIN, MT = K / 16, NTN = COUT / 8;
  constexpr int MPW = (MT + 7) / 8;  // m-tiles per warp (at most)
  static_assert(NTN % 2 == 0, "n-tiles in pairs");
  __shared__ __align__(128) bf16 s_in[(TH + 2) * (TW + 2) * CIN];
  __shared__ __align__(128) bf16 s_dy[TH * TW * COUT];
  __shared__ float s_b[kThreads];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lj = lane >> 3, lr = lane & 7;
  float acc[MPW][NTN][4];
#pragma unroll
  for (int i = 0; i < MPW; ++i)
#pragma unroll
    for (int n = 0; n < NTN; ++n)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][n][r] = 0.f;
  float bsum = 0.f;  // bias partial of channel threadIdx.x % COUT
  const int tiles_x = W / TW, tiles_y = H / TH;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int b = t / (tiles_x * tiles_y);
    const int ty0 = ((t / tiles_x) % tiles_y) * TH, tx0 = (t % tiles_x) * TW;
    __syncthreads();
    stage_halo<CIN>(s_in, in, b, ty0, tx0, H, W);
    constexpr int VPO = COUT / 8;
    for (int i = threadIdx.x; i < TH * TW * VPO; i += kThreads) {
      const int v = i % VPO, p = i / VPO, px = p % TW, py = p / TW;
      *reinterpret_cast<uint4*>(s_dy + tile_off<COUT>(p, v)) =
          reinterpret_cast<const uint4*>(dy + (((size_t)b * H + ty0 + py) * W + tx0 + px) * COUT)[v];
    }
    __syncthreads();
    {  // bias: fixed pixel order per thread
      const int co = threadIdx.x % COUT;
      for (int p = threadIdx.x / COUT; p < TH * TW; p += kThreads / COUT)
        bsum += __bfloat162float(s_dy[tile_off<COUT>(p, co >> 3) + (co & 7)]);
    }
#pragma unroll 1
    for (int ks = 0; ks < TH; ++ks) {
      // B fragments of this k-step (pixels ks*TW .. +15) for every n-tile
      unsigned bq[NTN / 2][4];
#pragma unroll
      for (int n = 0; n < NTN; n += 2)
        ldsm_x4_t(bq[n / 2], s_dy + tile_off<COUT>(ks * TW + lr + 8 * (lj & 1), n + (lj >> 1)));
#pragma unroll
      for (int i = 0; i < MPW; ++i) {
        const int mt = warp + 8 * i;
        if (mt >= MT) break;
        const int tap = (mt * 16) / CIN, ci0 = (mt * 16) % CIN, dyy = tap / 3, dxx = tap % 3;
        // A = in_col^T: matrices (px 0-7 | 8-15) x (ch ci0.. | ci0+8..), transposed
        unsigned af[4];
        {
          const int q = (ks + dyy) * (TW + 2) + lr + 8 * (lj >> 1) + dxx;
          ldsm_x4_t(af, s_in + tile_off<CIN>(q, (ci0 >> 3) + (lj & 1)));
        }
#pragma unroll
        for (int n = 0; n < NTN; ++n) {
          const unsigned bf[2] = {bq[n / 2][(n & 1) * 2], bq[n / 2][(n & 1) * 2 + 1]};
          mma_bf16(acc[i][n], af, bf);
        }
      }
    }
  }
  float* out = part + (size_t)blockIdx.x * (K * COUT + COUT);
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int i = 0; i < MPW; ++i) {
    const int mt = warp + 8 * i;
    if (mt >= MT) break;
#pragma unroll
    for (int n = 0; n < NTN; ++n)
#pragma unroll
      for (int h = 0; h < 2; ++h)
        *reinterpret_cast<float2*>(out + (size_t)(mt * 16 + gid + h * 8) * COUT + n * 8 + tig * 2) =
            make_float2(acc[i][n][h * 2], acc[i][n][h * 2 + 1]);
  }
  s_b[threadIdx.x] = bsum;
  __syncthreads();
  if (threadIdx.x < COUT) {
    float s = 0.f;
    for (int j = threadIdx.x; j < kThreads; j += COUT) s += s_b[j];
    out[K * COUT + threadIdx.x] = s;
  }
}

// grad[i] = sum_c part[c][i] in fixed order
__global__ void k_reduce_parts(const float* __restrict__ part, int nparts, int count, float* __restrict__ grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float s = 0.f;
  for (int c = 0; c < nparts; ++c) s += part[(size_t)c * count + i];
  grad[i] = s;
}

// dY' = dA * gelu'(y) (bf16), for the hidden layers
__global__ void k_gelu_back(const bf16* __restrict__ da, const float* __restrict__ y, size_t count,
                            bf16* __restrict__ dy) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    dy[i] = __float2bfloat16_rn(__bfloat162float(da[i]) * gelu_d(y[i]));
}

// MSE loss of the 2 output channels against the target; dY of the last
// layer (padded to 16 channels, zero beyond 2) and per-CTA loss partials
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ tgt, size_t npix, float scale,
                      const float* __restrict__ tmean, const float* __restrict__ tsd, bf16* __restrict__ dy,
                      float* __restrict__ lpart) {
  __shared__ float red[256];
  float s = 0.f;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      float g = 0.f;
      if (c < 2) {
        const float d = out[p * 2 + c] - (tgt[p * 2 + c] - tmean[c]) / tsd[c];
        s += d * d;
        g = 2.f * d * scale;
      }
      dy[p * 16 + c] = __float2bfloat16_rn(g);
    }
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) lpart[blockIdx.x] = red[0];
}

// dY of the last layer from a caller's output gradient g = dL/d(out) in
// physical output units: out = y * std + mean, so dL/dy = g * std (bf16,
// padded to 16 channels, zero beyond 2)
__global__ void k_gout(const float* __restrict__ g, size_t npix, const float* __restrict__ tsd,
                       bf16* __restrict__ dy) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix * 16; i += (size_t)gridDim.x * blockDim.x) {
    const size_t p = i >> 4;
    const int c = (int)(i & 15);
    dy[i] = __float2bfloat16_rn(c < 2 ? g[p * 2 + c] * tsd[c] : 0.f);
  }
}

// dL/dx (FP32 NHWC, 8 channels) from the gradient of the network's
// standardised bf16 input (16 channels): x' = (x - mean) / std
__global__ void k_gin(const bf16* __restrict__ da, size_t npix, const float* __restrict__ sd,
                      float* __restrict__ gx) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix * 8; i += (size_t)gridDim.x * blockDim.x) {
    const size_t p = i >> 3;
    const int c = (int)(i & 7);
    gx[i] = __bfloat162float(da[p * 16 + c]) / sd[c];
  }
}

// Adam on FP32 master weights; also writes the bf16 forward weights
// wf[k][co] (padded shapes) and the backward-data weights wb[k'][ci] with
// k' = (8 - tap)*COUTP + co.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int count, float lr, float b1, float b2, float eps, float bc1,
                       float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// master weights [9][cin][cout] (unpadded) -> wf [9*CINP][COUTP], wb [9*COUTP][CINP]
// and the same two matrices in the K-major UMMA layout of the tensor-core
// convolution: element (k, n) of a K x N matrix at ((k/8)*N + n)*8 + k%8.
__global__ void k_pack_weights(const float* __restrict__ wm, int cin, int cout, int cinp, int coutp,
                               bf16* __restrict__ wf, bf16* __restrict__ wb, bf16* __restrict__ wtf,
                               bf16* __restrict__ wtb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 9 * cinp * coutp) return;
  const int co = i % coutp, ci = (i / coutp) % cinp, tap = i / (coutp * cinp);
  const float v = (ci < cin && co < cout) ? wm[((size_t)tap * cin + ci) * cout + co] : 0.f;
  const bf16 h = __float2bfloat16_rn(v);
  const int kf = tap * cinp + ci, kb = (8 - tap) * coutp + co;
  wf[(size_t)kf * coutp + co] = h;
  wb[(size_t)kb * cinp + ci] = h;
  wtf[((size_t)(kf >> 3) * coutp + co) * 8 + (kf & 7)] = h;
  wtb[((size_t)(kb >> 3) * cinp + ci) * 8 + (kb & 7)] = h;
}

// padded weight gradient [9][cinp][coutp] -> parameter layout [9][cin][cout];
// the padded bias gradient (coutp entries after the weights) -> gb[cout]
__global__ void k_unpad_wgrad(const float* __restrict__ gp, int cin, int cout, int cinp, int coutp,
                              float* __restrict__ g, float* __restrict__ gb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nw = 9 * cin * cout;
  if (i < nw) {
    const int co = i % cout, ci = (i / cout) % cin, tap = i / (cout * cin);
    g[i] = gp[((size_t)tap * cinp + ci) * coutp + co];
  } else if (i < nw + cout) {
    gb[i - nw] = gp[(size_t)9 * cinp * coutp + (i - nw)];
  }
}

// FP32 NHWC [npix][c] -> bf16 NHWC [npix][cp], (x - mean[ch]) / std[ch],
// zero padding channels
__global__ void k_to_bf16(const float* __restrict__ x, size_t npix, int c, int cp, const float* __restrict__ mean,
                          const float* __restrict__ sd, bf16* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix * cp; i += (size_t)gridDim.x * blockDim.x) {
    const size_t p = i / cp;
    const int ch = (int)(i % cp);
    out[i] = __float2bfloat16_rn(ch < c ? (x[p * c + ch] - mean[ch]) / sd[ch] : 0.f);
  }
}

// out = y * std[ch] + mean[ch] for the 2 output channels (one fused
// multiply-add, as the fused closure path computes it)
__global__ void k_denorm(const float* __restrict__ y, size_t npix, const float* __restrict__ mean,
                         const float* __restrict__ sd, float* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npix * 2; i += (size_t)gridDim.x * blockDim.x) {
    const int ch = (int)(i & 1);
    out[i] = fmaf(y[i], sd[ch], mean[ch]);
  }
}

// unpadded dX of layer 0's input is not needed; bias-gradient buffers etc.
struct Layer {
  int cin, cout, cinp, coutp;
  size_t woff, boff;  // offsets in the parameter vector
};

// Resident CTAs of kernel k on the whole current device (computed once per
// kernel).
template <typename K>
int resident_ctas(K k) {
  int dev = 0, sms = 0, per_sm = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, 0),
             "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  return std::max(1, per_sm) * sms;
}

template <int CIN, int COUT>
void conv_launch(const bf16* in, const bf16* w, const float* b, int B, int H, int W, float* y, bf16* a, int act,
                 int cout_store, int ctas, cudaStream_t st) {
  const int tiles = B * (H / TH) * (W / TW);
  k_conv<CIN, COUT><<<std::min(tiles, ctas), kThreads, 0, st>>>(in, w, b, H, W, tiles, y, a, act, cout_store);
}

template <int CIN, int COUT>
void conv_tc_launch(const bf16* in, const bf16* w, const float* b, int B, int H, int W, float* y, bf16* a, int act,
                    int cout_store, int ctas, int* err, cudaStream_t st) {
  const int tiles = B * H * (W / kTcPix);
  // programmatic stream serialisation: the prologue overlaps the preceding
  // kernel's tail (k_conv_tc waits before its first read of `in`)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(std::min(tiles, ctas));
  cfg.blockDim = dim3(kTcThreads);
  cfg.dynamicSmemBytes = TcConv<CIN, COUT>::SMEM;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cuda_check(cudaLaunchKernelEx(&cfg, k_conv_tc<CIN, COUT>, in, w, b, H, W, tiles, y, a, act, cout_store, err),
             "k_conv_tc");
}
template <int CIN, int COUT>
int resident_tc_ctas() {
  cuda_check(cudaFuncSetAttribute(k_conv_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)TcConv<CIN, COUT>::SMEM),
             "cudaFuncSetAttribute(max dynamic smem)");
  // the whole unified L1/shared array as shared memory, so that several
  // CTAs (and their copy pipelines) share each SM
  cuda_check(cudaFuncSetAttribute(k_conv_tc<CIN, COUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared),
             "cudaFuncSetAttribute(carveout)");
  int dev = 0, sms = 0, per_sm = 0, smem_sm = 0, reserved = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv_tc<CIN, COUT>, kTcThreads,
                                                           TcConv<CIN, COUT>::SMEM),
             "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  // the shared-memory bound itself (with the carveout at its maximum)
  cuda_check(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev),
             "cudaDeviceGetAttribute");
  cuda_check(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev), "cudaDeviceGetAttribute");
  const int by_smem = smem_sm / (int)(TcConv<CIN, COUT>::SMEM + reserved);
  return std::max(1, std::max(per_sm, std::min(by_smem, 8))) * sms;
}

template <int CIN, int COUT>
void wgrad_launch(const bf16* in, const bf16* dy, int B, int H, int W, float* part, int nparts, cudaStream_t st) {
  const int tiles = B * (H / TH) * (W / TW);
  k_conv_wgrad<CIN, COUT><<<nparts, kThreads, 0, st>>>(in, dy, H, W, tiles, part);
}

}  // namespace

struct r2d3c_cnn {
  int H = 0, W = 0, Bmax = 0;
  unsigned long long serial = 0;  // unique per network created in this process
  int ctas[3] = {};               // resident CTAs of k_conv<16,32>, <32,32>, <32,16>
  int tc_ctas[3] = {};            // and of k_conv_tc
  bool use_tc = false;            // tcgen05 convolutions (W % 128 == 0)
  int* err = nullptr;             // set by a device wait that gave up
  cudaStream_t st = nullptr;
  Layer L[kLayers];
  size_t nparam = 0;
  float *wm = nullptr, *grad = nullptr, *am = nullptr, *av = nullptr;  // master params, grads, Adam moments
  bf16* wf[kLayers] = {};
  bf16* wb[kLayers] = {};
  bf16* wtf[kLayers] = {};  // forward / backward-data weights in the UMMA layout
  bf16* wtb[kLayers] = {};
  bf16* act[kLayers + 1] = {};   // act[0] = bf16 input (16 ch), act[l+1] = layer l output (bf16)
  float* pre[kLayers] = {};      // pre-activations y (f32), last = network output (2 ch)
  bf16 *dA = nullptr, *dY = nullptr;
  float* part = nullptr;
  float* lpart = nullptr;
  float* norm = nullptr;  // in mean[8], in std[8], out mean[2], out std[2]
  int nparts = 304;
  long long step = 0;
  std::vector<void*> owned;
  template <typename U>
  U* alloc(size_t n) {
    void* p = nullptr;
    cuda_check(cudaMalloc(&p, n * sizeof(U)), "cudaMalloc (cnn)");
    owned.push_back(p);
    return static_cast<U*>(p);
  }
  ~r2d3c_cnn() {
    for (void* p : owned) cudaFree(p);
    if (st) cudaStreamDestroy(st);
  }

  // a bounded device wait that gave up (tcgen05 convolutions) -> R2D3C_ETIMEOUT
  void check_err() {
    int h = 0;
    cuda_check(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H error flag");
    cuda_check(cudaStreamSynchronize(st), "sync");
    if (h) {
      cuda_check(cudaMemsetAsync(err, 0, sizeof(int), st), "memset");
      throw Error(kETIMEOUT, "a tensor-core convolution wait gave up");
    }
  }
  void conv(int l, const bf16* in, const bf16* w, int B, float* y, bf16* a, int act_on, bool bias, bool back) {
    const float* b = bias ? wm + L[l].boff : nullptr;
    // forward shapes (CINP, COUTP) or backward-data shapes (COUTP, CINP)
    const int ci = back ? L[l].coutp : L[l].cinp, co = back ? L[l].cinp : L[l].coutp;
    const int store = back ? co : (l == kLayers - 1 ? L[l].cout : co);
    if (use_tc) {
      const bf16* wt = back ? wtb[l] : wtf[l];  // the same matrix as w, UMMA layout
      if (ci == 16 && co == 32) conv_tc_launch<16, 32>(in, wt, b, B, H, W, y, a, act_on, store, tc_ctas[0], err, st);
      else if (ci == 32 && co == 32)
        conv_tc_launch<32, 32>(in, wt, b, B, H, W, y, a, act_on, store, tc_ctas[1], err, st);
      else if (ci == 32 && co == 16)
        conv_tc_launch<32, 16>(in, wt, b, B, H, W, y, a, act_on, store, tc_ctas[2], err, st);
      else throw Error(kEINVAL, "unsupported conv shape");
    } else if (ci == 16 && co == 32) conv_launch<16, 32>(in, w, b, B, H, W, y, a, act_on, store, ctas[0], st);
    else if (ci == 32 && co == 32) conv_launch<32, 32>(in, w, b, B, H, W, y, a, act_on, store, ctas[1], st);
    else if (ci == 32 && co == 16) conv_launch<32, 16>(in, w, b, B, H, W, y, a, act_on, store, ctas[2], st);
    else throw Error(kEINVAL, "unsupported conv shape");
    cuda_check(cudaGetLastError(), "k_conv");
  }
  void wgrad(int l, const bf16* in, const bf16* dy, int B) {
    const int ci = L[l].cinp, co = L[l].coutp;
    if (ci == 16 && co == 32) wgrad_launch<16, 32>(in, dy, B, H, W, part, nparts, st);
    else if (ci == 32 && co == 32) wgrad_launch<32, 32>(in, dy, B, H, W, part, nparts, st);
    else if (ci == 32 && co == 16) wgrad_launch<32, 16>(in, dy, B, H, W, part, nparts, st);
    else throw Error(kEINVAL, "unsupported wgrad shape");
    cuda_check(cudaGetLastError(), "k_conv_wgrad");
  }

  // forward of a batch of B inputs (f32 NHWC 8 ch) -> pre[kLayers-1] (f32 NHWC 2 ch);
  // the hidden layers' pre-activations (kept for the backward pass) are
  // written only when train is set
  void forward(const float* x, int B, bool train) {
    const size_t npix = (size_t)B * H * W;
    k_to_bf16<<<1024, 256, 0, st>>>(x, npix, 8, 16, norm, norm + 8, act[0]);
    cuda_check(cudaGetLastError(), "k_to_bf16");
    layers(B, train);
  }
  // the six layers from act[0] (bf16, 16 ch) into pre[kLayers-1]
  void layers(int B, bool train) {
    for (int l = 0; l < kLayers; ++l) {
      const bool last = l == kLayers - 1;
      conv(l, act[l], wf[l], B, last || train ? pre[l] : nullptr, last ? nullptr : act[l + 1], last ? 0 : 1, true,
           false);
    }
  }

  // gradients of the MSE loss into grad[]; returns the loss (host sync)
  double backward(const float* tgt, int B) {
    const size_t npix = (size_t)B * H * W;
    const float scale = 1.0f / (float)(npix * 2);
    k_mse<<<256, 256, 0, st>>>(pre[kLayers - 1], tgt, npix, scale, norm + 16, norm + 18, dY, lpart);
    cuda_check(cudaGetLastError(), "k_mse");
    backprop(B, nullptr);
    std::vector<float> lp(256);
    cuda_check(cudaMemcpyAsync(lp.data(), lpart, 256 * sizeof(float), cudaMemcpyDeviceToHost, st), "D2H loss");
    cuda_check(cudaStreamSynchronize(st), "sync");
    double s = 0.0;
    for (float v : lp) s += v;
    return s / (double)(npix * 2);
  }

  // From dY = dL/dy of the last layer (as the forward pass left it, with
  // the hidden pre-activations kept): the parameter gradients into grad[]
  // and, when gx is set, dL/dx of the FP32 input into gx
  void backprop(int B, float* gx) {
    const size_t npix = (size_t)B * H * W;
    for (int l = kLayers - 1; l >= 0; --l) {
      const Layer& ly = L[l];
      // dY holds dL/dy of layer l (bf16, coutp channels)
      wgrad(l, act[l], dY, B);
      // per-CTA partials: 9*cinp*coutp weight entries, then coutp bias entries
      const int kc = 9 * ly.cinp * ly.coutp + ly.coutp;
      k_reduce_parts<<<(kc + 255) / 256, 256, 0, st>>>(part, nparts, kc, part + (size_t)nparts * kc);
      cuda_check(cudaGetLastError(), "k_reduce_parts");
      // unpad into grad (layout [9][cin][cout], then the bias)
      unpad_wgrad(l, part + (size_t)nparts * kc);
      // dA of layer l's input = conv(dY, wb[l]) (backward data)
      if (l == 0) {
        if (gx) {
          conv(0, dY, wb[0], B, nullptr, dA, 0, false, true);
          k_gin<<<1024, 256, 0, st>>>(dA, npix, norm + 8, gx);
          cuda_check(cudaGetLastError(), "k_gin");
        }
        break;
      }
      // then dY' = dA * gelu'(pre[l-1])
      conv(l, dY, wb[l], B, nullptr, dA, 0, false, true);
      k_gelu_back<<<1024, 256, 0, st>>>(dA, pre[l - 1], npix * L[l - 1].coutp, dY);
      cuda_check(cudaGetLastError(), "k_gelu_back");
    }
  }

  void unpad_wgrad(int l, const float* gp) {
    const Layer& ly = L[l];
    const int c = 9 * ly.cin * ly.cout + ly.cout;
    k_unpad_wgrad<<<(c + 255) / 256, 256, 0, st>>>(gp, ly.cin, ly.cout, ly.cinp, ly.coutp, grad + ly.woff,
                                                    grad + ly.boff);
    cuda_check(cudaGetLastError(), "k_unpad_wgrad");
  }

  void pack() {
    for (int l = 0; l < kLayers; ++l) {
      const Layer& ly = L[l];
      const int c = 9 * ly.cinp * ly.coutp;
      k_pack_weights<<<(c + 255) / 256, 256, 0, st>>>(wm + ly.woff, ly.cin, ly.cout, ly.cinp, ly.coutp, wf[l], wb[l],
                                                      wtf[l], wtb[l]);
      cuda_check(cudaGetLastError(), "k_pack_weights");
    }
  }

  void adam(float lr) {
    ++step;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float bc1 = 1.f - std::pow(b1, (float)step), bc2 = 1.f - std::pow(b2, (float)step);
    k_adam<<<(int)((nparam + 255) / 256), 256, 0, st>>>(wm, grad, am, av, (int)nparam, lr, b1, b2, eps, bc1, bc2);
    cuda_check(cudaGetLastError(), "k_adam");
    pack();
  }
};

namespace r2d3c {
// Forward of one batch queued on `stream` (no synchronisation; capturable):
// the network's own buffers and weights, the output denormalised into d_out.
void cnn_forward_on(r2d3c_cnn* c, const float* d_x, int batch, float* d_out, cudaStream_t stream) {
  cudaStream_t own = c->st;
  c->st = stream;
  try {
    c->forward(d_x, batch, false);
    k_denorm<<<512, 256, 0, stream>>>(c->pre[kLayers - 1], (size_t)batch * c->H * c->W, c->norm + 16,
                                      c->norm + 18, d_out);
    cuda_check(cudaGetLastError(), "k_denorm");
  } catch (...) {
    c->st = own;
    throw;
  }
  c->st = own;
}
void cnn_check_err(r2d3c_cnn* c) { c->check_err(); }
// The network's input activation (bf16 [H][W][16] of batch entry 0), its
// standardised output (f32 [H][W][2]) and its normalisation (in mean[8],
// in std[8], out mean[2], out std[2]), for callers that fill the input and
// read the output themselves (the fused LES step)
void cnn_io(r2d3c_cnn* c, void** act0, const float** out, const float** norm) {
  *act0 = c->act[0];
  *out = c->pre[kLayers - 1];
  *norm = c->norm;
}
// The six layers of a batch whose input activation is already in place,
// queued on `stream` (capturable)
void cnn_layers_on(r2d3c_cnn* c, int batch, cudaStream_t stream) {
  cudaStream_t own = c->st;
  c->st = stream;
  try {
    c->layers(batch, false);
  } catch (...) {
    c->st = own;
    throw;
  }
  c->st = own;
}
void cnn_shape(const r2d3c_cnn* c, int* H, int* W, int* max_batch, unsigned long long* serial) {
  *H = c->H;
  *W = c->W;
  *max_batch = c->Bmax;
  *serial = c->serial;
}
}  // namespace r2d3c

namespace {
int fail(const Error& e) {
  last_error_slot() = e.what();
  return e.code;
}
}  // namespace

extern "C" {

int r2d3c_cnn_create(int H, int W, int max_batch, int seed, r2d3c_cnn** out) {
  try {
    if (!out) throw Error(kEINVAL, "NULL argument");
    *out = nullptr;
    if (H < TH || W < TW || H % TH || W % TW) throw Error(kEINVAL, "H must be a multiple of 8 and W of 16");
    if (max_batch < 1) throw Error(kEINVAL, "max_batch must be >= 1");
    std::unique_ptr<r2d3c_cnn> c(new r2d3c_cnn());
    c->H = H;
    c->W = W;
    c->Bmax = max_batch;
    static std::atomic<unsigned long long> next_serial{1};
    c->serial = next_serial++;
    c->ctas[0] = resident_ctas(k_conv<16, 32>);
    c->ctas[1] = resident_ctas(k_conv<32, 32>);
    c->ctas[2] = resident_ctas(k_conv<32, 16>);
    // tcgen05 convolutions where a tile of 128 pixels fits a row;
    // R2D3C_CNN_CONV=mma selects the warp-level MMA kernels everywhere
    const char* conv_env = std::getenv("R2D3C_CNN_CONV");
    if (conv_env && std::strcmp(conv_env, "mma") != 0 && std::strcmp(conv_env, "tcgen05") != 0)
      throw Error(kEINVAL, "R2D3C_CNN_CONV must be mma or tcgen05");
    c->use_tc = W % kTcPix == 0 && !(conv_env && std::strcmp(conv_env, "mma") == 0);
    if (c->use_tc) {
      c->tc_ctas[0] = resident_tc_ctas<16, 32>();
      c->tc_ctas[1] = resident_tc_ctas<32, 32>();
      c->tc_ctas[2] = resident_tc_ctas<32, 16>();
    }
    cuda_check(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking), "cudaStreamCreate");
    size_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
      c->L[l] = Layer{kCin[l], kCout[l], kCinPad[l], kCoutPad[l], off, 0};
      off += (size_t)9 * kCin[l] * kCout[l];
      c->L[l].boff = off;
      off += kCout[l];
    }
    c->nparam = off;
    c->wm = c->alloc<float>(off);
    c->grad = c->alloc<float>(off);
    c->am = c->alloc<float>(off);
    c->av = c->alloc<float>(off);
    cuda_check(cudaMemsetAsync(c->am, 0, off * sizeof(float), c->st), "memset");
    cuda_check(cudaMemsetAsync(c->av, 0, off * sizeof(float), c->st), "memset");
    cuda_check(cudaMemsetAsync(c->grad, 0, off * sizeof(float), c->st), "memset");
    // Kaiming-uniform weights (fan_in = 9 cin), zero biases, seeded
    std::vector<float> h(off, 0.f);
    std::mt19937 rng((unsigned)seed);
    for (int l = 0; l < kLayers; ++l) {
      const float bound = std::sqrt(6.0f / (9.0f * (float)kCin[l])) * (l == kLayers - 1 ? 0.1f : 1.0f);
      std::uniform_real_distribution<float> U(-bound, bound);
      for (size_t i = 0; i < (size_t)9 * kCin[l] * kCout[l]; ++i) h[c->L[l].woff + i] = U(rng);
    }
    cuda_check(cudaMemcpyAsync(c->wm, h.data(), off * sizeof(float), cudaMemcpyHostToDevice, c->st), "H2D");
    const size_t npix = (size_t)max_batch * H * W;
    for (int l = 0; l < kLayers; ++l) {
      c->wf[l] = c->alloc<bf16>((size_t)9 * kCinPad[l] * kCoutPad[l]);
      c->wb[l] = c->alloc<bf16>((size_t)9 * kCinPad[l] * kCoutPad[l]);
      c->wtf[l] = c->alloc<bf16>((size_t)9 * kCinPad[l] * kCoutPad[l]);
      c->wtb[l] = c->alloc<bf16>((size_t)9 * kCinPad[l] * kCoutPad[l]);
      c->pre[l] = c->alloc<float>(npix * (l == kLayers - 1 ? kCout[l] : kCoutPad[l]));
    }
    c->act[0] = c->alloc<bf16>(npix * 16);
    for (int l = 0; l < kLayers; ++l) c->act[l + 1] = c->alloc<bf16>(npix * kCoutPad[l]);
    c->dA = c->alloc<bf16>(npix * 32);
    c->dY = c->alloc<bf16>(npix * 32);  // dL/dy of the current layer (<= 32 channels)
    c->part = c->alloc<float>((size_t)(c->nparts + 1) * (9 * 32 * 32 + 32));
    c->lpart = c->alloc<float>(256);
    c->norm = c->alloc<float>(20);
    c->err = c->alloc<int>(1);
    cuda_check(cudaMemsetAsync(c->err, 0, sizeof(int), c->st), "memset");
    const float ident[20] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 1, 1};
    cuda_check(cudaMemcpyAsync(c->norm, ident, sizeof(ident), cudaMemcpyHostToDevice, c->st), "H2D");
    c->pack();
    cuda_check(cudaStreamSynchronize(c->st), "sync");
    *out = c.release();
  } catch (const Error& e) {
    return fail(e);
  } catch (const std::exception& e) {
    last_error_slot() = e.what();
    return R2D3C_EINVAL;
  }
  return R2D3C_OK;
}

int r2d3c_cnn_destroy(r2d3c_cnn* c) {
  delete c;
  return R2D3C_OK;
}

int r2d3c_cnn_num_params(const r2d3c_cnn* c, long long* n) {
  if (!c || !n) return R2D3C_EINVAL;
  *n = (long long)c->nparam;
  return R2D3C_OK;
}

int r2d3c_cnn_get_params(r2d3c_cnn* c, float* host) {
  try {
    if (!c || !host) throw Error(kEINVAL, "NULL argument");
    cuda_check(cudaMemcpyAsync(host, c->wm, c->nparam * sizeof(float), cudaMemcpyDeviceToHost, c->st), "D2H");
    cuda_check(cudaStreamSynchronize(c->st), "sync");
  } catch (const Error& e) {
    return fail(e);
  }
  return R2D3C_OK;
}

int r2d3c_cnn_set_params(r2d3c_cnn* c, const float* host) {
  try {
    if (!c || !host) throw Error(kEINVAL, "NULL argument");
    cuda_check(cudaMemcpyAsync(c->wm, host, c->nparam * sizeof(float), cudaMemcpyHostToDevice, c->st), "H2D");
    c->pack();
    cuda_check(cudaStreamSynchronize(c->st), "sync");
  } catch (const Error& e) {
    return fail(e);
  }
  return R2D3C_OK;
}

int r2d3c_cnn_set_normalization(r2d3c_cnn* c, const float* in_mean, const float* in_std, const float* out_mean,
                                const float* out_std) {
  try {
    if (!c || !in_mean || !in_std || !out_mean || !out_std) throw Error(kEINVAL, "NULL argument");
    float h[20];
    for (int i = 0; i < 8; ++i) {
      if (!(in_std[i] > 0.f)) throw Error(kEINVAL, "standard deviations must be positive");
      h[i] = in_mean[i];
      h[8 + i] = in_std[i];
    }
    for (int i = 0; i < 2; ++i) {
      if (!(out_std[i] > 0.f)) throw Error(kEINVAL, "standard deviations must be positive");
      h[16 + i] = out_mean[i];
      h[18 + i] = out_std[i];
    }
    cuda_check(cudaMemcpyAsync(c->norm, h, sizeof(h), cudaMemcpyHostToDevice, c->st), "H2D");
    cuda_check(cudaStreamSynchronize(c->st), "sync");
  } catch (const Error& e) {
    return fail(e);
  }
  return R2D3C_OK;
}

int r2d3c_cnn_forward(r2d3c_cnn* c, const float* d_x, int batch, float* d_out) {
  try {
    if (!c || !d_x || !d_out) throw Error(kEINVAL, "NULL argument");
    if (batch < 1 || batch > c->Bmax) throw Error(kEINVAL, "batch out of range");
    c->forward(d_x, batch, false);
    k_denorm<<<512, 256, 0, c->st>>>(c->pre[kLayers - 1], (size_t)batch * c->H * c->W, c->norm + 16, c->norm + 18,
                                     d_out);
    cuda_check(cudaGetLastError(), "k_denorm");
    c->check_err();
  } catch (const Error& e) {
    return fail(e);
  }
  return R2D3C_OK;
}

int r2d3c_cnn_gradients(r2d3c_cnn* c, const float* d_x, const float* d_y, int batch, float* host_grad,
                        double* loss) {
  try {
    if (!c || !d_x || !d_y) throw Error(kEINVAL, "NULL argument");
    if (batch < 1 || batch > c->Bmax) throw Error(kEINVAL, "batch out of range");
    c->forward(d_x, batch, true);
    const double l = c->backward(d_y, batch);
    c->check_err();
    if (loss) *loss = l;
    if (host_grad) {
      cuda_check(cudaMemcpyAsync(host_grad, c->grad, c->nparam * sizeof(float), cudaMemcpyDeviceToHost, c->st),
                 "D2H");
      cuda_check(cudaStreamSynchronize(c->st), "sync");
    }
  } catch (const Error& e) {
    return fail(e);
  }
  return R2D3C_OK;
}

int r2d3c_cnn_backward(r2d3c_cnn* c, const float* d_x, const float* d_gout, int batch, float* d_gx,
                       float* host_grad) {
  try {
    if (!c || !d_x || !d_gout) throw Error(kEINVAL, "NULL argument");
    if (batch < 1 || batch > c->Bmax) throw Error(kEINVAL, "batch out of range");
    c->forward(d_x, batch, true);
    const size_t npix = (size_t)batch * c->H * c->W;
    k_gout<<<1024, 256, 0, c->st>>>(d_gout, npix, c->norm + 18, c->dY);
    cuda_check(cudaGetLastError(), "k_gout");
    c->backprop(batch, d_gx);
    c->check_err();
    if (host_grad) {
      cuda_check(cudaMemcpyAsync(host_grad, c->grad, c->nparam * sizeof(float), cudaMemcpyDeviceToHost, c->st),
                 "D2H");
      cuda_check(cudaStreamSynchronize(c->st), "sync");
    }
  } catch (const Error& e) {
    return fail(e);
  }
  return R2D3C_OK;
}

int r2d3c_cnn_train_step(r2d3c_cnn* c, const float* d_x, const float* d_y, int batch, float lr, double* loss) {
  try {
    if (!c || !d_x || !d_y) throw Error(kEINVAL, "NULL argument");
    if (batch < 1 || batch > c->Bmax) throw Error(kEINVAL, "batch out of range");
    c->forward(d_x, batch, true);
    const double l = c->backward(d_y, batch);
    c->adam(lr);
    c->check_err();
    if (loss) *loss = l;
  } catch (const Error& e) {
    return fail(e);
  }
  return R2D3C_OK;
}

}  // extern "C"

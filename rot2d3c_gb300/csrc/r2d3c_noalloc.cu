// Allocation-free 2-D complex-to-real transform (r2d3c_fft_c2r_noalloc).
//
// Some callers cannot allocate device memory: a host program whose device
// memory is entirely reserved by another allocator (a framework's caching
// pool, a fixed memory budget), or code paths where the implicit device
// synchronisation of cudaMalloc/cudaFree is not acceptable.  For them this
// file provides one variant of the FP64 C2R of r2d3c_fft_c2r_dev that uses
// no cudaMalloc, cudaFree or allocating library call: its scratch (the mixed
// plane between the column and the row pass) and its twiddle tables live in
// file-scope __device__ arrays of fixed size, held by every GPU that loads
// the library until the process exits.
//
// Limits and sharing rules:
//   - n <= kNoAllocMaxN (512); larger grids are rejected with R2D3C_EINVAL;
//   - all calls on one device share the same scratch array; calls whose GPU
//     work overlaps (different streams, or different host threads) race on
//     it, so callers must order them;
//   - the scratch keeps the previous call's contents; every element the
//     transform reads is written by the column pass of the same call first,
//     so nothing needs clearing;
//   - the first call on each device performs the set-up (twiddle upload with
//     cudaMemcpyToSymbol, a device synchronisation that makes the upload
//     complete before any stream of the caller can read it, and
//     cudaGetSymbolAddress of both arrays, with that device current); make
//     that first call before any stream capture.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/r2d3c.h"
#include "r2d3c_engine.h"
#include "r2d3c_kernels.cuh"

namespace r2d3c {
std::string& last_error_slot();
}

namespace {

using namespace r2d3c;

constexpr int kNoAllocMaxN = 512;
// mixed plane T[kx][y], (n/2+1) x n complex FP64, for the largest n
constexpr size_t kScratchElems = (size_t)(kNoAllocMaxN / 2 + 1) * kNoAllocMaxN;
// twiddle tables of every supported n <= 512, concatenated (16 + 32 + ... + 512)
constexpr int kTwElems = 2 * kNoAllocMaxN - 16;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double2 g_noalloc_scratch[kScratchElems];
static __device__ __align__(256) double2 g_noalloc_tw[kTwElems];

struct DevSlot {
  std::atomic<bool> ready{false};  // published (release) once the fields below are set
  double2* scratch = nullptr;  // device address of g_noalloc_scratch
  double2* tw = nullptr;       // device address of g_noalloc_tw
};
DevSlot g_slots[kMaxDevices];
std::mutex g_mu;

int tw_offset(int n) {  // start of the n-point table inside g_noalloc_tw
  int off = 0;
  for (int m = 16; m < n; m <<= 1) off += m;
  return off;
}

// The stage-major tables of the column and row kernels for one n, from the
// same FP64 roots as the engines' tables.
void host_twiddles(int n, double2* out) {
  std::vector<double> c(n), s(n);
  host_unit_roots(n, c.data(), s.data());
  switch (n) {
    case 16: build_stage_twiddles<double, 16, Cfg<double, 16>::E>(out, c.data(), s.data()); break;
    case 32: build_stage_twiddles<double, 32, Cfg<double, 32>::E>(out, c.data(), s.data()); break;
    case 64: build_stage_twiddles<double, 64, Cfg<double, 64>::E>(out, c.data(), s.data()); break;
    case 128: build_stage_twiddles<double, 128, Cfg<double, 128>::E>(out, c.data(), s.data()); break;
    case 256: build_stage_twiddles<double, 256, Cfg<double, 256>::E>(out, c.data(), s.data()); break;
    default: build_stage_twiddles<double, 512, Cfg<double, 512>::E>(out, c.data(), s.data()); break;
  }
}

// Per-device set-up, run by the first call on each device (with that device
// current).  The host names of the arrays are only stand-ins; the kernels get
// the device addresses returned by cudaGetSymbolAddress.
DevSlot& setup(int dev) {
  DevSlot& s = g_slots[dev];
  if (s.ready.load(std::memory_order_acquire)) return s;  // set-up done: no lock on the call path
  std::lock_guard<std::mutex> lk(g_mu);
  if (s.ready.load(std::memory_order_relaxed)) return s;
  std::vector<double2> h(kTwElems);
  for (int n = 16; n <= kNoAllocMaxN; n <<= 1) host_twiddles(n, h.data() + tw_offset(n));
  cuda_check(cudaMemcpyToSymbol(g_noalloc_tw, h.data(), sizeof(double2) * kTwElems),
             "cudaMemcpyToSymbol(no-alloc twiddles)");
  // A copy from pageable host memory may return before its DMA has landed,
  // and the kernels run on the caller's stream, which need not wait for the
  // legacy default stream (cudaStreamNonBlocking): finish the upload here.
  cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize(no-alloc set-up)");
  void* p = nullptr;
  cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
  s.scratch = static_cast<double2*>(p);
  p = nullptr;
  cuda_check(cudaGetSymbolAddress(&p, g_noalloc_tw), "cudaGetSymbolAddress(no-alloc twiddles)");
  s.tw = static_cast<double2*>(p);
  // the column and row kernels of every n use dynamic shared memory below 48 KB
  s.ready.store(true, std::memory_order_release);
  return s;
}

template <int N>
void launch(const double2* in, double* out, double2* scratch, const double2* tw, cudaStream_t st) {
  using C = Cfg<double, N, 1>;
  static_assert(C::SMEM <= 48 * 1024, "no-alloc sizes stay below the default shared-memory limit");
  k_colfft<double, N, +1><<<(N / 2 + 1 + C::G - 1) / C::G, C::THREADS, C::SMEM, st>>>(in, scratch, N / 2 + 1,
                                                                                      tw);
  cuda_check(cudaGetLastError(), "k_colfft (no-alloc)");
  k_rowc2r<double, N><<<(N / 2 + C::G - 1) / C::G, C::THREADS, C::SMEM, st>>>(scratch, out, nullptr, tw);
  cuda_check(cudaGetLastError(), "k_rowc2r (no-alloc)");
}

}  // namespace

extern "C" int r2d3c_fft_c2r_noalloc(int n, const double* d_in, double* d_out, void* stream) {
  try {
    if (!d_in || !d_out) throw Error(kEINVAL, "NULL argument");
    if (n < 16 || (n & (n - 1)) != 0)
      throw Error(kEINVAL, "n must be a power of two >= 16");
    if (n > kNoAllocMaxN)
      throw Error(kEINVAL, "n exceeds the allocation-free maximum of 512 (use r2d3c_fft_c2r_dev)");
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) throw Error(kEINVAL, "device index out of range");
    DevSlot& s = setup(dev);
    const double2* in = reinterpret_cast<const double2*>(d_in);
    const double2* tw = s.tw + tw_offset(n);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (n) {
      case 16: launch<16>(in, d_out, s.scratch, tw, st); break;
      case 32: launch<32>(in, d_out, s.scratch, tw, st); break;
      case 64: launch<64>(in, d_out, s.scratch, tw, st); break;
      case 128: launch<128>(in, d_out, s.scratch, tw, st); break;
      case 256: launch<256>(in, d_out, s.scratch, tw, st); break;
      default: launch<512>(in, d_out, s.scratch, tw, st); break;
    }
  } catch (const Error& e) {
    last_error_slot() = e.what();
    return e.code;
  } catch (const std::exception& e) {
    last_error_slot() = e.what();
    return R2D3C_EINVAL;
  }
  return R2D3C_OK;
}

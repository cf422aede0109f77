// One RK4 step of a small grid (n <= 512, one run) in a single launch: one
// thread-block cluster runs the twelve passes of the four substeps in turn
// (A, B, C per substep, plus the time step of the first), separated by
// cluster barriers (hardware barrier.cluster, no spin loop), with the mixed
// and bracket planes exchanged through L2.  At these sizes every pass is a
// few microseconds of latency-bound work, so the twelve launches of the
// separate-pass step and their gaps cost more than the work; the cluster
// spends only the barriers.  The passes are the same code as the separate
// kernels (r2d3c_pass_{a,b,c}.inc, here over virtual block indices), so the
// results are bit-identical; the plan autotuner times both forms.
#pragma once

#include <cooperative_groups.h>

#include "r2d3c_aux.cuh"

namespace r2d3c {

template <typename T, int N>
struct SmallStep {
  static constexpr int NT = PassNT<T, N>::value;
  using C = Cfg<T, N, NT>;
  static constexpr int TPF = C::TPF;
  static constexpr int THREADS = 256;
  static constexpr int G = THREADS / TPF;  // transform groups per CTA in every pass
  static constexpr int FA = 2;             // pass A: the six fields in two chunks
  static constexpr bool OK = N >= 32 && N <= 512 && THREADS % TPF == 0 && G >= 1 &&
                             CfgA<T, N>::TPF == TPF && PassAE<T, N>::value == C::E && PassSmem<T, N>::HOLD;
  static constexpr size_t SMEM = (size_t)G * PassSmem<T, N>::GROUP_ELEMS * sizeof(cpx<T>);
};

template <typename T>
struct SmallArgs {
  cpx<T>*ps, *vz, *c1, *c2, *c3, *c4, *tf, *pb;
  const cpx<T>*fp, *fz, *tau5, *tau6;
  const tw_t<T>*tw, *twa;
  const StepCoef* scs;
  double* scal;
  unsigned long long* enc;
  const CflCoef* cc;
  T inv_n4;
  int cfl_mode, add_time;
  DevGrid gd;
  Batch bs;
};

// the three pass bodies over a virtual block (x, z of nz), run 0, G groups
template <typename T, int N>
__device__ __forceinline__ void small_passA(const cpx<T>* __restrict__ ps, const cpx<T>* __restrict__ vz,
                                            cpx<T>* __restrict__ tf, DevGrid gd, const tw_t<T>* __restrict__ tw,
                                            Batch bs, int vbx, int vbz, int vbnz) {
  constexpr int EA = PassAE<T, N>::value;
#define R2D3C_VB_X vbx
#define R2D3C_VB_Y 0
#define R2D3C_VB_Z vbz
#define R2D3C_VB_NZ vbnz
#define R2D3C_VB_GPC (SmallStep<T, N>::G)
#include "r2d3c_pass_a.inc"
#undef R2D3C_VB_X
#undef R2D3C_VB_Y
#undef R2D3C_VB_Z
#undef R2D3C_VB_NZ
#undef R2D3C_VB_GPC
}

template <typename T, int N, bool CFL>
__device__ __forceinline__ void small_passB(const cpx<T>* __restrict__ tf, cpx<T>* __restrict__ pb, int kxo,
                                            DevGrid gd, T inv_n4, const tw_t<T>* __restrict__ tw,
                                            unsigned long long* __restrict__ cfl_enc, Batch bs, int vbx) {
#define R2D3C_VB_X vbx
#define R2D3C_VB_Y 0
#define R2D3C_VB_Z 0
#define R2D3C_VB_NZ 1
#define R2D3C_VB_GPC (SmallStep<T, N>::G)
#include "r2d3c_pass_b.inc"
#undef R2D3C_VB_X
#undef R2D3C_VB_Y
#undef R2D3C_VB_Z
#undef R2D3C_VB_NZ
#undef R2D3C_VB_GPC
}

template <typename T, int N>
__device__ __forceinline__ void small_passC(const cpx<T>* __restrict__ pb, const cpx<T>* c1in, const cpx<T>* c2in,
                                            const cpx<T>* ps, const cpx<T>* vz, const cpx<T>* __restrict__ fp,
                                            const cpx<T>* __restrict__ fz, cpx<T>* c1out, cpx<T>* c2out, DevGrid gd,
                                            const StepCoef* __restrict__ scs, const double* __restrict__ scal, int o,
                                            const tw_t<T>* __restrict__ tw, Batch bs, const cpx<T>* __restrict__ tau5,
                                            const cpx<T>* __restrict__ tau6, int vbx, int vbz, int vbnz) {
#define R2D3C_VB_X vbx
#define R2D3C_VB_Y 0
#define R2D3C_VB_Z vbz
#define R2D3C_VB_NZ vbnz
#define R2D3C_VB_GPC (SmallStep<T, N>::G)
#include "r2d3c_pass_c.inc"
#undef R2D3C_VB_X
#undef R2D3C_VB_Y
#undef R2D3C_VB_Z
#undef R2D3C_VB_NZ
#undef R2D3C_VB_GPC
}

// every CTA's global writes before the barrier are visible to every CTA
// after it (a device-scope fence, then the cluster's hardware barrier with
// its release / acquire semantics)
__device__ __forceinline__ void small_sync() {
  __threadfence();
  cooperative_groups::this_cluster().sync();
}

template <typename T, int N>
__global__ void __launch_bounds__(SmallStep<T, N>::THREADS, 1) k_step_small(SmallArgs<T> a) {
  using SS = SmallStep<T, N>;
  constexpr int NT = SS::NT;
  const auto cl = cooperative_groups::this_cluster();
  const int rank = (int)cl.block_rank(), ncl = (int)cl.num_blocks();
  const DevGrid gd = a.gd;
  const int nxC = ((gd.M + NT - 1) / NT + SS::G - 1) / SS::G;  // virtual CTAs over the column pairs
  const int nxB = (N / NT + SS::G - 1) / SS::G;                // and over the row pairs
  constexpr int NZC = kChunkC<T, N> ? 2 : 1;                   // pass C: C1 and C2 updates apart
  if (a.cfl_mode && rank == 0 && threadIdx.x == 0) a.enc[0] = 0ull;  // visible after the first barrier
  for (int o = 4; o >= 1; --o) {
    // the substep state: ps -> C1 -> C3 -> C1 -> ps (vz -> C2 -> C4 -> C2 -> vz), as the separate passes
    const cpx<T>* in1 = o == 4 ? a.ps : o == 2 ? a.c3 : a.c1;
    const cpx<T>* in2 = o == 4 ? a.vz : o == 2 ? a.c4 : a.c2;
    cpx<T>* out1 = o == 1 ? a.ps : o == 3 ? a.c3 : a.c1;
    cpx<T>* out2 = o == 1 ? a.vz : o == 3 ? a.c4 : a.c2;
    for (int t = rank; t < nxC * SS::FA; t += ncl)
      small_passA<T, N>(in1, in2, a.tf, gd, a.twa, a.bs, t % nxC, t / nxC, SS::FA);
    small_sync();
    for (int t = rank; t < nxB; t += ncl) {
      if (o == 4 && a.cfl_mode) small_passB<T, N, true>(a.tf, a.pb, gd.M, gd, a.inv_n4, a.tw, a.enc, a.bs, t);
      else small_passB<T, N, false>(a.tf, a.pb, gd.M, gd, a.inv_n4, a.tw, a.enc, a.bs, t);
    }
    small_sync();
    if (o == 4 && (a.cfl_mode || a.add_time)) {
      if (rank == 0 && threadIdx.x == 0) {
        if (a.cfl_mode) cfl_dt_one(a.enc, a.cc[0], a.scal, a.add_time);
        else a.scal[1] = __dadd_rn(a.scal[1], a.scal[0]);  // time += dt (k_add_time)
      }
      small_sync();
    }
    for (int t = rank; t < nxC * NZC; t += ncl)
      small_passC<T, N>(a.pb, in1, in2, a.ps, a.vz, a.fp, a.fz, out1, out2, gd, a.scs, a.scal, o, a.tw, a.bs, a.tau5,
                        a.tau6, t % nxC, t / nxC, NZC);
    small_sync();
  }
}

}  // namespace r2d3c

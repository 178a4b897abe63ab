#pragma once
// Degree-specialised FP32 stage kernel: fused DG right-hand side + LSRK stage (implementation;
// the variants are instantiated in bbdg_stage_fast_v*.cu and registered in bbdg_stage_fast.cu).
//
// Same algorithm and data layout as the generic stage kernel (bbdg_solver.cu) with the
// degree N a compile-time constant, which turns every multi-index computation into an
// immediate and lets one thread run a whole face lift chain in registers:
//
//   lift, per face f and chain c (src/BernsteinLift.jl:139-164):
//     E0 = L0 x,  L0 = (N+1)^2/2 R_{N+1} E_{N->N+1}, applied as its 7-point stencil
//         L0 x(i,j) = 1/2 [((i+1)^2+(j+1)^2+(k+1)^2) x(i,j) + (i+1) j x(i+1,j-1)
//                          + (i+1) k x(i+1,j) + (j+1) i x(i-1,j+1) + (j+1) k x(i,j+1)
//                          + (k+1) i x(i-1,j) + (k+1) j x(i,j-1)],   k = N-i-j
//     E_d = R_{N-d+1} E_{d-1}, all in registers; the face's volume stack holds E_d at layer d
//   the four face stacks are summed, with the l_d weights, through the permutations of
//   src/BernsteinLift.jl:207-218 by one thread per volume coefficient, together with the
//   volume term and the LSRK update.
//
// Wave (examples/3d_wave.jl:45-54): with affine elements the scaled normal n is constant on
// a face, so the u, v, w fluxes are B n_x, B n_y, B n_z with B = (cu n.du - dp)/2: two chains
// per face (A = (cp dp - n.du)/2 and B) instead of four.
// Maxwell (examples/3d_maxwell.jl:43-65): six flux components, six chains per face.
//
// Block organisation: EPB elements per tile; TPE "element threads" per element plus
// CHT "chain threads" (whole warps, one lift chain each). Tiles stream through a persistent
// loop in two phases: (A) the chain warp lifts tile i while the element threads form the
// volume term of tile i and the interface flux of tile i+1 (double-buffered chain inputs);
// (B) the element threads gather the lift stacks, add the volume term and apply the LSRK
// update, storing q, res and the outgoing face traces straight to HBM. q, geometry and
// connectivity of tile i+2 and res of tile i+1 arrive by bulk copies (cp.async.bulk,
// mbarrier completion, bounded waits) while tiles i and i+1 are being worked on.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <vector>

#include "bbdg_internal.cuh"
#include "bbdg_stack_slots.cuh"
#include "bbdg_stage_fast.cuh"

namespace bbfast {

__host__ __device__ constexpr int c_tri(int n, int j) { return j * (2 * n + 3 - j) / 2; }
__host__ __device__ constexpr int c_tet(int n, int k) {
  return ((n + 1) * (n + 2) * (n + 3) - (n + 1 - k) * (n + 2 - k) * (n + 3 - k)) / 6;
}
__host__ __device__ constexpr int c_ij(int n, int i, int j) { return i + c_tri(n, j); }
__host__ __device__ constexpr int c_ijk(int n, int i, int j, int k) {
  return i + c_tri(n, j) + c_tet(n, k) - j * k;
}
template <int PHYS>
struct FPhys;
template <>
struct FPhys<BB_WAVE> {
  static constexpr int NF = 4, NCH = 2, NW = 4;
};
template <>
struct FPhys<BB_MAXWELL> {
  static constexpr int NF = 6, NCH = 6, NW = 6;
};

template <int N, int PHYS, int EPB, int TPE>
struct FastLayout {
  static constexpr int NP = (N + 1) * (N + 2) * (N + 3) / 6;
  static constexpr int NFP = (N + 1) * (N + 2) / 2;
  static constexpr int NPM1 = N * (N + 1) * (N + 2) / 6;
  static constexpr int NF = FPhys<PHYS>::NF, NCH = FPhys<PHYS>::NCH, NW = FPhys<PHYS>::NW;
  static constexpr int NCHAIN = EPB * 4 * NCH;
  static constexpr int CHT = (NCHAIN + 31) / 32 * 32;  // chain threads, whole warps
  static constexpr int NTE = EPB * TPE;                // element threads
  static constexpr int NT = NTE + CHT;
  // chain stacks: element-face e4 = element * 4 + face holds its NCH chains interleaved,
  // stack entry q of chain ch at ((e4 * NPS + stack_slot<N>(q)) * NCH + ch). NPS = 1 mod 16
  // puts the same slot of the 32 chains of a warp (consecutive e4 and ch) in 32 different
  // banks for NCH = 2 and 6; the slots spread the gather's reads over the banks.
  static constexpr int NSLOT = StackSlots<N>::span > NP ? StackSlots<N>::span : NP;
  static constexpr int NPS = (NSLOT + 14) / 16 * 16 + 1;
  // w(beta) rows: NPM1 entries, then NZ zero entries from Z0 (a multiple of 8) on, one per bank
  // group of the gather's vector loads (16-byte entries: 8 lanes per phase, 8 groups; 24-byte
  // entries: 16 lanes per phase, bank pair 3 x mod 16); a coefficient with alpha_b = 0 reads the
  // zero entry whose group no other lane of its phase reads, so the zero never conflicts
  static constexpr int Z0 = (NPM1 + 7) / 8 * 8;
  static constexpr int NZ = NW == 4 ? 8 : 16;
  static constexpr int NPM1P = Z0 + NZ;
  // bytes; every bulk-copy destination starts on a 16-byte boundary
  static constexpr int QBYTES = NF * EPB * NP * 4;            // q tile, [NF][EPB][NP]
  static constexpr int GEOBYTES = EPB * BB_GEO_STRIDE * 4;     // [EPB][24]
  static constexpr int CONNBYTES = EPB * 16;                   // [EPB][4] int32
  static constexpr int SLOT = ((QBYTES + GEOBYTES + CONNBYTES) + 15) / 16 * 16;
  static constexpr int RES_B = 2 * SLOT;                       // after the two q slots
  static constexpr int G_B = RES_B + QBYTES;                   // [EPB*4][NPS][NCH] face stacks
  static constexpr int X_B = G_B + (NCHAIN * NPS * 4 + 15) / 16 * 16;  // [2][NCHAIN][NFP]
  static constexpr int W_B = X_B + (2 * NCHAIN * NFP * 4 + 15) / 16 * 16;  // [EPB][NPM1P][NW]
  static constexpr int GA_B = W_B + (NW * EPB * NPM1P * 4 + 15) / 16 * 16;  // [NP] uint4
  static constexpr int VN_B = GA_B + NP * 16;                  // [NPM1] uint2
  static constexpr int FVOL_B = VN_B + NPM1 * 8;               // [4][NFP] u16
  static constexpr int FPERM_B = FVOL_B + ((4 * NFP * 2 + 3) / 4 * 4);  // [6][NFP] u16
  static constexpr int FNB_B = FPERM_B + ((6 * NFP * 2 + 3) / 4 * 4);  // [4][6][NFP] u16
  static constexpr int TF_B = (FNB_B + 24 * NFP * 2 + 15) / 16 * 16;   // [NP] u32 face nodes
  static constexpr int BAR_B = (TF_B + NP * 4 + 15) / 16 * 16;         // 3 mbarriers
  static constexpr int BYTES = BAR_B + 32;
  // element groups for the named-barrier hand-offs between the chain warps and the element
  // threads: GS elements per group, NG groups, two barriers per group (ids 1..2 NG)
  static constexpr int GS = EPB <= 7 ? 1 : (EPB + 6) / 7;
  static constexpr int NG = EPB / GS;
  static constexpr int GCOUNT = GS * TPE + CHT;  // threads at each hand-off
  static_assert(EPB % GS == 0 && 2 * NG <= 15, "named barriers 1..15 cover the groups");
  // resident blocks per SM the register budget is sized for (2 when two tiles fit in the
  // shared memory of an SM, else 1)
  static constexpr int MINB = 2 * BYTES <= 227 * 1024 ? 2 : 1;
  static_assert((EPB * NP * 4) % 16 == 0, "tile segments must be multiples of 16 bytes");
  static_assert(NFP < 255, "face node indices are packed in bytes");
  static_assert(NPM1P <= 1024 && NPS <= 1024, "w indices and stack slots fit the packed table");
  static_assert(TPE % 32 == 0 && TPE >= 32, "element threads come in whole warps");
};

// ---- bulk copies and mbarriers (inline PTX) -----------------------------------------
__device__ __forceinline__ uint32_t s_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(s_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Named hardware barriers (ids 1..15; id 0 is __syncthreads): bar.sync waits until `count`
// threads have arrived, bar.arrive counts the caller without waiting. Both are executed by
// whole warps.
__device__ __forceinline__ void nbar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void nbar_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// Bounded wait for the phase with the given parity: `limit` polls (2^24, about a second, by
// default), then false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    if (mbar_test(bar, parity)) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tma_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          s_addr(dst)),
      "l"(src), "r"(bytes), "r"(s_addr(bar))
      : "memory");
}
// Asks the memory system to bring [src, src + bytes) into L2 (no completion to wait for).
__device__ __forceinline__ void l2_prefetch(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// One face lift chain for compile-time N: x = chain input (NFP values, smem); g = the face's
// volume stack with entries NCH apart, g[stack_slot<N>(c_ijk(N,i,j,d)) * NCH] = F_d(i,j) =
// l_d E_d(i,j) (slots fold to immediates: the loops are unrolled). The
// chain carries F_d itself: l_d / l_{d-1} = -(N-d+1)/(d+1) and R_{N-d+1} divides by N-d+1, so
// F_d = -1/(d+1) [(i+1) F_{d-1}(i+1,j) + (j+1) F_{d-1}(i,j+1) + (N-d+1-i-j) F_{d-1}(i,j)]
// (F_0 = E_0 = L0 x). All of x is read before g is written.
template <int N, int NCH>
__device__ __forceinline__ void lift_chain(const float* x, float* g) {
  constexpr int NFP = (N + 1) * (N + 2) / 2;
  float X[NFP];
#pragma unroll
  for (int m = 0; m < NFP; ++m) X[m] = x[m];
  float E[NFP];
#pragma unroll
  for (int j = 0; j <= N; ++j) {
#pragma unroll
    for (int i = 0; i + j <= N; ++i) {
      const int k = N - i - j;
      float v = float((i + 1) * (i + 1) + (j + 1) * (j + 1) + (k + 1) * (k + 1)) * X[c_ij(N, i, j)];
      if (j > 0) v = fmaf(float((i + 1) * j), X[c_ij(N, i + 1, j - 1)], v);
      if (k > 0) v = fmaf(float((i + 1) * k), X[c_ij(N, i + 1, j)], v);
      if (i > 0) v = fmaf(float((j + 1) * i), X[c_ij(N, i - 1, j + 1)], v);
      if (k > 0) v = fmaf(float((j + 1) * k), X[c_ij(N, i, j + 1)], v);
      if (i > 0) v = fmaf(float((k + 1) * i), X[c_ij(N, i - 1, j)], v);
      if (j > 0) v = fmaf(float((k + 1) * j), X[c_ij(N, i, j - 1)], v);
      E[c_ij(N, i, j)] = 0.5f * v;
    }
  }
#pragma unroll
  for (int m = 0; m < NFP; ++m) g[stack_slot<N>(m) * NCH] = E[m];  // layer 0 (c_ijk(N,i,j,0) = c_ij(N,i,j))
#pragma unroll
  for (int d = 1; d <= N; ++d) {
    const int n = N - d + 1;  // input degree; E indexed with the degree-N layout
    const float inv = -1.0f / float(d + 1);
#pragma unroll
    for (int j = 0; j < n; ++j) {
#pragma unroll
      for (int i = 0; i + j < n; ++i) {
        // reduction_multiply! (src/BernsteinLift.jl:81-85) times l_d / l_{d-1}, in place in
        // ascending order
        const float v = float(i + 1) * inv * E[c_ij(N, i + 1, j)] +
                        (float(j + 1) * inv * E[c_ij(N, i, j + 1)] +
                         float(n - i - j) * inv * E[c_ij(N, i, j)]);
        E[c_ij(N, i, j)] = v;
        g[stack_slot<N>(c_ijk(N, i, j, d)) * NCH] = v;
      }
    }
  }
}

template <int N, int PHYS, int EPB, int TPE>
__global__ void __launch_bounds__(FastLayout<N, PHYS, EPB, TPE>::NT,
                                  FastLayout<N, PHYS, EPB, TPE>::MINB)
    stage_fast_kernel(FastStageParams P) {
  using L = FastLayout<N, PHYS, EPB, TPE>;
  constexpr int NP = L::NP, NFP = L::NFP, NPM1 = L::NPM1, NF = L::NF, NCH = L::NCH;
  constexpr int NPS = L::NPS, NCHAIN = L::NCHAIN, NW = L::NW, NTE = L::NTE, NT = L::NT;
  constexpr int NZ_W = EPB * L::NZ * NW;  // zero-entry floats of all elements
  constexpr int FT = TPE / 4;                     // element threads per face
  constexpr int FR = (NFP + FT - 1) / FT;         // face nodes per element thread
  constexpr int VR = (NPM1 + TPE - 1) / TPE;      // degree N-1 points per element thread
  constexpr int GR = (NP + TPE - 1) / TPE;        // coefficients per element thread
  extern __shared__ __align__(16) unsigned char smem[];
  float* sRes = reinterpret_cast<float*>(smem + L::RES_B);
  float* sG = reinterpret_cast<float*>(smem + L::G_B);
  float* sX = reinterpret_cast<float*>(smem + L::X_B);  // chain inputs, two tiles
  float* sW = reinterpret_cast<float*>(smem + L::W_B);
  // per coefficient alpha: degree N-1 indices of alpha - e_b (NPM1 = zero entry when
  // alpha_b = 0) and face-stack positions; alpha_b; l_d of its layer on each face
  uint4* sGA = reinterpret_cast<uint4*>(smem + L::GA_B);
  uint2* sVN = reinterpret_cast<uint2*>(smem + L::VN_B);  // beta -> indices of beta + e_a
  uint16_t* sFvol = reinterpret_cast<uint16_t*>(smem + L::FVOL_B);
  uint16_t* sFperm = reinterpret_cast<uint16_t*>(smem + L::FPERM_B);
  // partner face nf, orientation o, node a -> volume index of the partner's node
  uint16_t* sFnb = reinterpret_cast<uint16_t*>(smem + L::FNB_B);
  // per coefficient: its node index on faces f0..f3 (one byte each, 0xff = not on the face)
  uint32_t* sTF = reinterpret_cast<uint32_t*>(smem + L::TF_B);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::BAR_B);  // [0],[1] q slots, [2] res
  __shared__ int s_fail;
  const int tid = threadIdx.x;
  const int64_t K = P.K;
  // this launch's tiles end at ntiles (the host guarantees K % EPB == 0)
  const int64_t ntiles = P.tile_end > 0 ? P.tile_end : K / EPB;
  const uint32_t wlim = P.wait_iters ? P.wait_iters : (1u << 24);
  const bool stage = P.mode != 0;
  // element threads: element le, lane u within the element
  const int le = tid / TPE, u = tid - (tid / TPE) * TPE;
  const bool is_elem = tid < NTE;

  auto slot_q = [](int s) { return reinterpret_cast<float*>(smem + s * L::SLOT); };
  auto slot_geo = [](int s) { return reinterpret_cast<float*>(smem + s * L::SLOT + L::QBYTES); };
  auto slot_conn = [](int s) {
    return reinterpret_cast<int32_t*>(smem + s * L::SLOT + L::QBYTES + L::GEOBYTES);
  };
  const float* gq = P.q;
  const float* gres = P.res;
  const float* ggeo = P.geo;
  const int32_t* gconn = P.conn;
  // tile t's q, geometry and connectivity -> slot s (thread 0 only). With `leave_out` (the
  // test-only fault mode) the slot's barrier is armed but the copies are not issued, so that
  // phase never completes and the bounded waits on it run out.
  auto issue_main = [=](int64_t t, int s, bool leave_out = false) {
    const int64_t e0 = t * EPB;
    mbar_expect_tx(&bar[s], L::QBYTES + L::GEOBYTES + L::CONNBYTES);
    if (leave_out) return;
#pragma unroll
    for (int m = 0; m < NF; ++m)
      tma_load(slot_q(s) + m * EPB * NP, gq + ((size_t)m * K + e0) * NP, EPB * NP * 4, &bar[s]);
    tma_load(slot_geo(s), ggeo + e0 * BB_GEO_STRIDE, L::GEOBYTES, &bar[s]);
    tma_load(slot_conn(s), gconn + e0 * 4, L::CONNBYTES, &bar[s]);
  };
  // tile t's q, geometry, connectivity and res -> L2, two tiles before they are copied in
  auto prefetch_tile = [=](int64_t t) {
    const int64_t e0 = t * EPB;
#pragma unroll
    for (int m = 0; m < NF; ++m) {
      l2_prefetch(gq + ((size_t)m * K + e0) * NP, EPB * NP * 4);
      if (stage) l2_prefetch(gres + ((size_t)m * K + e0) * NP, EPB * NP * 4);
    }
    l2_prefetch(ggeo + e0 * BB_GEO_STRIDE, L::GEOBYTES);
    l2_prefetch(gconn + e0 * 4, L::CONNBYTES);
  };
  auto issue_res = [=](int64_t t) {
    const int64_t e0 = t * EPB;
    mbar_expect_tx(&bar[2], L::QBYTES);
#pragma unroll
    for (int m = 0; m < NF; ++m)
      tma_load(sRes + m * EPB * NP, gres + ((size_t)m * K + e0) * NP, EPB * NP * 4, &bar[2]);
  };

  if (tid == 0) {
    s_fail = 0;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_async_smem();
  }
  // constant tables (built from the degree tables in global memory)
  {
    const uint32_t* gw = P.gtab;
    // w index of alpha - e_b, or -1 when alpha_b = 0
    auto wnb = [&](int n, int b) {
      const uint32_t c = gw[P.o_node3 + n];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16, l = N - i - j - k;
      const int ab = b == 0 ? i : b == 1 ? j : b == 2 ? k : l;
      if (ab == 0) return -1;
      return ijk3(N - 1, i - (b == 0), j - (b == 1), k - (b == 2));
    };
    auto group_of = [](int x) { return NW == 4 ? (x & 7) : ((3 * x) & 15); };
    for (int t = tid; t < NP; t += NT) {
      const uint32_t c = gw[P.o_node3 + t];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16, l = N - i - j - k;
      uint32_t mb[4];
      const int lane = (t % TPE) & 31, phase = L::NZ;  // lanes of one vector-load phase
      const int n0 = t - (lane % phase);
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int x = wnb(t, b);
        if (x >= 0) {
          mb[b] = (uint32_t)x;
          continue;
        }
        uint32_t used = 0;
        for (int q = 0; q < phase; ++q) {
          const int nq = n0 + q;
          if (nq >= NP || (nq % TPE) / 32 != (t % TPE) / 32) continue;
          const int xq = wnb(nq, b);
          if (xq >= 0) used |= 1u << group_of(xq);
        }
        int zs = 0;
        while (zs < L::NZ - 1 && ((used >> group_of(L::Z0 + zs)) & 1u)) ++zs;
        mb[b] = (uint32_t)(L::Z0 + zs);
      }
      // stack slots of this coefficient on faces f0 (i,k,j), f1 (j,k,l), f2 (j,k,i), f3 (i,j,k)
      // (the slot map is in the degree tables: no switch in the kernel's set-up code)
      const uint16_t* gs = reinterpret_cast<const uint16_t*>(gw + P.o_sslot);
      const uint32_t p0 = gs[ijk3(N, i, k, j)], p1 = gs[ijk3(N, j, k, l)];
      const uint32_t p2 = gs[ijk3(N, j, k, i)], p3 = gs[t];
      // 10-bit fields: .x w indices of alpha - e_b for b = 0..2, .y stack slots on f0..f2,
      // .w stack slot on f3 and the w index for b = 3; .z alpha's barycentric indices
      // (i, j, k, l), one byte each
      sGA[t] = make_uint4(mb[0] | (mb[1] << 10) | (mb[2] << 20), p0 | (p1 << 10) | (p2 << 20),
                          (uint32_t)i | ((uint32_t)j << 8) | ((uint32_t)k << 16) | ((uint32_t)l << 24),
                          p3 | (mb[3] << 10));
      // face nodes: f0 (j=0) at (i,k), f1 (l=0) at (j,k), f2 (i=0) at (j,k), f3 (k=0) at (i,j)
      const uint32_t a0 = j == 0 ? (uint32_t)ij2(N, i, k) : 0xffu;
      const uint32_t a1 = l == 0 ? (uint32_t)ij2(N, j, k) : 0xffu;
      const uint32_t a2 = i == 0 ? (uint32_t)ij2(N, j, k) : 0xffu;
      const uint32_t a3 = k == 0 ? (uint32_t)ij2(N, i, j) : 0xffu;
      sTF[t] = a0 | (a1 << 8) | (a2 << 16) | (a3 << 24);
    }
    for (int t = tid; t < NPM1; t += NT) {
      const uint32_t c = gw[P.o_node3m1 + t];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16;
      sVN[t] = make_uint2(ijk3(N, i + 1, j, k) | (ijk3(N, i, j + 1, k) << 16),
                          ijk3(N, i, j, k + 1) | (ijk3(N, i, j, k) << 16));
    }
    for (int t = tid; t < NZ_W; t += NT)
      sW[((t / (L::NZ * NW)) * L::NPM1P + L::Z0 + (t / NW) % L::NZ) * NW + t % NW] = 0.f;
    const uint16_t* gf = reinterpret_cast<const uint16_t*>(gw + P.o_fvol);
    for (int t = tid; t < 4 * NFP; t += NT) sFvol[t] = gf[t];
    const uint16_t* gp = reinterpret_cast<const uint16_t*>(gw + P.o_fperm);
    for (int t = tid; t < 6 * NFP; t += NT) sFperm[t] = gp[t];
    for (int t = tid; t < 24 * NFP; t += NT) {
      const int fo = t / NFP, a = t - fo * NFP;
      const uint16_t* gfv = reinterpret_cast<const uint16_t*>(gw + P.o_fvol);
      sFnb[t] = gfv[(fo / 6) * NFP + gp[(fo % 6) * NFP + a]];
    }
  }
  __syncthreads();
  // the first two tiles of this block go to the two slots; the first chain thread issues
  // every bulk copy and counts them per barrier (for the drain at the end)
  const int64_t t0 = P.tile_begin + blockIdx.x;
  const bool issuer = tid == NTE;
  uint32_t iss0 = 0u, iss1 = 0u, iss2 = 0u;
  if (issuer && t0 < ntiles) {
    issue_main(t0, 0);
    ++iss0;
    if (stage) issue_res(t0), ++iss2;
    if (t0 + gridDim.x < ntiles) issue_main(t0 + gridDim.x, 1), ++iss1;
    if (t0 + 2 * (int64_t)gridDim.x < ntiles) prefetch_tile(t0 + 2 * (int64_t)gridDim.x);
  }
  uint32_t ph = 0u;  // bit b: parity of the phase barrier b waits for next (element threads)
  const float rkA = P.rkA, rkB = P.rkB, dt = P.dt, tau = P.tau;
  // face handled by this element thread in the flux and trace phases
  const int ff = u / FT, fa0 = u - (u / FT) * FT;

  // interface flux of face ff of element le of tile t (q in slot s) -> chain inputs xbuf
  auto flux_tile = [&](int64_t t, int s, float* xbuf) {
    const int64_t e0 = t * EPB;
    const float* sQ = slot_q(s);
    const float* sGeo = slot_geo(s);
    const int32_t* sConn = slot_conn(s);
    const int32_t c = sConn[le * 4 + ff];
    const int64_t nbr = (int64_t)((uint32_t)c >> 5);
    const int nface = (c >> 3) & 3, o = c & 7;
    const bool bad = nbr >= K || o > 5;
    const bool inside = nbr >= e0 && nbr < e0 + EPB;
    if (bad && fa0 == 0) atomicOr(P.status, 1);
    const float* g = sGeo + le * BB_GEO_STRIDE;
    const float nx = g[12 + ff], ny = g[16 + ff], nz = g[20 + ff];
    float cp = 1.f, cu = 1.f;
    if (tau > 0.f) {
      const float n2 = nx * nx + ny * ny + nz * nz;
      const float rJf = rsqrtf(n2);
      cp = tau * n2 * rJf;  // tau |n|
      cu = tau * rJf;       // tau / |n|
    }
    // outside-tile neighbour traces: issue every global load before using any
    float tr[FR][NF];
    const float* tbase = P.trace_in + ((size_t)(bad ? 0 : nbr) * 4 + nface) * NF * NFP;
#pragma unroll
    for (int r = 0; r < FR; ++r) {
      const int a = fa0 + r * FT;
      if (a < NFP && !inside && !bad && BB_DCHECK(sFperm[o * NFP + a] < NFP, P.status)) {
        const float* tp = tbase + sFperm[o * NFP + a];
#pragma unroll
        for (int m = 0; m < NF; ++m) tr[r][m] = __ldg(tp + m * NFP);
      }
    }
    const int pin = (int)(nbr - e0);
    float* xin0 = xbuf + ((le * 4 + ff) * NCH) * NFP;
#pragma unroll
    for (int r = 0; r < FR; ++r) {
      const int a = fa0 + r * FT;
      if (a >= NFP) continue;
      float d[NF];
      const float* qM = sQ + le * NP + sFvol[ff * NFP + a];
      // debug builds: every table-derived node index in range (else the node's jump is 0)
      const bool dbad =
          !BB_DCHECK(sFvol[ff * NFP + a] < NP &&
                         (inside ? sFnb[(nface * 6 + o) * NFP + a] < NP
                                 : sFperm[o * NFP + a] < NFP),
                     P.status);
      if (bad || dbad) {
#pragma unroll
        for (int m = 0; m < NF; ++m) d[m] = 0.f;
      } else if (inside) {
        const float* qP = sQ + pin * NP + sFnb[(nface * 6 + o) * NFP + a];
#pragma unroll
        for (int m = 0; m < NF; ++m) d[m] = qP[m * EPB * NP] - qM[m * EPB * NP];
      } else {
#pragma unroll
        for (int m = 0; m < NF; ++m) d[m] = tr[r][m] - qM[m * EPB * NP];
      }
      float* xin = xin0 + a;
      if constexpr (PHYS == BB_WAVE) {
        const float ndotdU = nx * d[1] + ny * d[2] + nz * d[3];
        xin[0] = 0.5f * (cp * d[0] - ndotdU);    // p flux
        xin[NFP] = 0.5f * (cu * ndotdU - d[0]);  // (u,v,w) flux / n
      } else {
        const float Hx = d[0], Hy = d[1], Hz = d[2], Ex = d[3], Ey = d[4], Ez = d[5];
        const float ndH = nx * Hx + ny * Hy + nz * Hz;
        const float ndE = nx * Ex + ny * Ey + nz * Ez;
        const float ax[6] = {0.f, Ez, -Ey, 0.f, -Hz, Hy};
        const float ay[6] = {-Ez, 0.f, Ex, Hz, 0.f, -Hx};
        const float az[6] = {Ey, -Ex, 0.f, -Hy, Hx, 0.f};
        const float nd[6] = {ndH * nx, ndH * ny, ndH * nz, ndE * nx, ndE * ny, ndE * nz};
#pragma unroll
        for (int m = 0; m < 6; ++m)
          xin[m * NFP] = 0.5f * ax[m] * nx + 0.5f * ay[m] * ny + 0.5f * az[m] * nz +
                         0.5f * (cp * d[m]) - 0.5f * (cu * nd[m]);
      }
    }
  };

  // prologue: flux of the first tile
  if (is_elem && t0 < ntiles) {
    if (!mbar_wait(&bar[0], 0u, wlim)) {
      s_fail = 1;
      atomicOr(P.status, 2);
    }
    ph ^= 1u;
    flux_tile(t0, 0, sX);
  }
  __syncthreads();

  // Hand-offs per tile (every thread runs the same barrier sequence in every iteration, also
  // after a failure, when the work is skipped; so no barrier can wait for a thread that left):
  //   B->A, at the start of tile i > 0: each element group's threads and the chain warps sync
  //     on the group's barrier 1 + NG + g: the group has finished tile i-1 (its w may be
  //     rewritten), and once the chain warps have passed all groups, the stacks, slot s^1 and
  //     the res buffer are free and tile i's chain inputs are written;
  //   A->B: the chain warps arrive on barrier 1 + g after the lifts of tile i, the group's
  //     threads sync on it after forming w and the next tile's flux.
  constexpr int GCOUNT = L::GCOUNT, NG = L::NG;
  const int grp = le / L::GS;
  volatile int* vfail = &s_fail;
  int it = 0;
  for (int64_t tile = t0; tile < ntiles; tile += gridDim.x, ++it) {
    const int s = it & 1;
    const int64_t e0 = tile * EPB;
    const int64_t tnext = tile + gridDim.x;
    float* sQ = slot_q(s);
    const float* sGeo = slot_geo(s);
    const int32_t* sConn = slot_conn(s);

    // ---- A. chain warps: lift chains of this tile || element threads: volume term of
    //         this tile, then the interface flux of the next tile -------------------------
    if (!is_elem) {
      if (it > 0) {
        for (int g = 0; g < NG; ++g) nbar_sync(1 + NG + g, GCOUNT);
        if (issuer && !*vfail && (tnext < ntiles || stage)) {
          fence_async_smem();  // order the generic-proxy reads before the copies
          if (tnext < ntiles) {
            issue_main(tnext, s ^ 1, P.fault == 1 && it == 1);
            if (s) ++iss0;
            else ++iss1;
          }
          if (stage) issue_res(tile), ++iss2;
          if (tnext + gridDim.x < ntiles) prefetch_tile(tnext + gridDim.x);
        }
      }
      const int c = tid - NTE;
      if (!*vfail && c < NCHAIN)
        lift_chain<N, NCH>(sX + (s * NCHAIN + c) * NFP, sG + (c / NCH) * NPS * NCH + c % NCH);
      for (int g = 0; g < NG; ++g) nbar_arrive(1 + g, GCOUNT);
    } else if (it > 0 && (nbar_sync(1 + NG + grp, GCOUNT), *vfail)) {
      // a wait ran out: keep to the barrier sequence, skip the work
    } else {
      // the tile after next: its outside-tile neighbour traces (one contiguous NF x Nfp block
      // per face) are pulled into L2 now, a whole tile ahead of its flux phase
      const int64_t tpre = tnext + gridDim.x;
      int32_t cpre = 0;
      const bool pre = fa0 == 0 && tpre < ntiles && P.trace_in != nullptr;
      if (pre) cpre = __ldg(gconn + (tpre * EPB + le) * 4 + ff);
      const float* g = sGeo + le * BB_GEO_STRIDE;
      // barycentric weights of J d/dx, J d/dy, J d/dz: g_a = (rxJ, sxJ, txJ, -sum)/2; the
      // sum over a is formed as sum_{a<3} g_a (x_a - x_3), which cancels smooth data
      const float gx[3] = {0.5f * g[0], 0.5f * g[1], 0.5f * g[2]};
      const float gy[3] = {0.5f * g[3], 0.5f * g[4], 0.5f * g[5]};
      const float gz[3] = {0.5f * g[6], 0.5f * g[7], 0.5f * g[8]};
      const float* q0 = sQ + le * NP;
      // w(beta) at degree N-1; vol(alpha) = sum_b alpha_b w(alpha - e_b) is formed in B
#pragma unroll
      for (int r = 0; r < VR; ++r) {
        const int vg = r * (TPE / 32) + (u >> 5), lane = u & 31;
        if (lane >= P.vlen[vg]) continue;
        const int b = P.vstart[vg] + lane;
        const uint2 vn = sVN[b];
        const int idx[4] = {(int)(vn.x & 0xffff), (int)(vn.x >> 16), (int)(vn.y & 0xffff),
                            (int)(vn.y >> 16)};
        float w[NW];
#pragma unroll
        for (int m = 0; m < NW; ++m) w[m] = 0.f;
        if constexpr (PHYS == BB_WAVE) {
          const float p3 = q0[idx[3]], u3 = q0[EPB * NP + idx[3]], v3 = q0[2 * EPB * NP + idx[3]],
                      w3 = q0[3 * EPB * NP + idx[3]];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float p = q0[idx[a]] - p3, uu = q0[EPB * NP + idx[a]] - u3,
                        v = q0[2 * EPB * NP + idx[a]] - v3, ww = q0[3 * EPB * NP + idx[a]] - w3;
            w[0] += gx[a] * uu + gy[a] * v + gz[a] * ww;
            w[1] += gx[a] * p;
            w[2] += gy[a] * p;
            w[3] += gz[a] * p;
          }
        } else {
          float x3[6];
#pragma unroll
          for (int m = 0; m < 6; ++m) x3[m] = q0[m * EPB * NP + idx[3]];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float Hx = q0[idx[a]] - x3[0], Hy = q0[EPB * NP + idx[a]] - x3[1],
                        Hz = q0[2 * EPB * NP + idx[a]] - x3[2];
            const float Ex = q0[3 * EPB * NP + idx[a]] - x3[3],
                        Ey = q0[4 * EPB * NP + idx[a]] - x3[4],
                        Ez = q0[5 * EPB * NP + idx[a]] - x3[5];
            w[0] += -gy[a] * Ez + gz[a] * Ey;
            w[1] += gx[a] * Ez - gz[a] * Ex;
            w[2] += -gx[a] * Ey + gy[a] * Ex;
            w[3] += gy[a] * Hz - gz[a] * Hy;
            w[4] += -gx[a] * Hz + gz[a] * Hx;
            w[5] += gx[a] * Hy - gy[a] * Hx;
          }
        }
        float* wd = sW + (le * L::NPM1P + b) * NW;
        if constexpr (NW == 4) {
          *reinterpret_cast<float4*>(wd) = make_float4(w[0], w[1], w[2], w[3]);
        } else {
#pragma unroll
          for (int m = 0; m < NW; m += 2) *reinterpret_cast<float2*>(wd + m) = make_float2(w[m], w[m + 1]);
        }
      }
      if (pre) {
        const int64_t nb = (int64_t)((uint32_t)cpre >> 5);
        const int nfc = (cpre >> 3) & 3;
        if (nb < K && (nb < tpre * EPB || nb >= (tpre + 1) * EPB)) {
          // the bulk prefetch wants a 16-byte aligned start and size; a face block
          // (NF * NFP floats) need not be, so widen it to 16-byte boundaries. The trace
          // buffer starts on such a boundary and its length (16 K NF NFP bytes) is a
          // multiple of 16, so the widened range stays inside it.
          const uintptr_t a0 = (uintptr_t)(P.trace_in + ((size_t)nb * 4 + nfc) * NF * NFP);
          const uintptr_t lo = a0 & ~(uintptr_t)15;
          const uintptr_t hi = (a0 + (uintptr_t)(NF * NFP * 4) + 15) & ~(uintptr_t)15;
          l2_prefetch(reinterpret_cast<const void*>(lo), (uint32_t)(hi - lo));
        }
      }
      if (tnext < ntiles) {
        if (!mbar_wait(&bar[s ^ 1], (ph >> (s ^ 1)) & 1u, wlim)) {
          s_fail = 1;
          atomicOr(P.status, 2);
        }
        ph ^= 1u << (s ^ 1);
        if (!*vfail) flux_tile(tnext, s ^ 1, sX + (s ^ 1) * NCHAIN * NFP);
      }
      if (stage && !*vfail) {
        if (!mbar_wait(&bar[2], (ph >> 2) & 1u, wlim)) {
          s_fail = 1;
          atomicOr(P.status, 2);
        }
        ph ^= 4u;
      }
    }
    if (is_elem) nbar_sync(1 + grp, GCOUNT);

    // ---- B. sum lift stacks + volume term, divide by J, LSRK update ------------------
    if (is_elem && !*vfail) {
      const float* g = sGeo + le * BB_GEO_STRIDE;
      const float invJ = g[9];
      float nxf[4], nyf[4], nzf[4];
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        nxf[f] = g[12 + f];
        nyf[f] = g[16 + f];
        nzf[f] = g[20 + f];
      }
      const float* G = sG + le * 4 * NPS * NCH;   // this element's four face stacks
      const float* wb = sW + le * L::NPM1P * NW;  // this element's w(beta), NW per point
      // faces whose partner lies outside this tile need their updated trace in HBM
      bool leave[4];
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        const int64_t nb = (int64_t)((uint32_t)sConn[le * 4 + f] >> 5);
        leave[f] = P.trace_out != nullptr && (nb < e0 || nb >= e0 + EPB);
      }
      // all right-hand sides of this thread first (shared-memory reads only), then the
      // updates and stores, so that no store sits between the loads of different r
      float rhs_all[GR][NF];
#pragma unroll
      for (int r = 0; r < GR; ++r) {
        const int n = u + r * TPE;
        if (n >= NP) continue;
        const uint4 ga = sGA[n];
        const int p[4] = {(int)(ga.y & 1023), (int)((ga.y >> 10) & 1023), (int)(ga.y >> 20),
                          (int)(ga.w & 1023)};
        const int xb[4] = {(int)(ga.x & 1023), (int)((ga.x >> 10) & 1023), (int)(ga.x >> 20),
                           (int)(ga.w >> 10)};
        // alpha_b as floats: byte b placed in the mantissa of 2^23, minus 2^23 (exact)
        float ab[4];
#pragma unroll
        for (int b = 0; b < 4; ++b)
          ab[b] = __uint_as_float(__byte_perm(ga.z, 0x4B000000u, 0x7540u + b)) - 8388608.0f;
        // vol(alpha) = sum_b alpha_b w(alpha - e_b), b = 3 first (as the fma nesting before)
        float vol[NW];
        if constexpr (NW == 4) {
          const float4 w3 = *reinterpret_cast<const float4*>(wb + xb[3] * 4);
          vol[0] = ab[3] * w3.x;
          vol[1] = ab[3] * w3.y;
          vol[2] = ab[3] * w3.z;
          vol[3] = ab[3] * w3.w;
#pragma unroll
          for (int b = 2; b >= 0; --b) {
            const float4 wv = *reinterpret_cast<const float4*>(wb + xb[b] * 4);
            vol[0] = fmaf(ab[b], wv.x, vol[0]);
            vol[1] = fmaf(ab[b], wv.y, vol[1]);
            vol[2] = fmaf(ab[b], wv.z, vol[2]);
            vol[3] = fmaf(ab[b], wv.w, vol[3]);
          }
        } else {
#pragma unroll
          for (int m = 0; m < NW; m += 2) {
            const float2 w3 = *reinterpret_cast<const float2*>(wb + xb[3] * NW + m);
            vol[m] = ab[3] * w3.x;
            vol[m + 1] = ab[3] * w3.y;
          }
#pragma unroll
          for (int b = 2; b >= 0; --b) {
#pragma unroll
            for (int m = 0; m < NW; m += 2) {
              const float2 wv = *reinterpret_cast<const float2*>(wb + xb[b] * NW + m);
              vol[m] = fmaf(ab[b], wv.x, vol[m]);
              vol[m + 1] = fmaf(ab[b], wv.y, vol[m + 1]);
            }
          }
        }
        float* rhs = rhs_all[r];
        if constexpr (PHYS == BB_WAVE) {
          // face order of src/BernsteinLift.jl:202-214: t=-1 face first, then f1, f2, f3;
          // the stacks already carry the l_d weights
          const float2 g3 = *reinterpret_cast<const float2*>(G + (3 * NPS + p[3]) * 2);
          float A = g3.x;
          float Bx = nxf[3] * g3.y, By = nyf[3] * g3.y, Bz = nzf[3] * g3.y;
#pragma unroll
          for (int f = 0; f < 3; ++f) {
            const float2 gf = *reinterpret_cast<const float2*>(G + (f * NPS + p[f]) * 2);
            A += gf.x;
            Bx = fmaf(nxf[f], gf.y, Bx);
            By = fmaf(nyf[f], gf.y, By);
            Bz = fmaf(nzf[f], gf.y, Bz);
          }
          rhs[0] = (A - vol[0]) * invJ;
          rhs[1] = (Bx - vol[1]) * invJ;
          rhs[2] = (By - vol[2]) * invJ;
          rhs[3] = (Bz - vol[3]) * invJ;
        } else {
          float v[6];
#pragma unroll
          for (int m = 0; m < 6; m += 2) {
            const float2 g3 = *reinterpret_cast<const float2*>(G + (3 * NPS + p[3]) * 6 + m);
            v[m] = g3.x;
            v[m + 1] = g3.y;
          }
#pragma unroll
          for (int f = 0; f < 3; ++f) {
#pragma unroll
            for (int m = 0; m < 6; m += 2) {
              const float2 gf = *reinterpret_cast<const float2*>(G + (f * NPS + p[f]) * 6 + m);
              v[m] += gf.x;
              v[m + 1] += gf.y;
            }
          }
#pragma unroll
          for (int m = 0; m < 6; ++m) rhs[m] = (v[m] + vol[m]) * invJ;
        }
      }
      float* __restrict__ gq_out = P.q;
      float* __restrict__ gres_out = P.res;
      float* __restrict__ grhs_out = P.rhs;
#pragma unroll
      for (int r = 0; r < GR; ++r) {
        const int n = u + r * TPE;
        if (n >= NP) continue;
        const float* rhs = rhs_all[r];
        const int item = le * NP + n;
        if (!stage) {
#pragma unroll
          for (int m = 0; m < NF; ++m) grhs_out[((size_t)m * K + e0) * NP + item] = rhs[m];
        } else {
          // q and res leave straight from registers (coalesced: item runs along the tile),
          // and so do the outgoing face traces of the coefficients that lie on a face
          float qn[NF];
#pragma unroll
          for (int m = 0; m < NF; ++m) {
            const float rr = fmaf(rkA, sRes[m * EPB * NP + item], dt * rhs[m]);
            qn[m] = fmaf(rkB, rr, sQ[m * EPB * NP + item]);
            gres_out[((size_t)m * K + e0) * NP + item] = rr;
            gq_out[((size_t)m * K + e0) * NP + item] = qn[m];
          }
          const uint32_t tf = sTF[n];
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            const uint32_t a = (tf >> (8 * f)) & 0xffu;
            if (a != 0xffu && leave[f]) {
              float* dst = P.trace_out + ((size_t)(e0 + le) * 4 + f) * NF * NFP + a;
#pragma unroll
              for (int m = 0; m < NF; ++m) dst[m * NFP] = qn[m];
            }
          }
        }
      }
    }
  }
  if (issuer) {
    // let the copies this thread issued land before the block exits: immediate when the
    // element threads consumed them, bounded otherwise
    if (iss0) mbar_wait(&bar[0], (iss0 - 1u) & 1u, wlim);
    if (iss1) mbar_wait(&bar[1], (iss1 - 1u) & 1u, wlim);
    if (iss2) mbar_wait(&bar[2], (iss2 - 1u) & 1u, wlim);
  }
}

// Volume-phase work split (host, once per variant): the NPM1 points beta, in index order, are
// cut into VR * TPE / 32 contiguous ranges of at most 32, one per warp-round, where the cuts
// minimise the shared-memory wavefronts of the phase's accesses: the NF-field q reads at
// beta + e_a (a = 0..3, 32 lanes, one word each) and the w(beta) store (NW floats per point, in
// 16-byte or 8-byte pieces). Exact dynamic programme over the cut positions.
struct VolGroups {
  uint16_t start[16];
  uint8_t len[16];
};
template <int N, int PHYS, int TPE>
VolGroups volume_groups() {
  constexpr int NPM1 = N * (N + 1) * (N + 2) / 6, NF = FPhys<PHYS>::NF, NW = FPhys<PHYS>::NW;
  constexpr int VR = (NPM1 + TPE - 1) / TPE, G = VR * (TPE / 32);
  static_assert(G <= 16 && NPM1 < 65536, "volume groups fit the launch parameters");
  std::vector<std::array<int, 4>> qi(NPM1);
  for (int k = 0, b = 0; k < N; ++k)
    for (int j = 0; j < N - k; ++j)
      for (int i = 0; i < N - j - k; ++i, ++b)
        qi[b] = {ijk3(N, i + 1, j, k), ijk3(N, i, j + 1, k), ijk3(N, i, j, k + 1), ijk3(N, i, j, k)};
  // wavefronts of one access: per phase of `lanes` lanes, the largest number of distinct
  // addresses (in units of `unit` words) that share a bank group
  auto wavefronts = [](const std::vector<int>& words, int unit, int lanes) {
    int tot = 0;
    const int groups = 32 / unit;
    for (size_t p0 = 0; p0 < words.size(); p0 += lanes) {
      int best = 0;
      for (int g = 0; g < groups; ++g) {
        int cnt = 0;
        std::vector<int> seen;
        for (size_t q = p0; q < words.size() && q < p0 + lanes; ++q) {
          const int a = words[q] / unit;
          if (a % groups != g) continue;
          bool dup = false;
          for (int x : seen) dup |= x == a;
          if (!dup) seen.push_back(a), ++cnt;
        }
        best = std::max(best, cnt);
      }
      tot += best;
    }
    return tot;
  };
  auto range_cost = [&](int a, int b) {
    if (b <= a) return 0;
    int c = 0;
    std::vector<int> w;
    for (int t = 0; t < 4; ++t) {
      w.clear();
      for (int x = a; x < b; ++x) w.push_back(qi[x][t]);
      c += NF * wavefronts(w, 1, 32);
    }
    w.clear();
    for (int x = a; x < b; ++x) w.push_back(x * NW);
    c += NW == 4 ? wavefronts(w, 4, 8) : (NW / 2) * wavefronts(w, 2, 16);
    return c;
  };
  std::vector<std::array<int, 33>> rc(NPM1 + 1);  // rc[a][n] = cost of [a, a + n)
  for (int a = 0; a <= NPM1; ++a)
    for (int n = 0; n <= 32; ++n) rc[a][n] = a + n <= NPM1 ? range_cost(a, a + n) : 0;
  const int INF = 1 << 29;
  std::vector<std::vector<int>> dp(G + 1, std::vector<int>(NPM1 + 1, INF)),
      arg(G + 1, std::vector<int>(NPM1 + 1, 0));
  dp[0][0] = 0;
  for (int g = 1; g <= G; ++g)
    for (int i = 0; i <= NPM1; ++i)
      for (int a = std::max(0, i - 32); a <= i; ++a) {
        if (dp[g - 1][a] >= INF) continue;
        const int c = dp[g - 1][a] + rc[a][i - a];
        if (c < dp[g][i]) dp[g][i] = c, arg[g][i] = a;
      }
  VolGroups v{};
  for (int g = G, i = NPM1; g >= 1; --g) {
    const int a = arg[g][i];
    v.start[g - 1] = (uint16_t)a;
    v.len[g - 1] = (uint8_t)(i - a);
    i = a;
  }
  return v;
}

template <int N, int PHYS, int EPB, int TPE>
int launch_fast_t(const FastLaunch& fl, const FastStageParams& P0, cudaStream_t st) {
  using L = FastLayout<N, PHYS, EPB, TPE>;
  auto kern = stage_fast_kernel<N, PHYS, EPB, TPE>;
  static const VolGroups vg = volume_groups<N, PHYS, TPE>();
  FastStageParams P = P0;
  for (int g = 0; g < 16; ++g) P.vstart[g] = vg.start[g], P.vlen[g] = vg.len[g];
  P.wait_iters = fl.wait_iters;
  P.fault = fl.fault;
  // shared-memory opt-in and resident blocks per SM, set up once per device (the host-buffer
  // path launches each stage in up to 24 tile ranges)
  static std::atomic<int> per_sm_of[64];
  int per_sm = fl.device >= 0 && fl.device < 64 ? per_sm_of[fl.device].load() : 0;
  if (per_sm < 1) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES) !=
        cudaSuccess)
      return BB_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, L::NT, L::BYTES) !=
            cudaSuccess ||
        per_sm < 1)
      return BB_ERR_CUDA;
    if (fl.device >= 0 && fl.device < 64) per_sm_of[fl.device].store(per_sm);
  }
  if (P.K % EPB != 0) return BB_ERR_ARG;
  const int64_t tend = P.tile_end > 0 ? P.tile_end : P.K / EPB;
  if (P.tile_begin < 0 || P.tile_begin >= tend || tend > P.K / EPB) return BB_ERR_ARG;
  const int64_t ntiles = tend - P.tile_begin;
  int64_t grid = (int64_t)per_sm * fl.num_sms;
  if (grid > ntiles) grid = ntiles;
  kern<<<(int)grid, L::NT, L::BYTES, st>>>(P);
  return cudaGetLastError() == cudaSuccess ? BB_OK : BB_ERR_CUDA;
}

}  // namespace bbfast

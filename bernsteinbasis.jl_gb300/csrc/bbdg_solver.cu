// Fused DG right-hand side + low-storage RK stage for the wave and Maxwell examples.
//
// One thread block owns a tile of `epb` consecutive elements and does, per RK stage:
//   1. stage q (all fields), geometry and connectivity of its tile in shared memory
//   2. interface flux at every face node (examples/3d_wave.jl:41-56,
//      examples/3d_maxwell.jl:185-209): the neighbour trace comes from shared memory when
//      the neighbour is in the same tile, otherwise from the trace buffer written by the
//      previous stage (only faces that cross a tile boundary are ever written or read)
//   3. volume term (3d_wave.jl:59-79): the geometric combination of Dr, Ds, Dt is applied
//      as sum_b alpha_b w(alpha - e_b), w(beta) = sum_a g_a x(beta + e_a), g the barycentric
//      weights of the physical derivative (Dr = (D0 - D3)/2 etc.)
//   4. lift of the four face fluxes (src/BernsteinLift.jl:139-220), accumulated in place
//   5. divide by J, LSRK update res = A res + dt rhs, q += B res; write q, res and the
//      tile's outgoing traces
// q and res are updated in place: no block reads another tile's q, so there is no race.
#include <cmath>
#include <cstring>

#include "bbdg_internal.cuh"
#include "bbdg_stage_fast.cuh"

namespace {

constexpr int kThreads = 256;

template <int PHYS>
struct Phys;
template <>
struct Phys<BB_WAVE> {
  static constexpr int NF = 4;  // p, u, v, w
  static constexpr int NW = 4;  // div(u,v,w), dp/dx, dp/dy, dp/dz (scaled by J)
  static constexpr float vol_sign = -1.f;
};
template <>
struct Phys<BB_MAXWELL> {
  static constexpr int NF = 6;  // Hx, Hy, Hz, Ex, Ey, Ez
  static constexpr int NW = 6;  // curl terms
  static constexpr float vol_sign = 1.f;
};

template <class T>
struct StageParams {
  DegTables tab;
  const uint32_t* gtab;
  const T* lj;
  int64_t K;
  int epb;
  int mode;             // 0: write rhs to `rhs`; 1: LSRK stage update of q and res
  T rkA, rkB, dt, tau;  // stage coefficients, time step, penalty (tau <= 0: as written)
  T* q;                 // [NF][K][Np]
  T* res;               // [NF][K][Np]
  T* rhs;               // mode 0 output [NF][K][Np]
  const T* trace_in;    // [K][4][NF][Nfp] or nullptr: gather neighbour traces from q
  T* trace_out;         // [K][4][NF][Nfp] or nullptr
  const T* geo;         // [K][BB_GEO_STRIDE]
  const int32_t* conn;  // [K][4]
  int* status;          // device error word
};

// Shared-memory layout of a tile (in units of T unless noted).
struct TileLayout {
  size_t q, out, flux, work, geo, lj, conn_bytes, tab_bytes, total;
  int work_elems;
};

template <class T, int PHYS>
TileLayout tile_layout(const DegTables& t, int epb) {
  constexpr int NF = Phys<PHYS>::NF, NW = Phys<PHYS>::NW;
  TileLayout L;
  const size_t Np = t.Np, Nfp = t.Nfp, S = np2(t.N + 1);
  size_t off = 0;
  L.q = off; off += (size_t)NF * epb * Np;
  L.out = off; off += (size_t)NF * epb * Np;
  L.flux = off; off += (size_t)epb * 4 * NF * Nfp;
  L.work = off;
  const size_t wvol = (size_t)NW * epb * t.NpM1, wlift = 2 * (size_t)epb * NF * S;
  L.work_elems = (int)(wvol > wlift ? wvol : wlift);
  off += L.work_elems;
  L.geo = off; off += (size_t)epb * BB_GEO_STRIDE;
  L.lj = off; off += t.N + 1;
  size_t bytes = align16(off * sizeof(T));
  L.conn_bytes = bytes; bytes += align16((size_t)epb * 4 * sizeof(int32_t));
  L.tab_bytes = bytes; bytes += (size_t)t.nwords * 4;
  L.total = align16(bytes);
  return L;
}

template <class T, int PHYS>
__global__ void __launch_bounds__(kThreads) stage_kernel(StageParams<T> P, TileLayout L) {
  constexpr int NF = Phys<PHYS>::NF, NW = Phys<PHYS>::NW;
  extern __shared__ __align__(16) unsigned char smem[];
  T* sbase = reinterpret_cast<T*>(smem);
  T* sQ = sbase + L.q;
  T* sOut = sbase + L.out;
  T* sFlux = sbase + L.flux;
  T* sWork = sbase + L.work;
  T* sGeo = sbase + L.geo;
  T* sLj = sbase + L.lj;
  int32_t* sConn = reinterpret_cast<int32_t*>(smem + L.conn_bytes);
  const SmemTables st =
      load_tables(P.tab, P.gtab, reinterpret_cast<uint32_t*>(smem + L.tab_bytes));
  const int N = P.tab.N, Np = P.tab.Np, NpM1 = P.tab.NpM1, Nfp = P.tab.Nfp;
  const int64_t K = P.K;
  const int epb = P.epb;
  for (int j = threadIdx.x; j <= N; j += blockDim.x) sLj[j] = P.lj[j];
  const int64_t ntiles = (K + epb - 1) / epb;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t e0 = tile * epb;
    const int ne = (int)min64(epb, K - e0);
    __syncthreads();
    // ---- 1. stage q, geometry, connectivity --------------------------------------------
    for (int fld = 0; fld < NF; ++fld)
      copy_g2s(sQ + (size_t)fld * epb * Np, P.q + ((size_t)fld * K + e0) * Np, ne * Np);
    copy_g2s(sGeo, P.geo + e0 * BB_GEO_STRIDE, ne * BB_GEO_STRIDE);
    for (int t = threadIdx.x; t < ne * 4; t += blockDim.x) sConn[t] = __ldg(P.conn + e0 * 4 + t);
    __syncthreads();

    // ---- 2. interface flux -------------------------------------------------------------
    for (int it = threadIdx.x; it < ne * 4 * Nfp; it += blockDim.x) {
      const int le = it / (4 * Nfp);
      const int rem = it - le * 4 * Nfp;
      const int f = rem / Nfp, a = rem - f * Nfp;
      const int32_t c = sConn[le * 4 + f];
      const int64_t nbr = (int64_t)((uint32_t)c >> 5);
      const int nface = (c >> 3) & 3, o = c & 7;
      T d[NF];
      const int vM = st.fvol[f * Nfp + a];
      if (nbr >= K || o > 5) {
        atomicOr(P.status, 1);
        for (int fld = 0; fld < NF; ++fld) d[fld] = T(0);
      } else {
        const int ap = st.fperm[o * Nfp + a];
        if (nbr >= e0 && nbr < e0 + ne) {
          const int vP = st.fvol[nface * Nfp + ap];
          const T* qP = sQ + (size_t)(nbr - e0) * Np + vP;
          const T* qM = sQ + (size_t)le * Np + vM;
#pragma unroll
          for (int fld = 0; fld < NF; ++fld) d[fld] = qP[(size_t)fld * epb * Np] - qM[(size_t)fld * epb * Np];
        } else if (P.trace_in) {
          const T* tp = P.trace_in + ((size_t)nbr * 4 + nface) * NF * Nfp + ap;
          const T* qM = sQ + (size_t)le * Np + vM;
#pragma unroll
          for (int fld = 0; fld < NF; ++fld) d[fld] = __ldg(tp + (size_t)fld * Nfp) - qM[(size_t)fld * epb * Np];
        } else {
          const int vP = st.fvol[nface * Nfp + ap];
          const T* qP = P.q + (size_t)nbr * Np + vP;
          const T* qM = sQ + (size_t)le * Np + vM;
#pragma unroll
          for (int fld = 0; fld < NF; ++fld) d[fld] = __ldg(qP + (size_t)fld * K * Np) - qM[(size_t)fld * epb * Np];
        }
      }
      const T* g = sGeo + le * BB_GEO_STRIDE;
      const T nx = g[12 + f], ny = g[16 + f], nz = g[20 + f];
      T cp = T(1), cu = T(1);
      if (P.tau > T(0)) {
        const T Jf = sqrt(nx * nx + ny * ny + nz * nz);
        cp = P.tau * Jf;
        cu = P.tau / Jf;
      }
      T fl[NF];
      if constexpr (PHYS == BB_WAVE) {
        // 3d_wave.jl:45-54
        const T ndotdU = nx * d[1] + ny * d[2] + nz * d[3];
        const T A = cp * d[0] - ndotdU;
        const T B = cu * ndotdU - d[0];
        fl[0] = T(0.5) * A;
        fl[1] = T(0.5) * (B * nx);
        fl[2] = T(0.5) * (B * ny);
        fl[3] = T(0.5) * (B * nz);
      } else {
        // 3d_maxwell.jl:189-207: 0.5 (fx nx + fy ny + fz nz)(du) + 0.5 du - 0.5 n (n.d)
        const T Hx = d[0], Hy = d[1], Hz = d[2], Ex = d[3], Ey = d[4], Ez = d[5];
        const T ndH = nx * Hx + ny * Hy + nz * Hz;
        const T ndE = nx * Ex + ny * Ey + nz * Ez;
        const T ax[6] = {T(0), Ez, -Ey, T(0), -Hz, Hy};
        const T ay[6] = {-Ez, T(0), Ex, Hz, T(0), -Hx};
        const T az[6] = {Ey, -Ex, T(0), -Hy, Hx, T(0)};
        const T nd[6] = {ndH * nx, ndH * ny, ndH * nz, ndE * nx, ndE * ny, ndE * nz};
#pragma unroll
        for (int m = 0; m < 6; ++m)
          fl[m] = T(0.5) * ax[m] * nx + T(0.5) * ay[m] * ny + T(0.5) * az[m] * nz +
                  T(0.5) * (cp * d[m]) - T(0.5) * (cu * nd[m]);
      }
      T* fo = sFlux + ((size_t)(le * 4 + f) * NF) * Nfp + a;
#pragma unroll
      for (int fld = 0; fld < NF; ++fld) fo[(size_t)fld * Nfp] = fl[fld];
    }

    // ---- 3a. volume term at degree N-1 -------------------------------------------------
    for (int it = threadIdx.x; it < ne * NpM1; it += blockDim.x) {
      const int le = it / NpM1, b = it - le * NpM1;
      const uint32_t c = st.node3m1[b];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16;
      const int idx[4] = {ijk3(N, i + 1, j, k), ijk3(N, i, j + 1, k), ijk3(N, i, j, k + 1),
                          ijk3(N, i, j, k)};
      const T* g = sGeo + le * BB_GEO_STRIDE;
      // barycentric weights of d/dx, d/dy, d/dz (times J): g_a = (rxJ, sxJ, txJ, -sum)/2;
      // the fourth weight is implied by the differences below
      T gx[3], gy[3], gz[3];
      gx[0] = T(0.5) * g[0]; gx[1] = T(0.5) * g[1]; gx[2] = T(0.5) * g[2];
      gy[0] = T(0.5) * g[3]; gy[1] = T(0.5) * g[4]; gy[2] = T(0.5) * g[5];
      gz[0] = T(0.5) * g[6]; gz[1] = T(0.5) * g[7]; gz[2] = T(0.5) * g[8];
      const T* q0 = sQ + (size_t)le * Np;
      auto F = [&](int fld, int a) { return q0[(size_t)fld * epb * Np + idx[a]]; };
      T w[NW];
#pragma unroll
      for (int m = 0; m < NW; ++m) w[m] = T(0);
      // sum_a g_a x(beta+e_a) with sum_a g_a = 0, formed as sum_{a<3} g_a (x_a - x_3) so
      // that smooth data cancels in the differences (as the reference's Dr = (D0 - D3)/2)
      if constexpr (PHYS == BB_WAVE) {
        const T p3 = F(0, 3), u3 = F(1, 3), v3 = F(2, 3), w3 = F(3, 3);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const T p = F(0, a) - p3, u = F(1, a) - u3, v = F(2, a) - v3, ww = F(3, a) - w3;
          w[0] += gx[a] * u + gy[a] * v + gz[a] * ww;
          w[1] += gx[a] * p;
          w[2] += gy[a] * p;
          w[3] += gz[a] * p;
        }
      } else {
        const T Hx3 = F(0, 3), Hy3 = F(1, 3), Hz3 = F(2, 3);
        const T Ex3 = F(3, 3), Ey3 = F(4, 3), Ez3 = F(5, 3);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const T Hx = F(0, a) - Hx3, Hy = F(1, a) - Hy3, Hz = F(2, a) - Hz3;
          const T Ex = F(3, a) - Ex3, Ey = F(4, a) - Ey3, Ez = F(5, a) - Ez3;
          w[0] += -gy[a] * Ez + gz[a] * Ey;  // d/dt Hx = -dEz/dy + dEy/dz
          w[1] += gx[a] * Ez - gz[a] * Ex;   // d/dt Hy
          w[2] += -gx[a] * Ey + gy[a] * Ex;  // d/dt Hz
          w[3] += gy[a] * Hz - gz[a] * Hy;   // d/dt Ex
          w[4] += -gx[a] * Hz + gz[a] * Hx;  // d/dt Ey
          w[5] += gx[a] * Hy - gy[a] * Hx;   // d/dt Ez
        }
      }
#pragma unroll
      for (int m = 0; m < NW; ++m) sWork[((size_t)m * epb + le) * NpM1 + b] = w[m];
    }
    __syncthreads();
    // ---- 3b. elevate back to degree N: out(alpha) = sign * sum_b alpha_b w(alpha - e_b) -
    for (int it = threadIdx.x; it < ne * Np; it += blockDim.x) {
      const int le = it / Np, n = it - le * Np;
      const uint32_t c = st.node3[n];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16, l = N - i - j - k;
      T acc[NW];
#pragma unroll
      for (int m = 0; m < NW; ++m) acc[m] = T(0);
      const T* wb = sWork + (size_t)le * NpM1;
      const size_t ws = (size_t)epb * NpM1;
      if (i > 0) {
        const int x = ijk3(N - 1, i - 1, j, k);
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[m] += T(i) * wb[m * ws + x];
      }
      if (j > 0) {
        const int x = ijk3(N - 1, i, j - 1, k);
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[m] += T(j) * wb[m * ws + x];
      }
      if (k > 0) {
        const int x = ijk3(N - 1, i, j, k - 1);
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[m] += T(k) * wb[m * ws + x];
      }
      if (l > 0) {
        const int x = ijk3(N - 1, i, j, k);
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[m] += T(l) * wb[m * ws + x];
      }
#pragma unroll
      for (int m = 0; m < NF; ++m)
        sOut[((size_t)m * epb + le) * Np + n] = T(Phys<PHYS>::vol_sign) * acc[m];
    }
    __syncthreads();

    // ---- 4. lift of the face fluxes, face t=-1 first as src/BernsteinLift.jl:202-205 ----
    {
      const int order[4] = {3, 0, 1, 2};
      const int S = np2(N + 1);
      T* bufA = sWork;
      T* bufB = sWork + (size_t)epb * NF * S;
      for (int q = 0; q < 4; ++q) {
        const int f = order[q];
        lift_face_accumulate<T>(N, f, ne, NF, st.node2, sFlux + (size_t)f * NF * Nfp,
                                4 * NF * Nfp, Nfp, sOut, Np, epb * Np, bufA, bufB, sLj);
      }
    }

    // ---- 5. divide by J, RK update, write back -----------------------------------------
    if (P.mode == 0) {
      for (int fld = 0; fld < NF; ++fld) {
        T* dst = P.rhs + ((size_t)fld * K + e0) * Np;
        const T* src = sOut + (size_t)fld * epb * Np;
        for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) {
          const int le = t / Np;
          dst[t] = src[t] * sGeo[le * BB_GEO_STRIDE + 9];
        }
      }
    } else {
      for (int fld = 0; fld < NF; ++fld) {
        T* gq = P.q + ((size_t)fld * K + e0) * Np;
        T* gr = P.res + ((size_t)fld * K + e0) * Np;
        T* sq = sQ + (size_t)fld * epb * Np;
        const T* so = sOut + (size_t)fld * epb * Np;
        for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) {
          const int le = t / Np;
          const T rhs = so[t] * sGeo[le * BB_GEO_STRIDE + 9];
          const T r = P.rkA * gr[t] + P.dt * rhs;
          const T qn = sq[t] + P.rkB * r;
          gr[t] = r;
          gq[t] = qn;
          sq[t] = qn;
        }
      }
      if (P.trace_out) {
        __syncthreads();
        for (int it = threadIdx.x; it < ne * 4 * NF * Nfp; it += blockDim.x) {
          const int le = it / (4 * NF * Nfp);
          int rem = it - le * 4 * NF * Nfp;
          const int f = rem / (NF * Nfp);
          rem -= f * NF * Nfp;
          const int fld = rem / Nfp, a = rem - fld * Nfp;
          const int64_t nbr = (int64_t)((uint32_t)sConn[le * 4 + f] >> 5);
          if (nbr >= e0 && nbr < e0 + ne) continue;  // neighbour inside the tile
          P.trace_out[((size_t)(e0 + le) * 4 + f) * NF * Nfp + (size_t)fld * Nfp + a] =
              sQ[((size_t)fld * epb + le) * Np + st.fvol[f * Nfp + a]];
        }
      }
    }
  }
}

// Writes every face trace of q (all faces) into the trace buffer.
template <class T, int NF>
__global__ void extract_traces_kernel(DegTables tab, const uint32_t* __restrict__ gtab,
                                      int64_t K, const T* __restrict__ q, T* __restrict__ tr) {
  const int Np = tab.Np, Nfp = tab.Nfp;
  const uint16_t* fvol = reinterpret_cast<const uint16_t*>(gtab + tab.o_fvol);
  const int64_t total = K * 4 * NF * Nfp;
  for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < total;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = it / (4 * NF * Nfp);
    int rem = (int)(it - e * 4 * NF * Nfp);
    const int f = rem / (NF * Nfp);
    rem -= f * NF * Nfp;
    const int fld = rem / Nfp, a = rem - fld * Nfp;
    tr[it] = q[((size_t)fld * K + e) * Np + fvol[f * Nfp + a]];
  }
}

// Carpenter & Kennedy (1994) five-stage fourth-order 2N-storage coefficients.
const double kRK4A[5] = {0.0, -567301805773.0 / 1357537059087.0,
                         -2404267990393.0 / 2016746695238.0,
                         -3550918686646.0 / 2091501179385.0,
                         -1275806237668.0 / 842570457699.0};
const double kRK4B[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                         1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                         2277821191437.0 / 14882151754819.0};

}  // namespace

// -------------------------------------------------------------------------------------
// solver object
// -------------------------------------------------------------------------------------
struct bb_solver {
  bb_ctx* ctx = nullptr;
  int physics = 0, N = 0, dtype = 0, nf = 0;
  int64_t K = 0;
  const int32_t* conn = nullptr;
  const void* geo = nullptr;
  double tau = 0.0;
  const DegTables* tab = nullptr;
  int epb = 0, threads = kThreads;
  int fast = -1;  // index of the degree-specialised FP32 variant in use, -1 = generic kernel
  int generic_only = 0;
  int grid = 0;
  size_t smem = 0;
  void* trace[2] = {nullptr, nullptr};
  size_t trace_bytes = 0;
  int* d_status = nullptr;
  cudaStream_t cap_stream = nullptr;
  // graph cache: one graph per starting trace buffer parity
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  void* g_q = nullptr;
  void* g_res = nullptr;
  double g_dt = 0.0;
  int g_epb = 0;
};

namespace {

int solver_layout(bb_solver* s, int epb, size_t* smem_out) {
  TileLayout L;
  if (s->physics == BB_WAVE)
    L = s->dtype == BB_F64 ? tile_layout<double, BB_WAVE>(*s->tab, epb)
                           : tile_layout<float, BB_WAVE>(*s->tab, epb);
  else
    L = s->dtype == BB_F64 ? tile_layout<double, BB_MAXWELL>(*s->tab, epb)
                           : tile_layout<float, BB_MAXWELL>(*s->tab, epb);
  *smem_out = L.total;
  return L.total <= s->ctx->smem_optin ? BB_OK : BB_ERR_ARG;
}

template <class T, int PHYS>
int launch_stage_t(bb_solver* s, int mode, int stage, double dt, void* q, void* res, void* rhs,
                   const void* tin, void* tout, cudaStream_t st) {
  bb_ctx* ctx = s->ctx;
  StageParams<T> P;
  P.tab = *s->tab;
  P.gtab = s->tab->d_words;
  P.lj = sizeof(T) == 8 ? (const T*)s->tab->d_lj : (const T*)s->tab->d_ljf;
  P.K = s->K;
  P.epb = s->epb;
  P.mode = mode;
  P.rkA = T(mode ? kRK4A[stage] : 0.0);
  P.rkB = T(mode ? kRK4B[stage] : 0.0);
  P.dt = T(dt);
  P.tau = T(s->tau);
  P.q = (T*)q;
  P.res = (T*)res;
  P.rhs = (T*)rhs;
  P.trace_in = (const T*)tin;
  P.trace_out = (T*)tout;
  P.geo = (const T*)s->geo;
  P.conn = s->conn;
  P.status = s->d_status;
  TileLayout L = tile_layout<T, PHYS>(*s->tab, s->epb);
  static_assert(sizeof(StageParams<T>) < 4096, "params");
  BB_CUDA(ctx, cudaFuncSetAttribute(stage_kernel<T, PHYS>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
  int per_sm = 0;
  BB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stage_kernel<T, PHYS>,
                                                             kThreads, L.total));
  if (per_sm < 1) return bb_fail(ctx, BB_ERR_ARG, "tile does not fit on an SM");
  const int64_t ntiles = (s->K + s->epb - 1) / s->epb;
  int64_t grid = (int64_t)per_sm * ctx->num_sms;
  if (grid > ntiles) grid = ntiles;
  stage_kernel<T, PHYS><<<(int)grid, kThreads, L.total, st>>>(P, L);
  return bb_check_launch(ctx, "stage_kernel");
}

int launch_fast(bb_solver* s, int mode, int stage, double dt, void* q, void* res, void* rhs,
                const void* tin, void* tout, cudaStream_t st) {
  FastStageParams P;
  const DegTables& t = *s->tab;
  P.gtab = t.d_words;
  P.o_node3 = t.o_node3;
  P.o_node3m1 = t.o_node3m1;
  P.o_fvol = t.o_fvol;
  P.o_fperm = t.o_fperm;
  P.K = s->K;
  P.mode = mode;
  P.rkA = float(mode ? kRK4A[stage] : 0.0);
  P.rkB = float(mode ? kRK4B[stage] : 0.0);
  P.dt = float(dt);
  P.tau = float(s->tau);
  P.q = (float*)q;
  P.res = (float*)res;
  P.rhs = (float*)rhs;
  P.trace_in = (const float*)tin;
  P.trace_out = (float*)tout;
  P.geo = (const float*)s->geo;
  P.conn = s->conn;
  P.status = s->d_status;
  FastLaunch fl;
  fl.num_sms = s->ctx->num_sms;
  const int rc = bb_fast_launch(s->fast, fl, P, st);
  if (rc) return bb_fail(s->ctx, rc, "stage_fast_kernel launch: %s", cudaGetErrorString(cudaGetLastError()));
  s->ctx->launches++;
  return BB_OK;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

int launch_stage(bb_solver* s, int mode, int stage, double dt, void* q, void* res, void* rhs,
                 const void* tin, void* tout, cudaStream_t st) {
  // the specialised kernels move tiles with 16-byte-aligned bulk copies
  if (s->fast >= 0 && aligned16(q) && (!res || aligned16(res)) && aligned16(s->geo) &&
      aligned16(s->conn))
    return launch_fast(s, mode, stage, dt, q, res, rhs, tin, tout, st);
  if (s->physics == BB_WAVE)
    return s->dtype == BB_F64
               ? launch_stage_t<double, BB_WAVE>(s, mode, stage, dt, q, res, rhs, tin, tout, st)
               : launch_stage_t<float, BB_WAVE>(s, mode, stage, dt, q, res, rhs, tin, tout, st);
  return s->dtype == BB_F64
             ? launch_stage_t<double, BB_MAXWELL>(s, mode, stage, dt, q, res, rhs, tin, tout, st)
             : launch_stage_t<float, BB_MAXWELL>(s, mode, stage, dt, q, res, rhs, tin, tout, st);
}

int launch_extract(bb_solver* s, const void* q, void* tr, cudaStream_t st) {
  const int64_t total = s->K * 4 * s->nf * s->tab->Nfp;
  int64_t grid = (total + 255) / 256;
  if (grid > (int64_t)s->ctx->num_sms * 16) grid = (int64_t)s->ctx->num_sms * 16;
  if (grid < 1) grid = 1;
  const DegTables& t = *s->tab;
  if (s->dtype == BB_F64) {
    if (s->nf == 4)
      extract_traces_kernel<double, 4><<<(int)grid, 256, 0, st>>>(t, t.d_words, s->K, (const double*)q, (double*)tr);
    else
      extract_traces_kernel<double, 6><<<(int)grid, 256, 0, st>>>(t, t.d_words, s->K, (const double*)q, (double*)tr);
  } else {
    if (s->nf == 4)
      extract_traces_kernel<float, 4><<<(int)grid, 256, 0, st>>>(t, t.d_words, s->K, (const float*)q, (float*)tr);
    else
      extract_traces_kernel<float, 6><<<(int)grid, 256, 0, st>>>(t, t.d_words, s->K, (const float*)q, (float*)tr);
  }
  return bb_check_launch(s->ctx, "extract_traces_kernel");
}

int check_status(bb_solver* s, cudaStream_t st) {
  int h = 0;
  BB_CUDA(s->ctx, cudaMemcpyAsync(&h, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  BB_CUDA(s->ctx, cudaStreamSynchronize(st));
  if (h) {
    cudaMemsetAsync(s->d_status, 0, sizeof(int), st);
    return bb_fail(s->ctx, BB_ERR_DEVICE, "device check failed (corrupt connectivity)");
  }
  return BB_OK;
}

void drop_graphs(bb_solver* s) {
  for (auto& g : s->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// One LSRK step (5 stages) starting from trace buffer `par`; ends in buffer 1 - par.
int enqueue_step(bb_solver* s, double dt, void* q, void* res, int par, cudaStream_t st) {
  for (int stage = 0; stage < 5; ++stage) {
    const int in = (par + stage) & 1;
    int rc = launch_stage(s, 1, stage, dt, q, res, nullptr, s->trace[in], s->trace[in ^ 1], st);
    if (rc) return rc;
  }
  return BB_OK;
}

int build_graph(bb_solver* s, double dt, void* q, void* res, int par) {
  bb_ctx* ctx = s->ctx;
  cudaGraph_t g = nullptr;
  BB_CUDA(ctx, cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(s, dt, q, res, par, s->cap_stream);
  cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bb_fail(ctx, BB_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&s->graph[par], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bb_fail(ctx, BB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return BB_OK;
}

}  // namespace

extern "C" int bb_solver_create(bb_ctx* ctx, int physics, int N, int64_t K, int dtype,
                                const int32_t* conn, const void* geo, double tau,
                                bb_solver** out) {
  if (!ctx || !out) return BB_ERR_ARG;
  *out = nullptr;
  if (physics != BB_WAVE && physics != BB_MAXWELL)
    return bb_fail(ctx, BB_ERR_ARG, "physics must be BB_WAVE or BB_MAXWELL");
  if (!valid_degree(N)) return bb_fail(ctx, BB_ERR_ARG, "degree N=%d outside 1..%d", N, BB_MAX_DEGREE);
  if (!valid_dtype(dtype)) return bb_fail(ctx, BB_ERR_ARG, "bad dtype");
  if (K < 1 || K >= (int64_t(1) << 27)) return bb_fail(ctx, BB_ERR_ARG, "K must be in 1..2^27-1");
  if (!conn || !geo) return bb_fail(ctx, BB_ERR_ARG, "null connectivity or geometry");
  if (!std::isfinite(tau)) return bb_fail(ctx, BB_ERR_ARG, "tau must be finite");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  const DegTables* t = bb_tables(ctx, N);
  if (!t) return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
  bb_solver* s = new (std::nothrow) bb_solver();
  if (!s) return BB_ERR_NOMEM;
  s->ctx = ctx;
  s->physics = physics;
  s->N = N;
  s->K = K;
  s->dtype = dtype;
  s->nf = physics == BB_WAVE ? 4 : 6;
  s->conn = conn;
  s->geo = geo;
  s->tau = tau;
  s->tab = t;
  // default tile: the largest of 12, 6, 4, 2, 1 elements that fits in 100 KB of smem
  const int cands[5] = {12, 6, 4, 2, 1};
  for (int c : cands) {
    size_t sm = 0;
    if (solver_layout(s, c, &sm) == BB_OK && sm <= 100 * 1024) {
      s->epb = c;
      s->smem = sm;
      break;
    }
  }
  if (!s->epb) {
    size_t sm = 0;
    if (solver_layout(s, 1, &sm) != BB_OK) {
      delete s;
      return bb_fail(ctx, BB_ERR_ARG, "degree %d does not fit in shared memory", N);
    }
    s->epb = 1;
    s->smem = sm;
  }
  if (dtype == BB_F32) {
    const int idx = bb_fast_find(N, physics, 0, 0, K);
    int e = 0, th = 0;
    size_t sm = 0;
    if (idx >= 0 && bb_fast_variant_info(idx, &e, &th, &sm) == BB_OK && sm <= ctx->smem_optin) {
      s->fast = idx;
      s->epb = e;
      s->threads = th;
      s->smem = sm;
    }
  }
  s->trace_bytes = (size_t)K * 4 * s->nf * t->Nfp * dtype_size(dtype);
  if (cudaMalloc(&s->trace[0], s->trace_bytes) != cudaSuccess ||
      cudaMalloc(&s->trace[1], s->trace_bytes) != cudaSuccess ||
      cudaMalloc(&s->d_status, sizeof(int)) != cudaSuccess ||
      cudaMemset(s->d_status, 0, sizeof(int)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(s->trace[0]);
    cudaFree(s->trace[1]);
    cudaFree(s->d_status);
    delete s;
    return bb_fail(ctx, BB_ERR_NOMEM, "solver allocation failed");
  }
  *out = s;
  return BB_OK;
}

extern "C" int bb_solver_destroy(bb_solver* s) {
  if (!s) return BB_ERR_ARG;
  cudaSetDevice(s->ctx->device);
  drop_graphs(s);
  cudaFree(s->trace[0]);
  cudaFree(s->trace[1]);
  cudaFree(s->d_status);
  if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
  delete s;
  return BB_OK;
}

extern "C" int bb_solver_set_tile(bb_solver* s, int epb, int threads) {
  if (!s) return BB_ERR_ARG;
  // degree-specialised FP32 variants first, unless the generic kernel was requested
  if (s->dtype == BB_F32 && !s->generic_only) {
    const int idx = bb_fast_find(s->N, s->physics, epb, threads, s->K);
    int e = 0, th = 0;
    size_t sm = 0;
    if (idx >= 0 && bb_fast_variant_info(idx, &e, &th, &sm) == BB_OK && sm <= s->ctx->smem_optin) {
      if (idx != s->fast || e != s->epb) drop_graphs(s);
      s->fast = idx;
      s->epb = e;
      s->threads = th;
      s->smem = sm;
      return BB_OK;
    }
  }
  if (threads != 0 && threads != kThreads)
    return bb_fail(s->ctx, BB_ERR_ARG, "no variant with %d threads per block", threads);
  if (epb == 0) epb = 6;
  if (epb < 1 || epb > 64) return bb_fail(s->ctx, BB_ERR_ARG, "elements per block must be 1..64");
  size_t sm = 0;
  if (solver_layout(s, epb, &sm) != BB_OK)
    return bb_fail(s->ctx, BB_ERR_ARG, "tile of %d elements exceeds shared memory", epb);
  if (epb != s->epb || s->fast >= 0) drop_graphs(s);
  s->fast = -1;
  s->epb = epb;
  s->threads = kThreads;
  s->smem = sm;
  return BB_OK;
}

extern "C" int bb_solver_set_kernel(bb_solver* s, int kind) {
  if (!s) return BB_ERR_ARG;
  if (kind != 0 && kind != 1) return bb_fail(s->ctx, BB_ERR_ARG, "kind must be 0 or 1");
  s->generic_only = kind;
  if (kind == 1 && s->fast >= 0) return bb_solver_set_tile(s, s->epb, kThreads);
  if (kind == 0 && s->fast < 0 && s->dtype == BB_F32 && bb_fast_find(s->N, s->physics, 0, 0, s->K) >= 0)
    return bb_solver_set_tile(s, 0, 0);
  return BB_OK;
}

extern "C" int bb_solver_get_kernel(const bb_solver* s) {
  return s ? (s->fast >= 0 ? 0 : 1) : -1;
}

extern "C" int bb_solver_get_tile(const bb_solver* s, int* epb, int* threads) {
  if (!s) return BB_ERR_ARG;
  if (epb) *epb = s->epb;
  if (threads) *threads = s->threads;
  return BB_OK;
}

extern "C" int bb_rhs(bb_solver* s, const void* q, void* rhs, void* stream) {
  if (!s || !q || !rhs) return s ? bb_fail(s->ctx, BB_ERR_ARG, "null pointer") : BB_ERR_ARG;
  if (q == rhs) return bb_fail(s->ctx, BB_ERR_ARG, "rhs must not alias q");
  int rc = bb_set_device(s->ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const void* tin = nullptr;
  if (s->fast >= 0) {  // the specialised kernel reads outside-tile traces from the buffer
    rc = launch_extract(s, q, s->trace[0], st);
    if (rc) return rc;
    tin = s->trace[0];
  }
  rc = launch_stage(s, 0, 0, 0.0, const_cast<void*>(q), nullptr, rhs, tin, nullptr, st);
  if (rc) return rc;
  return check_status(s, st);
}

extern "C" int bb_lsrk_run(bb_solver* s, double dt, int nsteps, void* q, void* res, int use_graph,
                           void* stream) {
  if (!s || !q || !res) return s ? bb_fail(s->ctx, BB_ERR_ARG, "null pointer") : BB_ERR_ARG;
  if (nsteps < 0 || !std::isfinite(dt)) return bb_fail(s->ctx, BB_ERR_ARG, "bad dt or nsteps");
  if (q == res) return bb_fail(s->ctx, BB_ERR_ARG, "res must not alias q");
  int rc = bb_set_device(s->ctx);
  if (rc) return rc;
  if (nsteps == 0) return BB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  // traces of the incoming state; stage kernels then keep them current
  rc = launch_extract(s, q, s->trace[0], st);
  if (rc) return rc;
  if (use_graph) {
    if (s->g_q != q || s->g_res != res || s->g_dt != dt || s->g_epb != s->epb) drop_graphs(s);
    for (int par = 0; par < 2; ++par)
      if (!s->graph[par]) {
        rc = build_graph(s, dt, q, res, par);
        if (rc) return rc;
      }
    s->g_q = q;
    s->g_res = res;
    s->g_dt = dt;
    s->g_epb = s->epb;
    for (int step = 0; step < nsteps; ++step) {
      BB_CUDA(s->ctx, cudaGraphLaunch(s->graph[step & 1], st));
      s->ctx->launches += 5;
    }
  } else {
    for (int step = 0; step < nsteps; ++step) {
      rc = enqueue_step(s, dt, q, res, step & 1, st);
      if (rc) return rc;
    }
  }
  return BB_OK;
}

extern "C" int bb_lsrk_run_host(bb_solver* s, double dt, int nsteps, const void* q_host_in,
                                void* q_host_out, void* q_dev, void* res_dev, int use_graph,
                                void* stream) {
  if (!s || !q_host_in || !q_host_out || !q_dev || !res_dev)
    return s ? bb_fail(s->ctx, BB_ERR_ARG, "null pointer") : BB_ERR_ARG;
  int rc = bb_set_device(s->ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = (size_t)s->nf * s->K * s->tab->Np * dtype_size(s->dtype);
  BB_CUDA(s->ctx, cudaMemcpyAsync(q_dev, q_host_in, bytes, cudaMemcpyHostToDevice, st));
  rc = bb_lsrk_run(s, dt, nsteps, q_dev, res_dev, use_graph, st);
  if (rc) return rc;
  BB_CUDA(s->ctx, cudaMemcpyAsync(q_host_out, q_dev, bytes, cudaMemcpyDeviceToHost, st));
  return BB_OK;
}

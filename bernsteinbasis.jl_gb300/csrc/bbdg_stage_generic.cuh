// Generic (runtime-degree) DG stage tile: shared by the per-solver stage kernel
// (bbdg_solver.cu) and the batched persistent kernel (bbdg_batch.cu).
//
// One thread block owns a tile of `epb` consecutive elements and does, per RK stage:
//   1. stage q (all fields), geometry and connectivity of its tile in shared memory
//   2. interface flux at every face node (examples/3d_wave.jl:41-56,
//      examples/3d_maxwell.jl:43-65): the neighbour trace comes from shared memory when
//      the neighbour is in the same tile, otherwise from the trace buffer written by the
//      previous stage (only faces that cross a tile boundary are ever written or read)
//   3. volume term (3d_wave.jl:59-79): the geometric combination of Dr, Ds, Dt is applied
//      as sum_b alpha_b w(alpha - e_b), w(beta) = sum_a g_a x(beta + e_a), g the barycentric
//      weights of the physical derivative (Dr = (D0 - D3)/2 etc.)
//   4. lift of the four face fluxes (src/BernsteinLift.jl:139-220), accumulated in place
//   5. divide by J, LSRK update res = A res + dt rhs, q += B res; write q, res and the
//      tile's outgoing traces
// q and res are updated in place: no block reads another tile's q, so there is no race.
#pragma once

#include "bbdg_internal.cuh"

template <int PHYS>
struct Phys;
template <>
struct Phys<BB_WAVE> {
  static constexpr int NF = 4;  // p, u, v, w
  static constexpr int NW = 4;  // div(u,v,w), dp/dx, dp/dy, dp/dz (scaled by J)
  static constexpr int NCH = 2;  // lift chains per face: pressure flux, scalar velocity flux
  static constexpr float vol_sign = -1.f;
};
template <>
struct Phys<BB_MAXWELL> {
  static constexpr int NF = 6;  // Hx, Hy, Hz, Ex, Ey, Ez
  static constexpr int NW = 6;  // curl terms
  static constexpr int NCH = 6;  // one lift chain per field
  static constexpr float vol_sign = 1.f;
};
// examples/3d_advec_scalar.jl: du = -(LIFT flux + J du/dx) / J; the flux is stored negated
// so that the shared "sign * volume + lift" combination gives the example's right-hand side.
template <>
struct Phys<BB_ADVECTION> {
  static constexpr int NF = 1;  // u
  static constexpr int NW = 1;  // J du/dx
  static constexpr int NCH = 1;
  static constexpr float vol_sign = -1.f;
};
// examples/3d_advec.jl: q = (u, v, w), fx(q) = (u, 0, 0), fy = fz = 0: the flux of the
// scalar example on each component, the volume term on u only; du = -(...) / J as above.
template <>
struct Phys<BB_ADVECTION3> {
  static constexpr int NF = 3;  // u, v, w
  static constexpr int NW = 1;  // J du/dx (v and w have no volume term)
  static constexpr int NCH = 3;
  static constexpr float vol_sign = -1.f;
};

template <class T>
struct StageParams {
  DegTables tab;
  const uint32_t* gtab;
  int64_t K;
  int64_t tile_begin, tile_end;  // stage_kernel's tiles [tile_begin, tile_end) (end 0 = all)
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

// Shared-memory layout of a tile (in units of T unless noted). chain != 0: the lift runs one
// thread per (element, face, chain) with the face stacks in shared memory (FP32 tiles that fit
// in kChainLiftBytes); chain == 0: the level-parallel lift with two ping-pong rows.
struct TileLayout {
  size_t q, out, flux, work, geo, pen, gh, conn_bytes, tab_bytes, total;
  int work_elems;
  int chain;
};
constexpr size_t kChainLiftBytes = 100 * 1024;
// The batched kernel uses the same rule, so that a tile timed on a single problem (how its
// size is chosen per physics and degree) runs the same code inside the batch.
constexpr size_t kBatchChainLiftBytes = kChainLiftBytes;

// Lift chains per face for NF fields (Phys<PHYS>::NCH): the wave's velocity flux is a scalar
// times the face normal, so its three components share one chain.
__host__ __device__ inline int lift_chains(int NF) { return NF == 4 ? 2 : NF; }

// Layout for degree N with Np/Nfp/NpM1 coefficients, NF fields, NW volume terms, scalars of
// `tsize` bytes and `nwords` 32-bit table words.
__host__ __device__ inline TileLayout tile_layout_with(int N, int NF, int NW, size_t tsize,
                                                      int nwords, int epb, int chain) {
  TileLayout L;
  const size_t Np = np3(N), Nfp = np2(N), NpM1 = np3(N - 1), S = np2(N + 1);
  const size_t nch = (size_t)lift_chains(NF);
  size_t off = 0;
  L.q = off; off += (size_t)NF * epb * Np;
  L.out = off; off += (size_t)NF * epb * Np;
  L.flux = off; off += (size_t)epb * 4 * NF * Nfp;
  L.work = off;
  const size_t wvol = (size_t)NW * epb * NpM1;
  const size_t wlift = chain ? (size_t)epb * 4 * nch * (Np + (Nfp | 1))  // stacks + rows
                             : 2 * (size_t)epb * nch * S;
  L.work_elems = (int)(wvol > wlift ? wvol : wlift);
  off += L.work_elems;
  L.geo = off; off += (size_t)epb * BB_GEO_STRIDE;
  L.pen = off; off += (size_t)epb * 8;  // per face: tau |n|, tau / |n|
  L.gh = off; off += (size_t)epb * 9;   // per element: rxJ ... txJ / 2
  size_t bytes = align16(off * tsize);
  L.conn_bytes = bytes; bytes += align16((size_t)epb * 4 * sizeof(int32_t));
  L.tab_bytes = bytes; bytes += (size_t)nwords * 4;
  L.total = align16(bytes);
  L.chain = chain;
  return L;
}

// FP32: the chain lift when its tile fits in `budget` bytes, else the level-parallel one.
// FP64 always takes the level-parallel lift: the chain phase keeps one thread per (element,
// face, chain) busy, too few to feed the FP64 pipe (wave N = 9, 2-element tiles: the pipe is
// 48 % busy with chains against 80 % level-parallel, 2.38 against 1.65 ms per stage).
__host__ __device__ inline TileLayout tile_layout_for(int N, int NF, int NW, size_t tsize,
                                                     int nwords, int epb,
                                                     size_t budget = kChainLiftBytes) {
  const TileLayout c = tile_layout_with(N, NF, NW, tsize, nwords, epb, 1);
  return tsize == 4 && c.total <= budget ? c : tile_layout_with(N, NF, NW, tsize, nwords, epb, 0);
}

// One face lift chain for run-time N, one thread (src/BernsteinLift.jl:139-164):
//   F_0 = L0 x (the 7-point stencil of (N+1)^2/2 R_{N+1} E_{N->N+1}), F_d = l_d E_d with
//   E_d = R_{N-d+1} E_{d-1}, carried as F_d = -1/(d+1) [(i+1) F_{d-1}(i+1,j) +
//   (j+1) F_{d-1}(i,j+1) + (N-d+1-i-j) F_{d-1}(i,j)] (l_d / l_{d-1} = -(N-d+1)/(d+1))
// in place in ascending order on the thread's shared-memory row E (degree-N layout), each F_d
// written to the face's stack g in volume order through the stack table fst (face f's
// entries: layer d, then j, then i, i + j <= N - d). Per point the same arithmetic as
// lift_face_accumulate, so both lifts give the same stacks.
template <class T>
__device__ void chain_lift_runtime(int N, const T* __restrict__ x, T* __restrict__ E,
                                   T* __restrict__ g, const uint16_t* __restrict__ fst) {
  int rb = 0;  // row offset of row j in the degree-N triangle
  for (int j = 0; j <= N; ++j) {
    const int rlen = N + 1 - j;
    const int rbn = rb + rlen;          // row j + 1
    const int rbp = rb - (rlen + 1);    // row j - 1 (used only when j > 0)
    for (int i = 0; i < rlen; ++i) {
      const T e = l0_point<T>(i, j, N - i - j, x, rb, rbn, rbp);
      E[rb + i] = e;
      g[fst[rb + i]] = e;  // layer 0: stack index = 2D index
    }
    rb = rbn;
  }
  int s = rb;  // == np2(N): first entry of layer 1
  for (int d = 1; d <= N; ++d) {
    const int n = N - d + 1;  // input degree of this reduction
    const T cd = -inv_int<T>(d + 1);  // l_d / (l_{d-1} n)
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const int rn = r + (N + 1 - j);  // next row in the degree-N layout
      for (int i = 0; i + j < n; ++i) {
        // in place, ascending: (i+1, j) and (i, j+1) are still degree-n values
        const T v = reduce_point<T>(i, j, n, E[r + i + 1], E[rn + i], E[r + i], cd);
        E[r + i] = v;
        g[fst[s++]] = v;
      }
      r = rn;
    }
  }
}

template <class T, int PHYS>
TileLayout tile_layout(const DegTables& t, int epb) {
  return tile_layout_for(t.N, Phys<PHYS>::NF, Phys<PHYS>::NW, sizeof(T), t.nwords, epb);
}

// One tile of the generic stage (all threads of the block call it). The degree tables are in
// shared memory (st); the layout L matches P's degree, physics and tile.
template <class T, int PHYS, bool CHAIN_LIFT = true>
__device__ void generic_stage_tile(const StageParams<T>& P, const TileLayout& L,
                                   const SmemTables& st, int64_t tile) {
  constexpr int NF = Phys<PHYS>::NF, NW = Phys<PHYS>::NW, NCH = Phys<PHYS>::NCH;
  extern __shared__ __align__(16) unsigned char smem[];
  T* sbase = reinterpret_cast<T*>(smem);
  T* sQ = sbase + L.q;
  T* sOut = sbase + L.out;
  T* sFlux = sbase + L.flux;
  T* sWork = sbase + L.work;
  T* sGeo = sbase + L.geo;
  T* sPen = sbase + L.pen;
  T* sGh = sbase + L.gh;
  int32_t* sConn = reinterpret_cast<int32_t*>(smem + L.conn_bytes);
  const int N = P.tab.N, Np = P.tab.Np, NpM1 = P.tab.NpM1, Nfp = P.tab.Nfp;
  const int64_t K = P.K;
  const int epb = P.epb;
  const FastDiv by_np(Np), by_npm1(NpM1), by_nfp(Nfp), by_4nfp(4 * Nfp), by_nfnp(NF * Np),
      by_nfnfp(NF * Nfp), by_4nfnfp(4 * NF * Nfp);
    const int64_t e0 = tile * epb;
    const int ne = (int)min64(epb, K - e0);
    __syncthreads();
    // ---- 1. stage q, geometry, connectivity --------------------------------------------
    for (int fld = 0; fld < NF; ++fld)
      copy_g2s(sQ + (size_t)fld * epb * Np, P.q + ((size_t)fld * K + e0) * Np, ne * Np);
    copy_g2s(sGeo, P.geo + e0 * BB_GEO_STRIDE, ne * BB_GEO_STRIDE);
    for (int t = threadIdx.x; t < ne * 4; t += blockDim.x) {
      sConn[t] = __ldg(P.conn + e0 * 4 + t);
      // the face's penalty weights (tau |n|, tau / |n|; 1 and 1 with tau <= 0), once per face:
      // a square root and a division are long sequences on the FP64 pipe
      const T* g = P.geo + (e0 + (t >> 2)) * BB_GEO_STRIDE + 12 + (t & 3);
      const T nx = __ldg(g), ny = __ldg(g + 4), nz = __ldg(g + 8);
      T cp = T(1), cu = T(1);
      if (P.tau > T(0)) {
        const T Jf = sqrt(nx * nx + ny * ny + nz * nz);
        cp = P.tau * Jf;
        cu = P.tau / Jf;
      }
      sPen[2 * t] = cp;
      sPen[2 * t + 1] = cu;
    }
    // barycentric weights of J d/dx, J d/dy, J d/dz: g_a = (rxJ, sxJ, txJ, -sum) / 2, once
    // per element rather than per volume point
    for (int t = threadIdx.x; t < ne * 9; t += blockDim.x) {
      const int le = t / 9;
      sGh[t] = T(0.5) * __ldg(P.geo + (e0 + le) * BB_GEO_STRIDE + (t - le * 9));
    }
    __syncthreads();

    // ---- 2. interface flux -------------------------------------------------------------
    for (int it = threadIdx.x; it < ne * 4 * Nfp; it += blockDim.x) {
      const int le = by_4nfp.div(it);
      const int rem = it - le * 4 * Nfp;
      const int f = by_nfp.div(rem), a = rem - f * Nfp;
      const int32_t c = sConn[le * 4 + f];
      const int64_t nbr = (int64_t)((uint32_t)c >> 5);
      const int nface = (c >> 3) & 3, o = c & 7;
      T d[NF];
      const int vM = st.fvol[f * Nfp + a];
      if (nbr >= K || o > 5) {
        atomicOr(P.status, 1);
        for (int fld = 0; fld < NF; ++fld) d[fld] = T(0);
      } else if (!BB_DCHECK(vM < Np && st.fperm[o * Nfp + a] < Nfp, P.status)) {
        for (int fld = 0; fld < NF; ++fld) d[fld] = T(0);
      } else {
        const int ap = st.fperm[o * Nfp + a];
        if (nbr >= e0 && nbr < e0 + ne) {
          const int vP = BB_DCHECK(st.fvol[nface * Nfp + ap] < Np, P.status)
                             ? st.fvol[nface * Nfp + ap] : vM;
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
          const int vP = BB_DCHECK(st.fvol[nface * Nfp + ap] < Np, P.status)
                             ? st.fvol[nface * Nfp + ap] : vM;
          const T* qP = P.q + (size_t)nbr * Np + vP;
          const T* qM = sQ + (size_t)le * Np + vM;
#pragma unroll
          for (int fld = 0; fld < NF; ++fld) d[fld] = __ldg(qP + (size_t)fld * K * Np) - qM[(size_t)fld * epb * Np];
        }
      }
      const T* g = sGeo + le * BB_GEO_STRIDE;
      const T nx = g[12 + f], ny = g[16 + f], nz = g[20 + f];
      const T cp = sPen[(le * 4 + f) * 2], cu = sPen[(le * 4 + f) * 2 + 1];
      T fl[NF];
      if constexpr (PHYS == BB_ADVECTION || PHYS == BB_ADVECTION3) {
        // 3d_advec_scalar.jl:24-29, 3d_advec.jl:44-45: 0.5 du nxJ - 0.5 du Jf per component
        // (negated, see Phys<BB_ADVECTION>)
        const T Jf = sqrt(nx * nx + ny * ny + nz * nz);
#pragma unroll
        for (int m = 0; m < NF; ++m) fl[m] = -(T(0.5) * d[m] * nx - T(0.5) * d[m] * Jf);
      } else if constexpr (PHYS == BB_WAVE) {
        // 3d_wave.jl:45-54
        // the velocity flux 0.5 B (nx, ny, nz) is stored as the scalar 0.5 B; the lift
        // multiplies its result by the normal
        const T ndotdU = nx * d[1] + ny * d[2] + nz * d[3];
        const T A = cp * d[0] - ndotdU;
        const T B = cu * ndotdU - d[0];
        fl[0] = T(0.5) * A;
        fl[1] = T(0.5) * B;
      } else {
        // 3d_maxwell.jl:52-63: 0.5 (fx nx + fy ny + fz nz)(du) + 0.5 du - 0.5 n (n.d)
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
      for (int ch = 0; ch < NCH; ++ch) fo[(size_t)ch * Nfp] = fl[ch];
    }

    // ---- 3a. volume term at degree N-1 -------------------------------------------------
    for (int it = threadIdx.x; it < ne * NpM1; it += blockDim.x) {
      const int le = by_npm1.div(it), b = it - le * NpM1;
      const uint32_t c = st.node3m1[b];
      const int i = c & 0xff, j = (c >> 8) & 0xff, k = c >> 16;
      const int idx[4] = {ijk3(N, i + 1, j, k), ijk3(N, i, j + 1, k), ijk3(N, i, j, k + 1),
                          ijk3(N, i, j, k)};
      // barycentric weights of d/dx, d/dy, d/dz (times J), staged per element; the fourth
      // weight is implied by the differences below
      const T* gx = sGh + le * 9;  // gx[a], then gy = gx + 3, gz = gx + 6
      const T* gy = gx + 3;
      const T* gz = gx + 6;
      const T* q0 = sQ + (size_t)le * Np;
      auto F = [&](int fld, int a) { return q0[(size_t)fld * epb * Np + idx[a]]; };
      T w[NW];
#pragma unroll
      for (int m = 0; m < NW; ++m) w[m] = T(0);
      // sum_a g_a x(beta+e_a) with sum_a g_a = 0, formed as sum_{a<3} g_a (x_a - x_3) so
      // that smooth data cancels in the differences (as the reference's Dr = (D0 - D3)/2)
      if constexpr (PHYS == BB_ADVECTION || PHYS == BB_ADVECTION3) {
        const T u3 = F(0, 3);
#pragma unroll
        for (int a = 0; a < 3; ++a) w[0] += gx[a] * (F(0, a) - u3);  // J du/dx
      } else if constexpr (PHYS == BB_WAVE) {
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
      const int le = by_np.div(it), n = it - le * Np;
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
        for (int m = 0; m < NW; ++m) acc[m] += small_int<T>(i) * wb[m * ws + x];
      }
      if (j > 0) {
        const int x = ijk3(N - 1, i, j - 1, k);
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[m] += small_int<T>(j) * wb[m * ws + x];
      }
      if (k > 0) {
        const int x = ijk3(N - 1, i, j, k - 1);
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[m] += small_int<T>(k) * wb[m * ws + x];
      }
      if (l > 0) {
        const int x = ijk3(N - 1, i, j, k);
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[m] += small_int<T>(l) * wb[m * ws + x];
      }
#pragma unroll
      for (int m = 0; m < NF; ++m) {
        const T v = m < NW ? acc[m < NW ? m : 0] : T(0);  // fields past NW: no volume term
        sOut[((size_t)m * epb + le) * Np + n] = Phys<PHYS>::vol_sign < 0 ? -v : v;
      }
    }
    __syncthreads();

    // ---- 4. lift of the face fluxes, face t=-1 first as src/BernsteinLift.jl:202-205 ----
    if (CHAIN_LIFT && L.chain) {
      // one thread per (element, face, chain); stacks land in volume order
      const int nchain = ne * 4 * NCH;
      const int rs = Nfp | 1;
      T* sStack = sWork;                                // [epb*4*NCH][Np]
      T* sRow = sWork + (size_t)epb * 4 * NCH * Np;     // [epb*4*NCH][rs]
      for (int c = threadIdx.x; c < nchain; c += blockDim.x) {
        const int ef = c / NCH, ch = c - ef * NCH;      // c = (le*4 + f)*NCH + ch
        chain_lift_runtime<T>(N, sFlux + ((size_t)ef * NF + ch) * Nfp, sRow + (size_t)c * rs,
                              sStack + (size_t)c * Np, st.fstack + (size_t)(ef & 3) * Np);
      }
      __syncthreads();
      // faces in the order 3, 0, 1, 2 (as lift_face_accumulate, so that both lifts agree)
      for (int it = threadIdx.x; it < ne * NF * Np; it += blockDim.x) {
        const int le = by_nfnp.div(it), rem = it - le * NF * Np;
        const int fld = by_np.div(rem), n = rem - fld * Np;
        T* o = sOut + ((size_t)fld * epb + le) * Np + n;
        T acc = *o;
        if (PHYS == BB_WAVE && fld > 0) {
          // velocity component fld - 1: the scalar chain times that normal component
          const T* g = sStack + ((size_t)le * 4 * NCH + 1) * Np + n;  // face f at + f*NCH*Np
          const T* nc = sGeo + le * BB_GEO_STRIDE + 12 + 4 * (fld - 1);
          acc = fma(nc[3], g[(size_t)3 * NCH * Np], acc);
          acc = fma(nc[0], g[0], acc);
          acc = fma(nc[1], g[(size_t)1 * NCH * Np], acc);
          acc = fma(nc[2], g[(size_t)2 * NCH * Np], acc);
        } else {
          const T* g = sStack + ((size_t)le * 4 * NCH + fld) * Np + n;
          acc += g[(size_t)3 * NCH * Np];
          acc += g[0];
          acc += g[(size_t)1 * NCH * Np];
          acc += g[(size_t)2 * NCH * Np];
        }
        *o = acc;
      }
      __syncthreads();
    } else {
      const int S = np2(N + 1);
      T* bufA = sWork;
      T* bufB = sWork + (size_t)epb * NCH * S;
      for (int q = 0; q < 4; ++q) {
        const int f = (q + 3) & 3;  // faces 3, 0, 1, 2
        lift_face_accumulate<T, PHYS == BB_WAVE>(N, f, ne, NCH, st.node2,
                                                 sFlux + (size_t)f * NF * Nfp, 4 * NF * Nfp, Nfp,
                                                 sOut, Np, epb * Np, bufA, bufB, sGeo + 12 + f);
      }
    }

    // ---- 5. divide by J, RK update, write back -----------------------------------------
    if (P.mode == 0) {
      for (int fld = 0; fld < NF; ++fld) {
        T* dst = P.rhs + ((size_t)fld * K + e0) * Np;
        const T* src = sOut + (size_t)fld * epb * Np;
        for (int t = threadIdx.x; t < ne * Np; t += blockDim.x) {
          const int le = by_np.div(t);
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
          const int le = by_np.div(t);
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
          const int le = by_4nfnfp.div(it);
          int rem = it - le * 4 * NF * Nfp;
          const int f = by_nfnfp.div(rem);
          rem -= f * NF * Nfp;
          const int fld = by_nfp.div(rem), a = rem - fld * Nfp;
          const int64_t nbr = (int64_t)((uint32_t)sConn[le * 4 + f] >> 5);
          if (nbr >= e0 && nbr < e0 + ne) continue;  // neighbour inside the tile
          P.trace_out[((size_t)(e0 + le) * 4 + f) * NF * Nfp + (size_t)fld * Nfp + a] =
              sQ[((size_t)fld * epb + le) * Np + st.fvol[f * Nfp + a]];
        }
      }
    }
}

// CPU oracle for the Bernstein DG hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file restates, loop for loop, the Julia reference vincentxwang/BernsteinBasis.jl:
//   src/ordering.jl:6-39                    index ordering (tri/tet offsets, ij/ijk_to_linear)
//   src/constants.jl:10-16                  lift-chain scalars l_j(N)
//   src/BernsteinDerivativeMatrix_3D.jl:96-231  fast_Dr/Ds/Dt_multiply! and the matrix mul!
//   src/BernsteinLift.jl:66-164             reduction_multiply!, elevation_multiply!,
//                                           face_lift_multiply!
//   src/BernsteinLift.jl:191-220,264-269    BernsteinLift mul! (vector and matrix form)
//   examples/3d_wave.jl:36-84               wave rhs_matvec!
//   examples/3d_maxwell.jl:36-93            Maxwell rhs_matvec!
// plus a 5-stage, 4th-order, 2N-storage low-storage Runge-Kutta (Carpenter & Kennedy 1994),
// which replaces the examples' OrdinaryDiffEq integrator (examples/3d_wave.jl:133-134).
//
// It is the checker for the CUDA path and the timed CPU baseline; nothing in the product
// links or calls it. Indices here are 0-based; the Julia source is 1-based.
// State layout follows the reference: Matrix{SVector{nf}} of size Np x K, column-major,
// i.e. q[(e*Np + node)*nf + field].
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// The reference's offset tuples hold 21 entries (ordering.jl:8-26): enough for degree 20,
// not for the degree N + 1 = 21 that the lift of degree 20 elevates to (row 21 of that
// triangle), so the reference's lift stops at N = 19. These tables run two entries further by
// the same formula, so that the library's N = 20 lift is checked; oracle_offsets exports the
// reference's 21.
constexpr int kOffsets = 23;
struct Offsets {
  int tri[kOffsets];
  int tet[kOffsets];
};

// ordering.jl:8-26 (tri_offsets / tet_offsets)
Offsets make_offsets(int N) {
  Offsets o;
  o.tri[0] = 0;
  o.tet[0] = 0;
  int c2 = 0, c3 = 0;
  for (int i = 1; i < kOffsets; ++i) {
    c2 += N + 2 - i;
    c3 += ((N + 2 - i) * (N + 3 - i)) / 2;
    o.tri[i] = c2;
    o.tet[i] = c3;
  }
  return o;
}

// ordering.jl:6 and :32-35, 0-based.
inline int ij_lin(int i, int j, const Offsets& o) { return i + o.tri[j]; }
inline int ijk_lin(int i, int j, int k, const Offsets& o) {
  return i + o.tri[j] + o.tet[k] - j * k;
}

// constants.jl:10-12
double l_j(int N, int j) {
  if (j > N) return 0.0;
  double b = 1.0;  // binomial(N, j), exact in double for N <= 20
  for (int m = 1; m <= j; ++m) b = b * (N - j + m) / m;
  return ((j % 2) ? -1.0 : 1.0) * b / (1.0 + j);
}

inline int np3(int N) { return (N + 1) * (N + 2) * (N + 3) / 6; }
inline int np2(int N) { return (N + 1) * (N + 2) / 2; }

// Small fixed-size vector standing in for StaticArrays.SVector{NF,T}.
template <class T, int NF>
struct SV {
  T v[NF];
  static SV zero() {
    SV r;
    for (int f = 0; f < NF; ++f) r.v[f] = T(0);
    return r;
  }
};
template <class T, int NF>
inline SV<T, NF> operator+(const SV<T, NF>& a, const SV<T, NF>& b) {
  SV<T, NF> r;
  for (int f = 0; f < NF; ++f) r.v[f] = a.v[f] + b.v[f];
  return r;
}
template <class T, int NF>
inline SV<T, NF> operator-(const SV<T, NF>& a, const SV<T, NF>& b) {
  SV<T, NF> r;
  for (int f = 0; f < NF; ++f) r.v[f] = a.v[f] - b.v[f];
  return r;
}
template <class T, int NF, class S>
inline SV<T, NF> operator*(S s, const SV<T, NF>& a) {
  SV<T, NF> r;
  for (int f = 0; f < NF; ++f) r.v[f] = T(s) * a.v[f];
  return r;
}
template <class T, int NF, class S>
inline SV<T, NF> operator/(const SV<T, NF>& a, S s) {
  SV<T, NF> r;
  for (int f = 0; f < NF; ++f) r.v[f] = a.v[f] / T(s);
  return r;
}
// Scalar "vectors" use plain T.
template <class T>
inline T zero_of(const T*) { return T(0); }
template <class T, int NF>
inline SV<T, NF> zero_of(const SV<T, NF>*) { return SV<T, NF>::zero(); }

// BernsteinDerivativeMatrix_3D.jl:96-132 (fast_Dr_multiply!)
template <class V>
void fast_Dr(V* out, int N, const V* x, const Offsets& o) {
  const V Z = zero_of(x);
  int row = 0;
  for (int k = 0; k <= N; ++k)
    for (int j = 0; j <= N - k; ++j)
      for (int i = 0; i <= N - j - k; ++i) {
        int l = N - i - j - k;
        V val = Z;
        V x_row = x[row];
        V x1 = x_row;
        V x4 = (i > 0) ? x[ijk_lin(i - 1, j, k, o)] : Z;
        val = val + i * (x1 - x4);
        if (j > 0) {
          x1 = x[ijk_lin(i + 1, j - 1, k, o)];
          x4 = x[ijk_lin(i, j - 1, k, o)];
          val = val + j * (x1 - x4);
        }
        if (k > 0) {
          x1 = x[ijk_lin(i + 1, j, k - 1, o)];
          x4 = x[ijk_lin(i, j, k - 1, o)];
          val = val + k * (x1 - x4);
        }
        x1 = (l > 0) ? x[ijk_lin(i + 1, j, k, o)] : Z;
        x4 = x_row;
        val = val + l * (x1 - x4);
        out[row] = 0.5 * val;
        ++row;
      }
}

// BernsteinDerivativeMatrix_3D.jl:138-174 (fast_Ds_multiply!)
template <class V>
void fast_Ds(V* out, int N, const V* x, const Offsets& o) {
  const V Z = zero_of(x);
  int row = 0;
  for (int k = 0; k <= N; ++k)
    for (int j = 0; j <= N - k; ++j)
      for (int i = 0; i <= N - j - k; ++i) {
        int l = N - i - j - k;
        V val = Z;
        V x_row = x[row];
        V x2, x4;
        if (i > 0) {
          x2 = x[ijk_lin(i - 1, j + 1, k, o)];
          x4 = x[ijk_lin(i - 1, j, k, o)];
          val = val + i * (x2 - x4);
        }
        x2 = x_row;
        x4 = (j > 0) ? x[ijk_lin(i, j - 1, k, o)] : Z;
        val = val + j * (x2 - x4);
        if (k > 0) {
          x2 = x[ijk_lin(i, j + 1, k - 1, o)];
          x4 = x[ijk_lin(i, j, k - 1, o)];
          val = val + k * (x2 - x4);
        }
        x2 = (l > 0) ? x[ijk_lin(i, j + 1, k, o)] : Z;
        x4 = x_row;
        val = val + l * (x2 - x4);
        out[row] = 0.5 * val;
        ++row;
      }
}

// BernsteinDerivativeMatrix_3D.jl:180-216 (fast_Dt_multiply!)
template <class V>
void fast_Dt(V* out, int N, const V* x, const Offsets& o) {
  const V Z = zero_of(x);
  int row = 0;
  for (int k = 0; k <= N; ++k)
    for (int j = 0; j <= N - k; ++j)
      for (int i = 0; i <= N - j - k; ++i) {
        int l = N - i - j - k;
        V val = Z;
        V x_row = x[row];
        V x3, x4;
        if (i > 0) {
          x3 = x[ijk_lin(i - 1, j, k + 1, o)];
          x4 = x[ijk_lin(i - 1, j, k, o)];
          val = val + i * (x3 - x4);
        }
        if (j > 0) {
          x3 = x[ijk_lin(i, j - 1, k + 1, o)];
          x4 = x[ijk_lin(i, j - 1, k, o)];
          val = val + j * (x3 - x4);
        }
        x3 = x_row;
        x4 = (k > 0) ? x[ijk_lin(i, j, k - 1, o)] : Z;
        val = val + k * (x3 - x4);
        x3 = (l > 0) ? x[ijk_lin(i, j, k + 1, o)] : Z;
        x4 = x_row;
        val = val + l * (x3 - x4);
        out[row] = 0.5 * val;
        ++row;
      }
}

template <class V>
void fast_D(int axis, V* out, int N, const V* x, const Offsets& o) {
  if (axis == 0) fast_Dr(out, N, x, o);
  else if (axis == 1) fast_Ds(out, N, x, o);
  else fast_Dt(out, N, x, o);
}

// BernsteinLift.jl:66-90 (reduction_multiply!, degree N -> N-1). `out` may alias `x`:
// the reference applies it in place, which is safe because reads run ahead of writes.
template <class V>
void reduction_multiply(V* out, int N, const V* x, const Offsets& o) {
  int row = 0;
  for (int j = 0; j <= N - 1; ++j)
    for (int i = 0; i <= N - 1 - j; ++i) {
      int li1 = ij_lin(i + 1, j, o);
      int li2 = ij_lin(i, j + 1, o);
      int li3 = ij_lin(i, j, o);
      V val = (i + 1) * x[li1] + ((j + 1) * x[li2] + (N - i - j) * x[li3]);
      out[row] = val / N;
      ++row;
    }
}

// BernsteinLift.jl:100-125 (elevation_multiply!, degree N -> N+1)
template <class V>
void elevation_multiply(V* out, int N, const V* x, const Offsets& o) {
  const V Z = zero_of(x);
  int row = 0;
  for (int j = 0; j <= N + 1; ++j)
    for (int i = 0; i <= N + 1 - j; ++i) {
      int k = N + 1 - i - j;
      V val = Z;
      if (i > 0) val = i * x[ij_lin(i - 1, j, o)];
      if (j > 0) val = j * x[ij_lin(i, j - 1, o)] + val;
      if (k > 0) val = k * x[ij_lin(i, j, o)] + val;
      out[row] = val / (N + 1);
      ++row;
    }
}

// BernsteinLift.jl:139-164 (face_lift_multiply!). E holds np2(N) entries, F np2(N+1).
template <class V>
void face_lift_multiply(V* out, int N, const V* x, V* E, V* F) {
  const Offsets oN = make_offsets(N);
  const Offsets oN1 = make_offsets(N + 1);
  elevation_multiply(F, N, x, oN);
  reduction_multiply(E, N + 1, F, oN1);
  const double s = double((N + 1) * (N + 1)) / 2.0;
  const int n0 = np2(N);
  for (int i = 0; i < n0; ++i) E[i] = s * E[i];
  int index1 = n0;
  for (int i = 0; i < n0; ++i) out[i] = E[i];
  reduction_multiply(E, N, E, oN);
  for (int j = 1; j <= N; ++j) {
    int diff = ((N + 1 - j) * (N + 2 - j)) / 2;
    double lj = l_j(N, j);
    for (int i = 0; i < diff; ++i) out[index1 + i] = lj * E[i];
    if (j < N) {
      index1 += diff;
      reduction_multiply(E, N - j, E, make_offsets(N - j));
    }
  }
}

// BernsteinLift.jl:191-220 (mul! for one element; x holds the 4 face blocks f1..f4)
template <class V>
void lift_mul(V* out, int N, const V* x, V* E, V* F, V* G1, V* G2, V* G3) {
  const Offsets o = make_offsets(N);
  const int nf = np2(N);
  face_lift_multiply(out, N, x + 3 * nf, E, F);
  face_lift_multiply(G1, N, x + 0 * nf, E, F);
  face_lift_multiply(G2, N, x + 1 * nf, E, F);
  face_lift_multiply(G3, N, x + 2 * nf, E, F);
  int row = 0;
  for (int k = 0; k <= N; ++k)
    for (int j = 0; j <= N - k; ++j)
      for (int i = 0; i <= N - k - j; ++i) {
        int l = N - i - j - k;
        out[row] = out[row] + G1[ijk_lin(i, k, j, o)];
        out[row] = out[row] + G2[ijk_lin(j, k, l, o)];
        out[row] = out[row] + G3[ijk_lin(j, k, i, o)];
        ++row;
      }
}

// Scratch of one BernsteinLift{V} (BernsteinLift.jl:12-27).
template <class V>
struct LiftScratch {
  std::vector<V> E, F, G1, G2, G3;
  explicit LiftScratch(int N)
      : E(np2(N)), F(np2(N + 1)), G1(np3(N)), G2(np3(N)), G3(np3(N)) {}
};

// --------------------------------------------------------------------------------------
// Example right-hand sides. Geometry follows StartUpDG's MeshData for affine tetrahedra:
//   geo9[e*9 + m]  = (rxJ, sxJ, txJ, ryJ, syJ, tyJ, rzJ, szJ, tzJ)[m] of element e
//   nJ[(e*NfpT + i)*3 + c] = (nxJ, nyJ, nzJ)[c] at face node i of element e
//   Fmask[i]  volume index of face node i (i < 4*Nfp, faces in reference order)
//   mapP[e*NfpT + i] global face-node index of the neighbour node (e' * NfpT + i')
//   J  the constant Jacobian md.J[1,1]; Jall (may be null) the per-element Jacobian. The
//      examples divide by md.J[1,1] (3d_wave.jl:82-83: "md.J is constant" on their uniform
//      meshes); with Jall the division is by each element's own J, which is the same on a
//      uniform mesh and the right one on a mesh whose elements differ in size.
// --------------------------------------------------------------------------------------

// examples/3d_wave.jl:20-33
template <class T>
inline void wave_fluxes(const SV<T, 4>& q, SV<T, 4>& fx, SV<T, 4>& fy, SV<T, 4>& fz) {
  const T p = q.v[0], u = q.v[1], v = q.v[2], w = q.v[3];
  fx = SV<T, 4>{{u, p, T(0), T(0)}};
  fy = SV<T, 4>{{v, T(0), p, T(0)}};
  fz = SV<T, 4>{{w, T(0), T(0), p}};
}

// examples/3d_maxwell.jl:20-33
template <class T>
inline void maxwell_fluxes(const SV<T, 6>& q, SV<T, 6>& fx, SV<T, 6>& fy, SV<T, 6>& fz) {
  const T Hx = q.v[0], Hy = q.v[1], Hz = q.v[2], Ex = q.v[3], Ey = q.v[4], Ez = q.v[5];
  fx = SV<T, 6>{{T(0), Ez, -Ey, T(0), -Hz, Hy}};
  fy = SV<T, 6>{{-Ez, T(0), Ex, Hz, T(0), -Hx}};
  fz = SV<T, 6>{{Ey, -Ex, T(0), -Hy, Hx, T(0)}};
}

template <class T, int NF>
void rhs_example(int N, int K, const SV<T, NF>* q, SV<T, NF>* du, const int* Fmask,
                 const int64_t* mapP, const T* geo9, const T* nJ, T J, const T* Jall, T tau,
                 int nthreads) {
  const int Np = np3(N);
  const int NfpT = 4 * np2(N);
  const Offsets o = make_offsets(N);
  using V = SV<T, NF>;
  std::vector<V> uM((size_t)NfpT * K), flux((size_t)NfpT * K);

  // uM .= view(q, rd.Fmask, :)   (3d_wave.jl:41)
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int e = 0; e < K; ++e)
    for (int i = 0; i < NfpT; ++i) uM[(size_t)e * NfpT + i] = q[(size_t)e * Np + Fmask[i]];

  // interface flux loop (3d_wave.jl:43-56, 3d_maxwell.jl:43-65)
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int e = 0; e < K; ++e)
    for (int i = 0; i < NfpT; ++i) {
      const size_t gi = (size_t)e * NfpT + i;
      const V duM = uM[(size_t)mapP[gi]] - uM[gi];
      const T nx = nJ[gi * 3 + 0], ny = nJ[gi * 3 + 1], nz = nJ[gi * 3 + 2];
      // Penalty weights. tau <= 0: the examples' flux exactly as written (cp = cu = 1).
      // tau > 0: upwind penalty scaled by the face Jacobian Jf = |nJ| (cp = tau Jf,
      // cu = tau / Jf), the dimensionally consistent form of the same flux.
      T cp = T(1), cu = T(1);
      if (tau > T(0)) {
        const T Jf = std::sqrt(nx * nx + ny * ny + nz * nz);
        cp = tau * Jf;
        cu = tau / Jf;
      }
      V fl;
      if constexpr (NF == 1 || NF == 3) {
        // examples/3d_advec_scalar.jl:24-29 and 3d_advec.jl:44-45: upwind flux of
        // du/dt + du/dx = 0 with the face Jacobian Jf = |nJ| (written with Jf as the examples
        // do; tau does not enter), on the SVector (u, v, w) in 3d_advec.jl
        const T Jf = std::sqrt(nx * nx + ny * ny + nz * nz);
        (void)cp;
        (void)cu;
        for (int f = 0; f < NF; ++f) fl.v[f] = T(0.5) * duM.v[f] * nx - T(0.5) * duM.v[f] * Jf;
      } else if constexpr (NF == 4) {
        const T ndotdU = nx * duM.v[1] + ny * duM.v[2] + nz * duM.v[3];
        const T a = cp * duM.v[0] - ndotdU;
        const T b = cu * ndotdU - duM.v[0];
        fl.v[0] = T(0.5) * a;
        fl.v[1] = T(0.5) * (b * nx);
        fl.v[2] = T(0.5) * (b * ny);
        fl.v[3] = T(0.5) * (b * nz);
      } else {
        const T ndotdH = nx * duM.v[0] + ny * duM.v[1] + nz * duM.v[2];
        const T ndotdE = nx * duM.v[3] + ny * duM.v[4] + nz * duM.v[5];
        // fx(duM), fy(duM), fz(duM) as in 3d_maxwell.jl:20-33
        const T Hx = duM.v[0], Hy = duM.v[1], Hz = duM.v[2];
        const T Ex = duM.v[3], Ey = duM.v[4], Ez = duM.v[5];
        const T fxv[6] = {T(0), Ez, -Ey, T(0), -Hz, Hy};
        const T fyv[6] = {-Ez, T(0), Ex, Hz, T(0), -Hx};
        const T fzv[6] = {Ey, -Ex, T(0), -Hy, Hx, T(0)};
        const T nd[6] = {ndotdH * nx, ndotdH * ny, ndotdH * nz,
                         ndotdE * nx, ndotdE * ny, ndotdE * nz};
        for (int f = 0; f < NF; ++f)
          fl.v[f] = T(0.5) * fxv[f] * nx + T(0.5) * fyv[f] * ny + T(0.5) * fzv[f] * nz +
                    T(0.5) * (cp * duM.v[f]) - T(0.5) * (cu * nd[f]);
      }
      flux[gi] = fl;
    }

  // element loop (3d_wave.jl:58-80, 3d_maxwell.jl:67-89)
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<V> fxu(Np), fyu(Np), fzu(Np);
    std::vector<V> d[9];
    for (auto& dd : d) dd.resize(Np);
    LiftScratch<V> L(N);
#pragma omp for schedule(static)
    for (int e = 0; e < K; ++e) {
      const V* qe = q + (size_t)e * Np;
      for (int n = 0; n < Np; ++n) {
        if constexpr (NF == 1) {
          fxu[n] = qe[n];  // fx(u) = u, fy = fz = 0 (3d_advec_scalar.jl:33-35)
          fyu[n] = V{};
          fzu[n] = V{};
        } else if constexpr (NF == 3) {
          fxu[n] = V{};    // fx(q) = (u, 0, 0), fy = fz = 0 (3d_advec.jl:20-33)
          fxu[n].v[0] = qe[n].v[0];
          fyu[n] = V{};
          fzu[n] = V{};
        } else if constexpr (NF == 4) {
          wave_fluxes(qe[n], fxu[n], fyu[n], fzu[n]);
        } else {
          maxwell_fluxes(qe[n], fxu[n], fyu[n], fzu[n]);
        }
      }
      fast_Dr(d[0].data(), N, fxu.data(), o);
      fast_Ds(d[1].data(), N, fxu.data(), o);
      fast_Dt(d[2].data(), N, fxu.data(), o);
      fast_Dr(d[3].data(), N, fyu.data(), o);
      fast_Ds(d[4].data(), N, fyu.data(), o);
      fast_Dt(d[5].data(), N, fyu.data(), o);
      fast_Dr(d[6].data(), N, fzu.data(), o);
      fast_Ds(d[7].data(), N, fzu.data(), o);
      fast_Dt(d[8].data(), N, fzu.data(), o);
      V* due = du + (size_t)e * Np;
      lift_mul(due, N, flux.data() + (size_t)e * NfpT, L.E.data(), L.F.data(), L.G1.data(),
               L.G2.data(), L.G3.data());
      const T* g = geo9 + (size_t)e * 9;
      for (int i = 0; i < Np; ++i) {
        V vol = g[0] * d[0][i] + g[1] * d[1][i] + g[2] * d[2][i] + g[3] * d[3][i] +
                g[4] * d[4][i] + g[5] * d[5][i] + g[6] * d[6][i] + g[7] * d[7][i] +
                g[8] * d[8][i];
        if constexpr (NF == 4)
          due[i] = due[i] - vol;  // wave: du -= ... (3d_wave.jl:76)
        else
          due[i] = due[i] + vol;  // Maxwell: du += ... (3d_maxwell.jl:85); advection :38-40
      }
      if constexpr (NF == 1 || NF == 3)  // du = -du / J (3d_advec_scalar.jl:41, 3d_advec.jl:61)
        for (int i = 0; i < Np; ++i) due[i] = V::zero() - due[i];
      // du ./= J[1,1]  (3d_wave.jl:83), or the element's own J
      const T Je = Jall ? Jall[e] : J;
      for (int i = 0; i < Np; ++i) due[i] = due[i] / Je;
    }
  }
}

// Carpenter & Kennedy (1994) five-stage fourth-order 2N-storage coefficients.
const double RK4A[5] = {0.0, -567301805773.0 / 1357537059087.0,
                        -2404267990393.0 / 2016746695238.0,
                        -3550918686646.0 / 2091501179385.0,
                        -1275806237668.0 / 842570457699.0};
const double RK4B[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                        1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                        2277821191437.0 / 14882151754819.0};

template <class T, int NF>
void lsrk_run(int N, int K, SV<T, NF>* q, SV<T, NF>* res, const int* Fmask,
              const int64_t* mapP, const T* geo9, const T* nJ, T J, const T* Jall, T tau, T dt,
              int nsteps, int nthreads) {
  const size_t n = (size_t)np3(N) * K;
  std::vector<SV<T, NF>> rhs(n);
  for (int step = 0; step < nsteps; ++step)
    for (int s = 0; s < 5; ++s) {
      rhs_example<T, NF>(N, K, q, rhs.data(), Fmask, mapP, geo9, nJ, J, Jall, tau, nthreads);
      const T a = T(RK4A[s]), b = T(RK4B[s]);
#pragma omp parallel for num_threads(nthreads) schedule(static)
      for (long long m = 0; m < (long long)n; ++m)
        for (int f = 0; f < NF; ++f) {
          res[m].v[f] = a * res[m].v[f] + dt * rhs[m].v[f];
          q[m].v[f] = q[m].v[f] + b * res[m].v[f];
        }
    }
}

template <class T>
void deriv_matrix(int axis, int N, int K, const T* x, T* out) {
  // BernsteinDerivativeMatrix_3D.jl:222-231: column loop over elements.
  const Offsets o = make_offsets(N);
  const int Np = np3(N);
  for (int e = 0; e < K; ++e) fast_D(axis, out + (size_t)e * Np, N, x + (size_t)e * Np, o);
}

template <class T>
void lift_matrix(int N, int K, const T* x, T* out, int nthreads) {
  // BernsteinLift.jl:264-269: column loop over elements.
  const int Np = np3(N), NfpT = 4 * np2(N);
#pragma omp parallel num_threads(nthreads)
  {
    LiftScratch<T> L(N);
#pragma omp for schedule(static)
    for (int e = 0; e < K; ++e)
      lift_mul(out + (size_t)e * Np, N, x + (size_t)e * NfpT, L.E.data(), L.F.data(),
               L.G1.data(), L.G2.data(), L.G3.data());
  }
}

}  // namespace

extern "C" {

int oracle_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_offsets(int N, int* tri, int* tet) {
  Offsets o = make_offsets(N);
  for (int i = 0; i < 21; ++i) {
    tri[i] = o.tri[i];
    tet[i] = o.tet[i];
  }
}

double oracle_l_j(int N, int j) { return l_j(N, j); }

void oracle_deriv_f64(int axis, int N, int K, const double* x, double* out) {
  deriv_matrix<double>(axis, N, K, x, out);
}
void oracle_deriv_f32(int axis, int N, int K, const float* x, float* out) {
  deriv_matrix<float>(axis, N, K, x, out);
}
void oracle_elevation_f64(int N, const double* x, double* out) {
  elevation_multiply(out, N, x, make_offsets(N));
}
void oracle_reduction_f64(int N, const double* x, double* out) {
  reduction_multiply(out, N, x, make_offsets(N));
}
void oracle_face_lift_f64(int N, const double* x, double* out) {
  std::vector<double> E(np2(N)), F(np2(N + 1));
  face_lift_multiply(out, N, x, E.data(), F.data());
}
void oracle_lift_f64(int N, int K, const double* x, double* out, int nthreads) {
  lift_matrix<double>(N, K, x, out, nthreads);
}
void oracle_lift_f32(int N, int K, const float* x, float* out, int nthreads) {
  lift_matrix<float>(N, K, x, out, nthreads);
}

// phys: 0 = wave (4 fields), 1 = Maxwell (6 fields), 2 = scalar advection (1 field,
// examples/3d_advec_scalar.jl), 3 = three-component advection (3 fields, examples/3d_advec.jl).
// q/du are AoS Np x K of SVector{nf}.
int oracle_rhs_f64(int phys, int N, int K, const double* q, double* du, const int* Fmask,
                   const int64_t* mapP, const double* geo9, const double* nJ, double J,
                   const double* Jall, double tau, int nthreads) {
  if (phys == 0)
    rhs_example<double, 4>(N, K, (const SV<double, 4>*)q, (SV<double, 4>*)du, Fmask, mapP,
                           geo9, nJ, J, Jall, tau, nthreads);
  else if (phys == 2)
    rhs_example<double, 1>(N, K, (const SV<double, 1>*)q, (SV<double, 1>*)du, Fmask, mapP,
                           geo9, nJ, J, Jall, tau, nthreads);
  else if (phys == 3)
    rhs_example<double, 3>(N, K, (const SV<double, 3>*)q, (SV<double, 3>*)du, Fmask, mapP,
                           geo9, nJ, J, Jall, tau, nthreads);
  else if (phys == 1)
    rhs_example<double, 6>(N, K, (const SV<double, 6>*)q, (SV<double, 6>*)du, Fmask, mapP,
                           geo9, nJ, J, Jall, tau, nthreads);
  else
    return 1;
  return 0;
}
int oracle_rhs_f32(int phys, int N, int K, const float* q, float* du, const int* Fmask,
                   const int64_t* mapP, const float* geo9, const float* nJ, float J,
                   const float* Jall, float tau, int nthreads) {
  if (phys == 0)
    rhs_example<float, 4>(N, K, (const SV<float, 4>*)q, (SV<float, 4>*)du, Fmask, mapP, geo9, nJ, J, Jall, tau, nthreads);
  else if (phys == 2)
    rhs_example<float, 1>(N, K, (const SV<float, 1>*)q, (SV<float, 1>*)du, Fmask, mapP, geo9, nJ, J, Jall, tau, nthreads);
  else if (phys == 3)
    rhs_example<float, 3>(N, K, (const SV<float, 3>*)q, (SV<float, 3>*)du, Fmask, mapP, geo9, nJ, J, Jall, tau, nthreads);
  else if (phys == 1)
    rhs_example<float, 6>(N, K, (const SV<float, 6>*)q, (SV<float, 6>*)du, Fmask, mapP, geo9, nJ, J, Jall, tau, nthreads);
  else
    return 1;
  return 0;
}

int oracle_lsrk_f64(int phys, int N, int K, double* q, double* res, const int* Fmask,
                    const int64_t* mapP, const double* geo9, const double* nJ, double J,
                    const double* Jall, double tau, double dt, int nsteps, int nthreads) {
  if (phys == 0)
    lsrk_run<double, 4>(N, K, (SV<double, 4>*)q, (SV<double, 4>*)res, Fmask, mapP, geo9, nJ, J, Jall, tau, dt, nsteps, nthreads);
  else if (phys == 2)
    lsrk_run<double, 1>(N, K, (SV<double, 1>*)q, (SV<double, 1>*)res, Fmask, mapP, geo9, nJ, J, Jall, tau, dt, nsteps, nthreads);
  else if (phys == 3)
    lsrk_run<double, 3>(N, K, (SV<double, 3>*)q, (SV<double, 3>*)res, Fmask, mapP, geo9, nJ, J, Jall, tau, dt, nsteps, nthreads);
  else if (phys == 1)
    lsrk_run<double, 6>(N, K, (SV<double, 6>*)q, (SV<double, 6>*)res, Fmask, mapP, geo9, nJ, J, Jall, tau, dt, nsteps, nthreads);
  else
    return 1;
  return 0;
}
int oracle_lsrk_f32(int phys, int N, int K, float* q, float* res, const int* Fmask,
                    const int64_t* mapP, const float* geo9, const float* nJ, float J,
                    const float* Jall, float tau, float dt, int nsteps, int nthreads) {
  if (phys == 0)
    lsrk_run<float, 4>(N, K, (SV<float, 4>*)q, (SV<float, 4>*)res, Fmask, mapP, geo9, nJ, J, Jall,
                       tau, dt, nsteps, nthreads);
  else if (phys == 2)
    lsrk_run<float, 1>(N, K, (SV<float, 1>*)q, (SV<float, 1>*)res, Fmask, mapP, geo9, nJ, J, Jall,
                       tau, dt, nsteps, nthreads);
  else if (phys == 3)
    lsrk_run<float, 3>(N, K, (SV<float, 3>*)q, (SV<float, 3>*)res, Fmask, mapP, geo9, nJ, J, Jall,
                       tau, dt, nsteps, nthreads);
  else if (phys == 1)
    lsrk_run<float, 6>(N, K, (SV<float, 6>*)q, (SV<float, 6>*)res, Fmask, mapP, geo9, nJ, J, Jall,
                       tau, dt, nsteps, nthreads);
  else
    return 1;
  return 0;
}

}  // extern "C"

// Internal declarations shared by the bbdg CUDA translation units (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bbdg.h"

// ------------------------------------------------------------------------------------
// Exact q = it / d for 0 <= it < 2^32 / d (d >= 1) by a multiply-high with ceil(2^32 / d):
// the index loops divide a flat item number by runtime sizes on every iteration.
struct FastDiv {
  uint32_t m;
  int d;
  __host__ __device__ explicit FastDiv(int d_)
      : m(d_ > 1 ? (uint32_t)(0xFFFFFFFFull / (uint64_t)d_ + 1ull) : 0u), d(d_) {}
  __device__ __forceinline__ int div(int it) const {
    return d > 1 ? (int)__umulhi((uint32_t)it, m) : it;
  }
};

// ------------------------------------------------------------------------------------
// Degree bookkeeping. Multi-indices follow src/ordering.jl: 3D coefficients are ordered
// k (outer), j, i (inner); 2D coefficients j (outer), i (inner).
// ------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int np2(int n) { return n < 0 ? 0 : (n + 1) * (n + 2) / 2; }
__host__ __device__ __forceinline__ int np3(int n) {
  return n < 0 ? 0 : (n + 1) * (n + 2) * (n + 3) / 6;
}
// Row offset of row j in the degree-n triangle (ordering.jl:8-16, 0-based).
__host__ __device__ __forceinline__ int tri_off(int n, int j) { return j * (2 * n + 3 - j) / 2; }
// Layer offset of layer k in the degree-n tetrahedron (ordering.jl:18-26):
// sum_{m=1..k} T(n+2-m) = tet(n+1) - tet(n+1-k), T/tet the triangular/tetrahedral numbers.
__host__ __device__ __forceinline__ int tet_off(int n, int k) {
  const int a = n + 1, b = n + 1 - k;
  return (a * (a + 1) * (a + 2) - b * (b + 1) * (b + 2)) / 6;
}
__host__ __device__ __forceinline__ int ij2(int n, int i, int j) { return i + tri_off(n, j); }
// ordering.jl:32-35, 0-based.
__host__ __device__ __forceinline__ int ijk3(int n, int i, int j, int k) {
  return i + tri_off(n, j) + tet_off(n, k) - j * k;
}

// Face f's node (a, b) at distance d from the face (layer d), as a 3D index of degree N.
// f0: j=0 face (i,k,j) -> (a,d,b); f1: l=0 face (j,k,l); f2: i=0 face (j,k,i);
// f3: k=0 face (i,j,k). These are the permutations of src/BernsteinLift.jl:207-218.
__host__ __device__ __forceinline__ int face_vol(int N, int f, int a, int b, int d) {
  switch (f) {
    case 0: return ijk3(N, a, d, b);
    case 1: return ijk3(N, N - a - b - d, a, b);
    case 2: return ijk3(N, d, a, b);
    default: return ijk3(N, a, b, d);
  }
}

// Device-resident lookup tables of one degree, built once per context.
struct DegTables {
  int N = 0, Np = 0, NpM1 = 0, Nfp = 0;
  // word offsets inside `words` (uint32 units)
  int o_node3 = 0;   // Np   packed (i | j<<8 | k<<16), degree N
  int o_node3m1 = 0; // NpM1 packed, degree N-1
  int o_node2 = 0;   // np3(N+1) uint16 (a | b<<8), 2D decode of degrees 0..N+1; degree n
                     // starts at np3(n-1)
  int o_fvol = 0;    // 4*Nfp uint16: face node -> volume index
  int o_fperm = 0;   // 6*Nfp uint16: face node -> neighbour face node, per orientation
  int o_fstack = 0;  // 4*Np uint16: face f's lift stack entry (layer, node) -> volume index
  int o_sslot = 0;   // Np uint16: stage-kernel stack slot of lift-stack entry q (stack_slot<N>)
  int nwords = 0;
  uint32_t* d_words = nullptr;
};
// 32-bit words of the degree-N tables, the sum of the DegTables sections above in order
// (shared-memory sizes of a tile are computed from it before the tables exist).
inline int deg_table_words(int N) {
  return np3(N) + np3(N - 1) + (np3(N + 1) + 1) / 2 + (4 * np2(N) + 1) / 2 +
         (6 * np2(N) + 1) / 2 + (4 * np3(N) + 1) / 2 + (np3(N) + 1) / 2;
}

// Orientation codes: face vertex m of this side is face vertex PERMS[o][m] of the partner,
// PERMS = (0,1,2),(0,2,1),(1,0,2),(1,2,0),(2,0,1),(2,1,0), packed 2 bits per entry.
__host__ __device__ __forceinline__ int perm_of(int o, int m) {
  constexpr uint64_t kPack = (0ull << 0) | (1ull << 2) | (2ull << 4) |     // (0,1,2)
                             (0ull << 6) | (2ull << 8) | (1ull << 10) |    // (0,2,1)
                             (1ull << 12) | (0ull << 14) | (2ull << 16) |  // (1,0,2)
                             (1ull << 18) | (2ull << 20) | (0ull << 22) |  // (1,2,0)
                             (2ull << 24) | (0ull << 26) | (1ull << 28) |  // (2,0,1)
                             (2ull << 30) | (1ull << 32) | (0ull << 34);   // (2,1,0)
  return int((kPack >> (2 * (3 * o + m))) & 3u);
}

struct bb_ctx {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  std::string last_error;
  int64_t launches = 0;
  std::mutex mu;
  DegTables* tabs[BB_MAX_DEGREE + 2] = {};
  double* d_red = nullptr;     // reduction scratch (FP64 partials)
  size_t red_cap = 0;          // entries
  double* h_red = nullptr;     // pinned host mirror
  int* d_status = nullptr;     // device error word of the GEMM / closure kernels
  uint32_t wait_iters = 0;     // bound of the device-side mbarrier waits (0 = 2^24 polls)
  int test_fault = 0;          // test-only fault mode (bb_ctx_set_test_fault)
  int64_t config_epoch = 0;    // bumped when either changes: captured graphs are rebuilt
};

// Error helpers -----------------------------------------------------------------------
int bb_fail(bb_ctx* ctx, int code, const char* fmt, ...);
#define BB_CUDA(ctx, call)                                                        \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return bb_fail((ctx), BB_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Builds (or returns the cached) tables of degree N. Returns nullptr on failure.
const DegTables* bb_tables(bb_ctx* ctx, int N);
// The context's device error word (allocated on first use; nullptr on failure).
int* bb_ctx_status_word(bb_ctx* ctx);
// Degree-specialised FP32 lift (bbdg_lift_fast.cu): nfaces 4 or 1; -1 when N has none.
// Degree-specialised FP32 derivatives (bbdg_deriv_fast.cu, N <= 15): mask 1, 2, 4 or 7; -1 when
// none applies.
int bb_deriv_fast(bb_ctx* ctx, const DegTables* t, int64_t K, int mask, const void* x, void* o0,
                  void* o1, void* o2, cudaStream_t st);
int bb_lift_fast(bb_ctx* ctx, const DegTables* t, int64_t K, int nfaces, const void* x,
                 void* out, cudaStream_t st);
// Makes the context's device current.
int bb_set_device(bb_ctx* ctx);
// Checks a launch and counts it.
int bb_check_launch(bb_ctx* ctx, const char* what);
// Error for a nonzero device status word. Bit 0: a kernel found corrupt connectivity (a
// neighbour index or orientation out of range) and skipped the access; bit 1: a bounded
// device-side wait ran out and the kernel returned early; bit 2: a debug index check failed
// (debug builds only). A time-out takes precedence.
int bb_device_status_error(bb_ctx* ctx, int word);

// Debug index checks, compiled in with -DBB_DEBUG_CHECKS (the BBDG_DEBUG=1 build): a
// table-derived or neighbour index outside its range sets bit 2 of the status word and the
// access is skipped; nothing traps. Off in the normal build, where the tables are trusted.
#ifdef BB_DEBUG_CHECKS
#define BB_DCHECK(cond, status) ((cond) ? true : (atomicOr((status), 4), false))
#else
#define BB_DCHECK(cond, status) true
#endif

inline size_t dtype_size(int dtype) { return dtype == BB_F64 ? 8 : 4; }
// Fields of a physics code, 0 if unknown.
__host__ __device__ inline int physics_nf(int physics) {
  return physics == BB_WAVE ? 4 : physics == BB_MAXWELL ? 6 : physics == BB_ADVECTION ? 1
       : physics == BB_ADVECTION3 ? 3 : 0;
}
// Volume-term components of a physics (the advection examples have one: J du/dx).
__host__ __device__ inline int physics_nw(int physics) {
  return physics == BB_ADVECTION3 ? 1 : physics_nf(physics);
}
inline bool valid_dtype(int dtype) { return dtype == BB_F32 || dtype == BB_F64; }
inline bool valid_degree(int N) { return N >= 1 && N <= BB_MAX_DEGREE; }

// Shared-memory view of the degree tables, filled by load_tables().
struct SmemTables {
  const uint32_t* node3;
  const uint32_t* node3m1;
  const uint16_t* node2;
  const uint16_t* fvol;
  const uint16_t* fperm;
  const uint16_t* fstack;
};

// Shared-memory view of tables already copied to `s`.
__device__ __forceinline__ SmemTables tables_view(const DegTables& t, const uint32_t* s) {
  SmemTables r;
  r.node3 = s + t.o_node3;
  r.node3m1 = s + t.o_node3m1;
  r.node2 = reinterpret_cast<const uint16_t*>(s + t.o_node2);
  r.fvol = reinterpret_cast<const uint16_t*>(s + t.o_fvol);
  r.fperm = reinterpret_cast<const uint16_t*>(s + t.o_fperm);
  r.fstack = reinterpret_cast<const uint16_t*>(s + t.o_fstack);
  return r;
}

// Copies `words` 32-bit words of tables into shared memory (all threads participate).
__device__ __forceinline__ SmemTables load_tables(const DegTables& t, const uint32_t* g,
                                                  uint32_t* s) {
  for (int w = threadIdx.x; w < t.nwords; w += blockDim.x) s[w] = __ldg(g + w);
  SmemTables r;
  r.node3 = s + t.o_node3;
  r.node3m1 = s + t.o_node3m1;
  r.node2 = reinterpret_cast<const uint16_t*>(s + t.o_node2);
  r.fvol = reinterpret_cast<const uint16_t*>(s + t.o_fvol);
  r.fperm = reinterpret_cast<const uint16_t*>(s + t.o_fperm);
  r.fstack = reinterpret_cast<const uint16_t*>(s + t.o_fstack);
  return r;
}

template <class T>
struct VecOf;
template <>
struct VecOf<float> {
  using type = float4;
  static constexpr int width = 4;
};
template <>
struct VecOf<double> {
  using type = double2;
  static constexpr int width = 2;
};

// Block-cooperative copy of n elements global -> shared, 128-bit when both are aligned.
template <class T>
__device__ __forceinline__ void copy_g2s(T* __restrict__ s, const T* __restrict__ g, int n) {
  using V = typename VecOf<T>::type;
  constexpr int W = VecOf<T>::width;
  if ((((uintptr_t)g | (uintptr_t)s) & 15) == 0) {
    const int nv = n / W;
    const V* gv = reinterpret_cast<const V*>(g);
    V* sv = reinterpret_cast<V*>(s);
    for (int t = threadIdx.x; t < nv; t += blockDim.x) sv[t] = __ldg(gv + t);
    for (int t = nv * W + threadIdx.x; t < n; t += blockDim.x) s[t] = __ldg(g + t);
  } else {
    for (int t = threadIdx.x; t < n; t += blockDim.x) s[t] = __ldg(g + t);
  }
}

// Block-cooperative copy shared -> global.
template <class T>
__device__ __forceinline__ void copy_s2g(T* __restrict__ g, const T* __restrict__ s, int n) {
  using V = typename VecOf<T>::type;
  constexpr int W = VecOf<T>::width;
  if ((((uintptr_t)g | (uintptr_t)s) & 15) == 0) {
    const int nv = n / W;
    V* gv = reinterpret_cast<V*>(g);
    const V* sv = reinterpret_cast<const V*>(s);
    for (int t = threadIdx.x; t < nv; t += blockDim.x) gv[t] = sv[t];
    for (int t = nv * W + threadIdx.x; t < n; t += blockDim.x) g[t] = s[t];
  } else {
    for (int t = threadIdx.x; t < n; t += blockDim.x) g[t] = s[t];
  }
}

// Rounds a shared-memory byte offset up to 16 bytes.
__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// Rounded product (never fused into a following add), so that "out += w * v" gives the same
// bits whether the product is stored first or added at once.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// Small non-negative integers (0 <= v < 2^21) and reciprocals 1/n (1 <= n <= BB_MAX_DEGREE + 1)
// as T, with the values T(v) and T(1) / T(n) give. In double both stay off the FP64 pipe,
// GB300's scarcest unit (about 1 TFLOP/s), which a conversion or a division would otherwise
// occupy like the arithmetic: the integer is assembled in the binary64 fields with integer
// instructions (for v in [2^e, 2^(e+1)): biased exponent 1023 + e and the e bits below the
// leading one at the top of the fraction, exact since e <= 20), and 1/n is read from a table
// whose entries the compiler rounds as the IEEE division does. In float the plain
// conversion and division stay.
template <class T>
__device__ __forceinline__ T small_int(int v) {
  return T(v);
}
template <>
__device__ __forceinline__ double small_int<double>(int v) {
  const int e = 31 - __clz(v | 1);
  const uint32_t hi = ((uint32_t)(1023 + e) << 20) | (((uint32_t)v << (20 - e)) & 0xFFFFFu);
  return __hiloint2double(v ? (int)hi : 0, 0);
}
static __constant__ double kInvInt[BB_MAX_DEGREE + 2] = {
    0.0,       1.0 / 1,  1.0 / 2,  1.0 / 3,  1.0 / 4,  1.0 / 5,  1.0 / 6,  1.0 / 7,
    1.0 / 8,   1.0 / 9,  1.0 / 10, 1.0 / 11, 1.0 / 12, 1.0 / 13, 1.0 / 14, 1.0 / 15,
    1.0 / 16,  1.0 / 17, 1.0 / 18, 1.0 / 19, 1.0 / 20, 1.0 / 21};
static_assert(BB_MAX_DEGREE + 2 == 22, "kInvInt lists 1/n for n = 1 .. BB_MAX_DEGREE + 1");
template <class T>
__device__ __forceinline__ T inv_int(int n) {
  return T(1) / T(n);
}
template <>
__device__ __forceinline__ double inv_int<double>(int n) {
  return kInvInt[n];
}
// v / 2 for 0 <= v < 2^21 (double only): the fields of small_int with the exponent one lower.
__device__ __forceinline__ double half_int_f64(int v) {
  const int e = 31 - __clz(v | 1);
  const uint32_t hi = ((uint32_t)(1022 + e) << 20) | (((uint32_t)v << (20 - e)) & 0xFFFFFu);
  return __hiloint2double(v ? (int)hi : 0, 0);
}

// Weights of a sum that is halved at the end (the derivative rows): in double the weight is
// v / 2 and the final product by 1/2 is dropped (finish_half returns the sum); every partial
// sum is then exactly half of the unhalved one, so the bits are the same and the FP64 pipe
// does one product less per output. In float the weight is v and the sum is halved.
template <class T>
__device__ __forceinline__ T halved_weight(int v) {
  if constexpr (sizeof(T) == 8) return half_int_f64(v);
  else return small_int<T>(v);
}
template <class T>
__device__ __forceinline__ T finish_half(T v) {
  if constexpr (sizeof(T) == 8) return v;
  else return T(0.5) * v;
}

// L0 x at face node (i, j) of degree N, k = N - i - j: the 7-point stencil of
// (N+1)^2/2 R_{N+1} E_{N->N+1} (src/BernsteinLift.jl:100-125 then :66-90 with the L0
// scaling), x in the 2D layout of degree N with row offsets rb (row j), rbn (row j+1) and
// rbp (row j-1). Shared by the level-parallel and the chain-per-thread lifts. In double the
// halving is folded into the stencil weights (c/2 instead of a final product by 1/2): every
// partial sum is then exactly half of the unhalved one, so the bits are the same and the
// FP64 pipe does one product less per point.
template <class T>
__device__ __forceinline__ T l0_point(int i, int j, int k, const T* x, int rb, int rbn, int rbp) {
  constexpr bool H = sizeof(T) == 8;
  auto c = [](int v) -> T {
    if constexpr (H) return half_int_f64(v);
    else return small_int<T>(v);
  };
  T v = c((i + 1) * (i + 1) + (j + 1) * (j + 1) + (k + 1) * (k + 1)) * x[rb + i];
  if (j > 0) v = fma(c((i + 1) * j), x[rbp + i + 1], v);  // x(i+1, j-1)
  if (k > 0) v = fma(c((i + 1) * k), x[rb + i + 1], v);   // x(i+1, j)
  if (i > 0) v = fma(c((j + 1) * i), x[rbn + i - 1], v);  // x(i-1, j+1)
  if (k > 0) v = fma(c((j + 1) * k), x[rbn + i], v);      // x(i, j+1)
  if (i > 0) v = fma(c((k + 1) * i), x[rb + i - 1], v);   // x(i-1, j)
  if (j > 0) v = fma(c((k + 1) * j), x[rbp + i], v);      // x(i, j-1)
  if constexpr (H) return v;
  else return mul_rn(T(0.5), v);
}

// reduction_multiply! (src/BernsteinLift.jl:81-85) at output (i, j) from degree n, times a
// scale: ((i+1) x(i+1,j) + (j+1) x(i,j+1) + (n-i-j) x(i,j)) * scale (scale = 1/n is the
// reference's step; the lifts pass l_d / (l_{d-1} n) = -1/(d+1) to carry the layer weights).
template <class T>
__device__ __forceinline__ T reduce_point(int i, int j, int n, T x_ip, T x_jp, T x_0, T scale) {
  return fma(small_int<T>(i + 1), x_ip, fma(small_int<T>(j + 1), x_jp, small_int<T>(n - i - j) * x_0)) *
         scale;
}

// One face's recursive lift, accumulated into a shared-memory volume block, for `ne`
// elements and `nfld` fields at once (src/BernsteinLift.jl:139-164 applied per face and
// summed through the permutations of :207-218):
//   layer 0 += F_0 = L0 x (7-point stencil);  layer d += F_d = l_d E_d, E_d = R_{N-d+1} E_{d-1}
// with l_d carried by the recursion: l_d / l_{d-1} = -(N-d+1)/(d+1) and R_n divides by
// n = N-d+1, so F_d = -1/(d+1) [(i+1) F_{d-1}(i+1,j) + (j+1) F_{d-1}(i,j+1) + (n-i-j) F_{d-1}(i,j)]
// and no product by l_d is left per point.
// Level-parallel: one thread per output coefficient, a block barrier between levels, and
// two ping-pong buffers (the reference's in-place reduction is not parallel-safe).
//   in(le, fld)  : Nfp face coefficients at in + (le*in_es + fld*in_fs)
//   out(le, fld) : Np volume coefficients at out + (le*out_es + fld*out_fs)
//   bufA/bufB    : ne*nfld*np2(N) scratch each
// WAVE_N (the wave stage, nfld = 2): chain 0 lifts the pressure flux into out field 0 and
// chain 1 the scalar velocity flux s, whose lift goes to out fields 1, 2, 3 times this face's
// normal (nrm[le*BB_GEO_STRIDE + 0 / 4 / 8] = nx, ny, nz): the velocity flux is s n and
// the lift is linear, so one chain serves the three components.
// All threads of the block must call it.
template <class T, bool WAVE_N = false>
__device__ void lift_face_accumulate(int N, int f, int ne, int nfld, const uint16_t* node2,
                                     const T* in, int in_es, int in_fs, T* out, int out_es,
                                     int out_fs, T* bufA, T* bufB, const T* nrm = nullptr) {
  const int S = np2(N);
  const int nchain = ne * nfld;
  const FastDiv by_nfld(nfld);
  auto add = [&](int le, int fld, int v, T val) {
    T* o = out + le * out_es + fld * out_fs + v;
    if (WAVE_N && fld == 1) {
      const T* g = nrm + le * BB_GEO_STRIDE;
      o[0] = fma(g[0], val, o[0]);
      o[out_fs] = fma(g[4], val, o[out_fs]);
      o[2 * out_fs] = fma(g[8], val, o[2 * out_fs]);
    } else {
      o[0] += val;
    }
  };
  // level 0: the L0 stencil on the degree-N face values
  {
    const uint16_t* dec = node2 + np3(N - 1);
    const FastDiv by_s(S);
    for (int it = threadIdx.x; it < nchain * S; it += blockDim.x) {
      const int ch = by_s.div(it), m = it - ch * S;
      const int le = by_nfld.div(ch), fld = ch - le * nfld;
      const T* x = in + le * in_es + fld * in_fs;
      const int a = dec[m] & 0xff, b = dec[m] >> 8, c = N - a - b;
      const int rb = tri_off(N, b);
      const T e = l0_point<T>(a, b, c, x, rb, rb + (N + 1 - b), rb - (N + 2 - b));
      bufA[ch * S + m] = e;
      add(le, fld, face_vol(N, f, a, b, 0), e);
    }
  }
  __syncthreads();
  T* src = bufA;
  T* dst = bufB;
  for (int d = 1; d <= N; ++d) {
    const int n = N + 1 - d;         // input degree
    const int cnt = np2(n - 1);      // outputs
    const uint16_t* dec = node2 + np3(n - 2);
    const T cd = -inv_int<T>(d + 1);  // l_d / (l_{d-1} n)
    const FastDiv by_cnt(cnt);
    for (int it = threadIdx.x; it < nchain * cnt; it += blockDim.x) {
      const int ch = by_cnt.div(it), m = it - ch * cnt;
      const int le = by_nfld.div(ch), fld = ch - le * nfld;
      const int a = dec[m] & 0xff, b = dec[m] >> 8;
      const T* x = src + ch * S;
      const T val = reduce_point<T>(a, b, n, x[ij2(n, a + 1, b)], x[ij2(n, a, b + 1)],
                                    x[ij2(n, a, b)], cd);
      dst[ch * S + m] = val;
      add(le, fld, face_vol(N, f, a, b, d), val);
    }
    __syncthreads();
    T* tmp = src;
    src = dst;
    dst = tmp;
  }
}

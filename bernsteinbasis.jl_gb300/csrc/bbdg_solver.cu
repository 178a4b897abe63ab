// DG solver object: fused right-hand side + low-storage RK stage for the wave and Maxwell
// examples. The generic (runtime-degree) stage tile is in bbdg_stage_generic.cuh, the
// degree-specialised FP32 kernels in bbdg_stage_fast.cu; this file owns trace buffers,
// kernel selection, LSRK stepping and CUDA graphs.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "bbdg_internal.cuh"
#include "bbdg_stage_fast.cuh"
#include "bbdg_stage_generic.cuh"

namespace {

constexpr int kThreads = 256;

template <class T, int PHYS>
__global__ void __launch_bounds__(kThreads) stage_kernel(StageParams<T> P, TileLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SmemTables st =
      load_tables(P.tab, P.gtab, reinterpret_cast<uint32_t*>(smem + L.tab_bytes));
  const int64_t ntiles = P.tile_end > 0 ? P.tile_end : (P.K + P.epb - 1) / P.epb;
  for (int64_t tile = P.tile_begin + blockIdx.x; tile < ntiles; tile += gridDim.x)
    generic_stage_tile<T, PHYS>(P, L, st, tile);
}

// Writes every face trace (all faces) of elements [e_begin, e_end) of q into the trace buffer.
// An element's 4 NF Nfp trace entries are contiguous in the buffer; each block first decodes
// entry i into (field, volume node) once (shared table), then copies element after element:
// one table read, one gather from the element's field rows, one coalesced store per entry.
template <class T, int NF>
__global__ void extract_traces_kernel(DegTables tab, const uint32_t* __restrict__ gtab,
                                      int64_t K, const T* __restrict__ q, T* __restrict__ tr,
                                      int64_t e_begin, int64_t e_end) {
  extern __shared__ uint32_t s_src[];  // entry i: field << 16 | volume node
  const int Np = tab.Np, Nfp = tab.Nfp, W = 4 * NF * Nfp;
  const uint16_t* fvol = reinterpret_cast<const uint16_t*>(gtab + tab.o_fvol);
  for (int i = threadIdx.x; i < W; i += blockDim.x) {
    const int f = i / (NF * Nfp), rem = i - f * NF * Nfp, fld = rem / Nfp, a = rem - fld * Nfp;
    s_src[i] = ((uint32_t)fld << 16) | fvol[f * Nfp + a];
  }
  __syncthreads();
  const size_t field = (size_t)K * Np;
  for (int64_t e = e_begin + blockIdx.x; e < e_end; e += gridDim.x) {
    const T* qe = q + (size_t)e * Np;
    T* te = tr + (size_t)e * W;
    for (int i = threadIdx.x; i < W; i += blockDim.x) {
      const uint32_t v = s_src[i];
      te[i] = qe[(v >> 16) * field + (v & 0xffffu)];
    }
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
// bb_lsrk_run_host's schedule: the elements split into C ranges of whole tiles ("chunks"),
// uploaded in breadth-first order over the chunk neighbour graph; each LSRK stage runs chunk
// by chunk on its own stream, a chunk as soon as the previous stage has finished on every
// chunk that holds one of its elements' neighbours.
struct HostPlan {
  int epb = 0, C = 0;
  std::vector<int64_t> tb, eb;  // chunk c: tiles [tb[c], tb[c+1]), elements [eb[c], eb[c+1])
  std::vector<int> up;          // chunks in upload order
  std::vector<int> order[5];    // chunks in launch order, per stage
  std::vector<int> ready0;      // order[0][i] may run once uploads 0..ready0[i] are in
  std::vector<int> wait[5];     // order[s][i] (s >= 1) waits for launch wait[s][i] of stage s-1
  std::vector<cudaEvent_t> ev;  // 5 C stage launches, C uploads, start, middle, done
  cudaEvent_t& stage_ev(int s, int i) { return ev[(size_t)s * C + i]; }
  cudaEvent_t& up_ev(int p) { return ev[(size_t)5 * C + p]; }
  cudaEvent_t& start_ev() { return ev[(size_t)6 * C]; }
  cudaEvent_t& mid_ev() { return ev[(size_t)6 * C + 1]; }
  cudaEvent_t& done_ev() { return ev[(size_t)6 * C + 2]; }
};

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
  // bb_lsrk_run_host: upload and download streams, one stream per LSRK stage, the schedule
  cudaStream_t copy_stream = nullptr;
  cudaStream_t down_stream = nullptr;
  cudaStream_t stage_stream[5] = {};
  HostPlan* plan = nullptr;
  // graph cache: one graph per starting trace buffer parity
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  void* g_q = nullptr;
  void* g_res = nullptr;
  double g_dt = 0.0;
  int g_epb = 0;
  int64_t g_epoch = -1;  // the context's config_epoch the graphs were captured under
  // bb_lsrk_run_host's one-step schedule as a graph, for the buffers and dt it was made with
  cudaGraphExec_t host_graph = nullptr;
  const void* hg_in = nullptr;
  void* hg_out = nullptr;
  void* hg_q = nullptr;
  void* hg_res = nullptr;
  double hg_dt = 0.0;
  int hg_epb = 0;
  int64_t hg_epoch = -1;
};

namespace {

int solver_layout(bb_solver* s, int epb, size_t* smem_out, int* chain_out = nullptr) {
  TileLayout L;
  if (s->physics == BB_WAVE)
    L = s->dtype == BB_F64 ? tile_layout<double, BB_WAVE>(*s->tab, epb)
                           : tile_layout<float, BB_WAVE>(*s->tab, epb);
  else if (s->physics == BB_ADVECTION)
    L = s->dtype == BB_F64 ? tile_layout<double, BB_ADVECTION>(*s->tab, epb)
                           : tile_layout<float, BB_ADVECTION>(*s->tab, epb);
  else if (s->physics == BB_ADVECTION3)
    L = s->dtype == BB_F64 ? tile_layout<double, BB_ADVECTION3>(*s->tab, epb)
                           : tile_layout<float, BB_ADVECTION3>(*s->tab, epb);
  else
    L = s->dtype == BB_F64 ? tile_layout<double, BB_MAXWELL>(*s->tab, epb)
                           : tile_layout<float, BB_MAXWELL>(*s->tab, epb);
  *smem_out = L.total;
  if (chain_out) *chain_out = L.chain;
  return L.total <= s->ctx->smem_optin ? BB_OK : BB_ERR_ARG;
}

// tb, te: the launch covers tiles [tb, te) of the solver's tile size (te = 0: all tiles).
template <class T, int PHYS>
int launch_stage_t(bb_solver* s, int mode, int stage, double dt, void* q, void* res, void* rhs,
                   const void* tin, void* tout, cudaStream_t st, int64_t tb = 0,
                   int64_t te = 0) {
  bb_ctx* ctx = s->ctx;
  StageParams<T> P;
  P.tab = *s->tab;
  P.gtab = s->tab->d_words;
  P.K = s->K;
  P.tile_begin = tb;
  P.tile_end = te;
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
  const int64_t ntiles = (te > 0 ? te : (s->K + s->epb - 1) / s->epb) - tb;
  if (ntiles < 1) return bb_fail(ctx, BB_ERR_ARG, "empty tile range");
  int64_t grid = (int64_t)per_sm * ctx->num_sms;
  if (grid > ntiles) grid = ntiles;
  stage_kernel<T, PHYS><<<(int)grid, kThreads, L.total, st>>>(P, L);
  return bb_check_launch(ctx, "stage_kernel");
}

int launch_fast(bb_solver* s, int mode, int stage, double dt, void* q, void* res, void* rhs,
                const void* tin, void* tout, cudaStream_t st, int64_t tb = 0, int64_t te = 0) {
  FastStageParams P;
  const DegTables& t = *s->tab;
  P.gtab = t.d_words;
  P.o_node3 = t.o_node3;
  P.o_node3m1 = t.o_node3m1;
  P.o_fvol = t.o_fvol;
  P.o_fperm = t.o_fperm;
  P.o_sslot = t.o_sslot;
  P.K = s->K;
  P.tile_begin = tb;
  P.tile_end = te;
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
  fl.device = s->ctx->device;
  fl.wait_iters = s->ctx->wait_iters;
  fl.fault = s->ctx->test_fault;
  const int rc = bb_fast_launch(s->fast, fl, P, st);
  if (rc) return bb_fail(s->ctx, rc, "stage_fast_kernel launch: %s", cudaGetErrorString(cudaGetLastError()));
  s->ctx->launches++;
  return BB_OK;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

int launch_stage(bb_solver* s, int mode, int stage, double dt, void* q, void* res, void* rhs,
                 const void* tin, void* tout, cudaStream_t st, int64_t tb = 0, int64_t te = 0) {
  // the specialised kernels move tiles with 16-byte-aligned bulk copies and store q, res
  // and rhs with 16-byte vector stores
  if (s->fast >= 0 && aligned16(q) && (!res || aligned16(res)) && (!rhs || aligned16(rhs)) &&
      aligned16(s->geo) && aligned16(s->conn))
    return launch_fast(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te);
  if (s->physics == BB_WAVE)
    return s->dtype == BB_F64
               ? launch_stage_t<double, BB_WAVE>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te)
               : launch_stage_t<float, BB_WAVE>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te);
  if (s->physics == BB_ADVECTION)
    return s->dtype == BB_F64
               ? launch_stage_t<double, BB_ADVECTION>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te)
               : launch_stage_t<float, BB_ADVECTION>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te);
  if (s->physics == BB_ADVECTION3)
    return s->dtype == BB_F64
               ? launch_stage_t<double, BB_ADVECTION3>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te)
               : launch_stage_t<float, BB_ADVECTION3>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te);
  return s->dtype == BB_F64
             ? launch_stage_t<double, BB_MAXWELL>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te)
             : launch_stage_t<float, BB_MAXWELL>(s, mode, stage, dt, q, res, rhs, tin, tout, st, tb, te);
}

// Traces of elements [e0, e1) (e1 = -1: to the end).
int launch_extract(bb_solver* s, const void* q, void* tr, cudaStream_t st, int64_t e0 = 0,
                   int64_t e1 = -1) {
  if (e1 < 0) e1 = s->K;
  if (e1 <= e0) return BB_OK;
  int64_t grid = e1 - e0;
  if (grid > (int64_t)s->ctx->num_sms * 8) grid = (int64_t)s->ctx->num_sms * 8;
  const DegTables& t = *s->tab;
  const size_t smem = (size_t)4 * s->nf * t.Nfp * sizeof(uint32_t);
#define BB_EXTRACT(T_, NF_)                                                                \
  extract_traces_kernel<T_, NF_><<<(int)grid, 256, smem, st>>>(t, t.d_words, s->K,         \
                                                                (const T_*)q, (T_*)tr, e0, e1)
  if (s->dtype == BB_F64) {
    if (s->nf == 4) BB_EXTRACT(double, 4);
    else if (s->nf == 1) BB_EXTRACT(double, 1);
    else if (s->nf == 3) BB_EXTRACT(double, 3);
    else BB_EXTRACT(double, 6);
  } else {
    if (s->nf == 4) BB_EXTRACT(float, 4);
    else if (s->nf == 1) BB_EXTRACT(float, 1);
    else if (s->nf == 3) BB_EXTRACT(float, 3);
    else BB_EXTRACT(float, 6);
  }
#undef BB_EXTRACT
  return bb_check_launch(s->ctx, "extract_traces_kernel");
}

int check_status(bb_solver* s, cudaStream_t st) {
  int h = 0;
  BB_CUDA(s->ctx, cudaMemcpyAsync(&h, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  BB_CUDA(s->ctx, cudaStreamSynchronize(st));
  if (h) {
    cudaMemsetAsync(s->d_status, 0, sizeof(int), st);
    return bb_device_status_error(s->ctx, h);
  }
  return BB_OK;
}

void drop_graphs(bb_solver* s) {
  for (auto& g : s->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  if (s->host_graph) {
    cudaGraphExecDestroy(s->host_graph);
    s->host_graph = nullptr;
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
  if (physics_nf(physics) == 0)
    return bb_fail(ctx, BB_ERR_ARG,
                   "physics must be BB_WAVE, BB_MAXWELL, BB_ADVECTION or BB_ADVECTION3");
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
  s->nf = physics_nf(physics);
  s->conn = conn;
  s->geo = geo;
  s->tau = tau;
  s->tab = t;
  // default tile: the largest of 12, 6, 4, 2 elements whose tile runs the chain lift (FP32
  // tiles that fit its shared-memory budget); else, in this order, 4, 2, 6, 12 or 1 elements
  // within 100 KB (FP64 always lifts level-parallel: wave N = 9 takes 2 elements)
  const int cands[2][5] = {{12, 6, 4, 2, 0}, {4, 2, 6, 12, 1}};
  for (int pass = 0; pass < 2 && !s->epb; ++pass)
    for (int c : cands[pass]) {
      size_t sm = 0;
      int chain = 0;
      if (c > 0 && solver_layout(s, c, &sm, &chain) == BB_OK && sm <= 100 * 1024 &&
          (pass == 1 || chain)) {
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
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  if (s->down_stream) cudaStreamDestroy(s->down_stream);
  for (auto& x : s->stage_stream)
    if (x) cudaStreamDestroy(x);
  if (s->plan) {
    for (auto& e : s->plan->ev)
      if (e) cudaEventDestroy(e);
    delete s->plan;
  }
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

extern "C" int bb_stage_tile_bytes(int physics, int N, int dtype, int epb, int64_t* bytes,
                                   int* chain) {
  if (physics_nf(physics) == 0 || !valid_degree(N) || !valid_dtype(dtype) || epb < 1 ||
      epb > 64 || !bytes)
    return BB_ERR_ARG;
  const int nwords = deg_table_words(N);
  const int nf = physics_nf(physics);
  const TileLayout L = tile_layout_for(N, nf, physics_nw(physics), dtype_size(dtype), nwords, epb);
  *bytes = (int64_t)L.total;
  if (chain) *chain = L.chain;
  return BB_OK;
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

extern "C" int bb_solver_check(bb_solver* s, void* stream) {
  if (!s) return BB_ERR_ARG;
  int rc = bb_set_device(s->ctx);
  if (rc) return rc;
  return check_status(s, (cudaStream_t)stream);
}

namespace {

// nsteps LSRK steps from traces of q already current in trace buffer par0.
int run_steps(bb_solver* s, double dt, int nsteps, void* q, void* res, int use_graph,
              cudaStream_t st, int par0 = 0) {
  int rc = BB_OK;
  if (use_graph) {
    if (s->g_q != q || s->g_res != res || s->g_dt != dt || s->g_epb != s->epb ||
        s->g_epoch != s->ctx->config_epoch)
      drop_graphs(s);
    for (int par = 0; par < 2; ++par)
      if (!s->graph[par]) {
        rc = build_graph(s, dt, q, res, par);
        if (rc) return rc;
      }
    s->g_q = q;
    s->g_res = res;
    s->g_dt = dt;
    s->g_epb = s->epb;
    s->g_epoch = s->ctx->config_epoch;
    for (int step = 0; step < nsteps; ++step) {
      BB_CUDA(s->ctx, cudaGraphLaunch(s->graph[(par0 + step) & 1], st));
      s->ctx->launches += 5;
    }
  } else {
    for (int step = 0; step < nsteps; ++step) {
      rc = enqueue_step(s, dt, q, res, (par0 + step) & 1, st);
      if (rc) return rc;
    }
  }
  return BB_OK;
}

// bb_lsrk_run_host's streams, made on first use.
int ensure_host_streams(bb_solver* s) {
  cudaStream_t* all[7] = {&s->copy_stream, &s->down_stream, &s->stage_stream[0],
                          &s->stage_stream[1], &s->stage_stream[2], &s->stage_stream[3],
                          &s->stage_stream[4]};
  for (cudaStream_t* x : all)
    if (!*x && cudaStreamCreateWithFlags(x, cudaStreamNonBlocking) != cudaSuccess)
      return bb_fail(s->ctx, BB_ERR_CUDA, "stream creation failed");
  return BB_OK;
}

// bb_lsrk_run_host's schedule (HostPlan without its events) for K elements in tiles of epb,
// from a host copy of the packed connectivity: up to kHostMaxChunks chunks of at least 8
// tiles, the chunk neighbour graph (chunk c touches chunk d when an element of c has a face
// neighbour in d; entries that name no element, which the kernels report, add no edge), the
// upload order (breadth-first from chunk 0, lower chunks first) and the launch order and
// waits of each stage.
constexpr int kHostMaxChunks = BB_HOST_MAX_CHUNKS;
static_assert(kHostMaxChunks <= 64, "chunk neighbour sets are 64-bit masks");
void plan_schedule(int64_t K, int epb, const int32_t* conn, HostPlan* P) {
  const int64_t ntiles = (K + epb - 1) / epb;
  const int C = (int)std::min<int64_t>(kHostMaxChunks, std::max<int64_t>(1, ntiles / 8));
  P->epb = epb;
  P->C = C;
  P->tb.assign(C + 1, 0);
  P->eb.assign(C + 1, 0);
  for (int c = 0; c <= C; ++c) {
    P->tb[c] = ntiles * c / C;
    P->eb[c] = std::min<int64_t>(K, P->tb[c] * epb);
  }
  std::vector<uint64_t> nb(C, 0);  // neighbour chunks of each chunk (itself included)
  for (int c = 0; c < C; ++c) {
    nb[c] |= uint64_t(1) << c;
    for (int64_t e = P->eb[c]; e < P->eb[c + 1]; ++e)
      for (int f = 0; f < 4; ++f) {
        const int64_t n = conn[(size_t)e * 4 + f] >> 5;
        if (n < 0 || n >= K) continue;
        const int cn = (int)(std::upper_bound(P->eb.begin(), P->eb.end(), n) - P->eb.begin()) - 1;
        nb[c] |= uint64_t(1) << cn;
        nb[cn] |= uint64_t(1) << c;
      }
  }
  std::vector<int> pos(C, -1);
  P->up.clear();
  for (int root = 0; root < C; ++root) {
    if (pos[root] >= 0) continue;
    size_t head = P->up.size();
    pos[root] = (int)P->up.size();
    P->up.push_back(root);
    while (head < P->up.size()) {
      const int c = P->up[head++];
      for (int d = 0; d < C; ++d)
        if ((nb[c] >> d & 1) && pos[d] < 0) {
          pos[d] = (int)P->up.size();
          P->up.push_back(d);
        }
    }
  }
  // stage 0 (of a step fed by the uploads): a chunk may run once every neighbour chunk is in;
  // stage s: once stage s-1 has run on every neighbour chunk (its stream runs in order)
  std::vector<int> key(C), idx(C);
  auto sort_by = [&](std::vector<int>& order, const std::vector<int>& tie) {
    order.resize(C);
    for (int c = 0; c < C; ++c) order[c] = c;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
      return key[a] != key[b] ? key[a] < key[b] : tie[a] < tie[b];
    });
  };
  for (int c = 0; c < C; ++c) {
    key[c] = 0;
    for (int d = 0; d < C; ++d)
      if (nb[c] >> d & 1) key[c] = std::max(key[c], pos[d]);
  }
  sort_by(P->order[0], pos);
  P->ready0.resize(C);
  for (int i = 0; i < C; ++i) P->ready0[i] = key[P->order[0][i]];
  P->wait[0].assign(C, -1);
  for (int st = 1; st < 5; ++st) {
    for (int i = 0; i < C; ++i) idx[P->order[st - 1][i]] = i;
    for (int c = 0; c < C; ++c) {
      key[c] = 0;
      for (int d = 0; d < C; ++d)
        if (nb[c] >> d & 1) key[c] = std::max(key[c], idx[d]);
    }
    sort_by(P->order[st], idx);
    P->wait[st].resize(C);
    for (int i = 0; i < C; ++i) P->wait[st][i] = key[P->order[st][i]];
  }
}

// Builds (or keeps) bb_lsrk_run_host's schedule for the solver's tile size, with its events;
// the connectivity is read once from the device.
int build_host_plan(bb_solver* s) {
  if (s->plan && s->plan->epb == s->epb) return BB_OK;
  if (s->plan) {
    for (auto& e : s->plan->ev)
      if (e) cudaEventDestroy(e);
    delete s->plan;
    s->plan = nullptr;
  }
  HostPlan* P = new (std::nothrow) HostPlan();
  if (!P) return BB_ERR_NOMEM;
  std::vector<int32_t> conn;
  try {
    conn.resize((size_t)s->K * 4);
  } catch (const std::bad_alloc&) {
    delete P;
    return bb_fail(s->ctx, BB_ERR_NOMEM, "host schedule allocation failed");
  }
  if (cudaMemcpy(conn.data(), s->conn, conn.size() * sizeof(int32_t), cudaMemcpyDefault) !=
      cudaSuccess) {
    delete P;
    return bb_fail(s->ctx, BB_ERR_CUDA, "connectivity download failed");
  }
  try {
    plan_schedule(s->K, s->epb, conn.data(), P);
  } catch (const std::bad_alloc&) {
    delete P;
    return bb_fail(s->ctx, BB_ERR_NOMEM, "host schedule allocation failed");
  }
  const int C = P->C;
  P->ev.assign((size_t)6 * C + 3, nullptr);
  for (auto& e : P->ev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
      for (auto& x : P->ev)
        if (x) cudaEventDestroy(x);
      delete P;
      return bb_fail(s->ctx, BB_ERR_CUDA, "event creation failed");
    }
  s->plan = P;
  return BB_OK;
}

// Copies field slices of elements [e0, e1) between the device state and a host buffer.
int copy_range(bb_solver* s, char* dst, const char* src, int64_t e0, int64_t e1,
               cudaMemcpyKind kind, cudaStream_t st) {
  const size_t row = (size_t)s->tab->Np * dtype_size(s->dtype);
  for (int f = 0; f < s->nf; ++f) {
    const size_t off = ((size_t)f * s->K + e0) * row;
    BB_CUDA(s->ctx, cudaMemcpyAsync(dst + off, src + off, (size_t)(e1 - e0) * row, kind, st));
  }
  return BB_OK;
}

// One LSRK step chunk by chunk on the stage streams (HostPlan). par: the trace buffer the step
// starts from. upload: the chunks are first uploaded (copy_stream), and each one's traces are
// extracted as it lands; otherwise the traces are current and stage 0 is free to run.
// download: each chunk goes to hout as soon as its last stage is done.
//
// Every item (an upload, an extraction, a stage launch, a download) gets a level one above
// that of the item it waits for and of its predecessor on its stream, and the items are
// enqueued by level: CUDA maps streams onto a few hardware queues, and streams that share one
// then see the items in about the order they can run instead of stage after stage.
int host_plan_step(bb_solver* s, double dt, void* q, void* res, int par, bool upload,
                   bool download, const char* hin, char* hout) {
  HostPlan& P = *s->plan;
  const int C = P.C;
  enum { UP, EXTRACT, STAGE, DOWN };
  struct Item {
    int level, stream, seq, kind, stage, i;
  };
  // at most 8 C items (C <= kHostMaxChunks); levels of the uploads and stage launches
  std::array<Item, 8 * kHostMaxChunks> items;
  size_t nitems = 0;
  // streams: 0 uploads, 1..5 stages 0..4, 6 downloads
  std::array<int, kHostMaxChunks> lv_up{};
  std::array<int, 5 * kHostMaxChunks> lv_stage{};
  int seq = 0, last = -1;
  if (upload)
    for (int p = 0; p < C; ++p) {
      lv_up[p] = p;
      items[nitems++] = Item{p, 0, seq++, UP, 0, p};
    }
  int i = 0;
  last = -1;
  for (int p = 0; p < C; ++p) {
    if (upload) {
      last = std::max(last + 1, lv_up[p] + 1);
      items[nitems++] = Item{last, 1, seq++, EXTRACT, 0, p};
    }
    for (; i < C && (!upload || P.ready0[i] <= p); ++i) {
      last = last + 1;
      lv_stage[i] = last;
      items[nitems++] = Item{last, 1, seq++, STAGE, 0, i};
    }
  }
  for (int st = 1; st < 5; ++st) {
    last = -1;
    for (int j = 0; j < C; ++j) {
      last = std::max(last + 1, lv_stage[(size_t)(st - 1) * C + P.wait[st][j]] + 1);
      lv_stage[(size_t)st * C + j] = last;
      items[nitems++] = Item{last, 1 + st, seq++, STAGE, st, j};
    }
  }
  if (download) {
    last = -1;
    for (int j = 0; j < C; ++j) {
      last = std::max(last + 1, lv_stage[(size_t)4 * C + j] + 1);
      items[nitems++] = Item{last, 6, seq++, DOWN, 4, j};
    }
  }
  std::sort(items.begin(), items.begin() + nitems, [](const Item& a, const Item& b) {
    return a.level != b.level ? a.level < b.level
                              : a.stream != b.stream ? a.stream < b.stream : a.seq < b.seq;
  });
  cudaStream_t* ss = s->stage_stream;
  int waited[5] = {-1, -1, -1, -1, -1};
  for (size_t k = 0; k < nitems; ++k) {
    const Item& it = items[k];
    int rc = BB_OK;
    if (it.kind == UP) {
      const int c = P.up[it.i];
      rc = copy_range(s, static_cast<char*>(q), hin, P.eb[c], P.eb[c + 1], cudaMemcpyHostToDevice,
                      s->copy_stream);
      if (rc) return rc;
      BB_CUDA(s->ctx, cudaEventRecord(P.up_ev(it.i), s->copy_stream));
    } else if (it.kind == EXTRACT) {
      const int c = P.up[it.i];
      BB_CUDA(s->ctx, cudaStreamWaitEvent(ss[0], P.up_ev(it.i), 0));
      rc = launch_extract(s, q, s->trace[par], ss[0], P.eb[c], P.eb[c + 1]);
    } else if (it.kind == STAGE) {
      const int st = it.stage, c = P.order[st][it.i];
      if (st > 0 && P.wait[st][it.i] != waited[st]) {
        waited[st] = P.wait[st][it.i];
        BB_CUDA(s->ctx, cudaStreamWaitEvent(ss[st], P.stage_ev(st - 1, waited[st]), 0));
      }
      const int in = (par + st) & 1;
      rc = launch_stage(s, 1, st, dt, q, res, nullptr, s->trace[in], s->trace[in ^ 1], ss[st],
                        P.tb[c], P.tb[c + 1]);
      if (rc) return rc;
      BB_CUDA(s->ctx, cudaEventRecord(P.stage_ev(st, it.i), ss[st]));
    } else {
      const int c = P.order[4][it.i];
      BB_CUDA(s->ctx, cudaStreamWaitEvent(s->down_stream, P.stage_ev(4, it.i), 0));
      rc = copy_range(s, hout, static_cast<const char*>(q), P.eb[c], P.eb[c + 1],
                      cudaMemcpyDeviceToHost, s->down_stream);
    }
    if (rc) return rc;
  }
  return BB_OK;
}

}  // namespace

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
  return run_steps(s, dt, nsteps, q, res, use_graph, st);
}

namespace {

// Page-locked host memory (cudaHostAlloc / cudaHostRegister): copies from and to it can be
// captured into a graph.
bool pinned_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // the error of this query only
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Enqueues bb_lsrk_run_host's work (after the host plan and streams exist): every stream
// starts after the caller's earlier work on st, and st waits for the last download.
int enqueue_host_run(bb_solver* s, double dt, int nsteps, const void* q_host_in,
                     void* q_host_out, void* q_dev, void* res_dev, int use_graph, cudaStream_t st) {
  HostPlan& P = *s->plan;
  char* hout = static_cast<char*>(q_host_out);
  BB_CUDA(s->ctx, cudaEventRecord(P.start_ev(), st));
  BB_CUDA(s->ctx, cudaStreamWaitEvent(s->copy_stream, P.start_ev(), 0));
  BB_CUDA(s->ctx, cudaStreamWaitEvent(s->down_stream, P.start_ev(), 0));
  for (cudaStream_t x : s->stage_stream) BB_CUDA(s->ctx, cudaStreamWaitEvent(x, P.start_ev(), 0));
  int rc = host_plan_step(s, dt, q_dev, res_dev, 0, true, nsteps == 1,
                          static_cast<const char*>(q_host_in), hout);
  if (rc) return rc;
  if (nsteps > 1) {
    // the middle steps on the caller's stream once the first step is done everywhere
    BB_CUDA(s->ctx, cudaEventRecord(P.mid_ev(), s->stage_stream[4]));
    BB_CUDA(s->ctx, cudaStreamWaitEvent(st, P.mid_ev(), 0));
    rc = run_steps(s, dt, nsteps - 2, q_dev, res_dev, use_graph, st, 1);
    if (rc) return rc;
    BB_CUDA(s->ctx, cudaEventRecord(P.mid_ev(), st));
    for (cudaStream_t x : s->stage_stream) BB_CUDA(s->ctx, cudaStreamWaitEvent(x, P.mid_ev(), 0));
    rc = host_plan_step(s, dt, q_dev, res_dev, (nsteps - 1) & 1, false, true, nullptr, hout);
    if (rc) return rc;
  }
  BB_CUDA(s->ctx, cudaEventRecord(P.done_ev(), s->down_stream));
  BB_CUDA(s->ctx, cudaStreamWaitEvent(st, P.done_ev(), 0));
  return BB_OK;
}

}  // namespace

// Host state in and out, pipelined over element chunks (HostPlan): the uploads, each LSRK
// stage and the downloads run on their own streams, ordered by events only where the mesh
// couples the chunks, so the two copy directions overlap each other and the compute. With
// several steps the first runs chunk by chunk behind the uploads, the middle ones as whole
// launches (or the step graphs) on the caller's stream, and the last chunk by chunk ahead of
// the downloads. One step with use_graph set and pinned host buffers is captured once into a
// graph (per host and device buffers and dt) and replayed: one launch instead of a few
// hundred calls, and the graph, not the order of the streams, decides what runs side by side. The caller's stream
// waits for the last download, so the call stays stream-ordered.
extern "C" int bb_lsrk_run_host(bb_solver* s, double dt, int nsteps, const void* q_host_in,
                                void* q_host_out, void* q_dev, void* res_dev, int use_graph,
                                void* stream) {
  if (!s || !q_host_in || !q_host_out || !q_dev || !res_dev)
    return s ? bb_fail(s->ctx, BB_ERR_ARG, "null pointer") : BB_ERR_ARG;
  if (nsteps < 0 || !std::isfinite(dt)) return bb_fail(s->ctx, BB_ERR_ARG, "bad dt or nsteps");
  if (q_dev == res_dev) return bb_fail(s->ctx, BB_ERR_ARG, "res must not alias q");
  int rc = bb_set_device(s->ctx);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bytes = (size_t)s->nf * s->K * s->tab->Np * dtype_size(s->dtype);
  if (nsteps == 0) {
    BB_CUDA(s->ctx, cudaMemcpyAsync(q_dev, q_host_in, bytes, cudaMemcpyHostToDevice, st));
    BB_CUDA(s->ctx, cudaMemcpyAsync(q_host_out, q_dev, bytes, cudaMemcpyDeviceToHost, st));
    return BB_OK;
  }
  rc = ensure_host_streams(s);
  if (rc) return rc;
  rc = build_host_plan(s);
  if (rc) return rc;
  if (!use_graph || nsteps != 1 || !pinned_host(q_host_in) || !pinned_host(q_host_out))
    return enqueue_host_run(s, dt, nsteps, q_host_in, q_host_out, q_dev, res_dev, use_graph, st);
  if (s->host_graph &&
      (s->hg_in != q_host_in || s->hg_out != q_host_out || s->hg_q != q_dev ||
       s->hg_res != res_dev || s->hg_dt != dt || s->hg_epb != s->epb ||
       s->hg_epoch != s->ctx->config_epoch)) {
    cudaGraphExecDestroy(s->host_graph);
    s->host_graph = nullptr;
  }
  if (!s->host_graph) {
    cudaGraph_t g = nullptr;
    BB_CUDA(s->ctx, cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
    const int64_t launches = s->ctx->launches;
    rc = enqueue_host_run(s, dt, 1, q_host_in, q_host_out, q_dev, res_dev, 0, s->cap_stream);
    cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
    s->ctx->launches = launches;  // counted when the graph runs
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess)
      return bb_fail(s->ctx, BB_ERR_CUDA, "host-path capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->host_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      s->host_graph = nullptr;
      return bb_fail(s->ctx, BB_ERR_CUDA, "host-path instantiate: %s", cudaGetErrorString(e));
    }
    s->hg_in = q_host_in;
    s->hg_out = q_host_out;
    s->hg_q = q_dev;
    s->hg_res = res_dev;
    s->hg_dt = dt;
    s->hg_epb = s->epb;
    s->hg_epoch = s->ctx->config_epoch;
  }
  BB_CUDA(s->ctx, cudaGraphLaunch(s->host_graph, st));
  s->ctx->launches += 6 * s->plan->C;  // C trace extractions and 5 C stage launches
  return BB_OK;
}

// The schedule bb_lsrk_run_host uses for K elements in tiles of epb with this (host) packed
// connectivity; host-only. Arrays hold at least BB_HOST_MAX_CHUNKS (+1 for chunk_tiles)
// entries per row: chunk_tiles[c] = first tile of chunk c (chunk_tiles[C] = tile count),
// up = upload order, order[s*max + i] = i-th chunk stage s launches, ready0[i] = last upload
// position order[0][i] needs, wait[s*max + i] = launch of stage s-1 that order[s][i] waits for.
extern "C" int bb_host_schedule(int64_t K, int epb, const int32_t* conn_host, int* nchunks,
                                int64_t* chunk_tiles, int* up, int* order, int* ready0,
                                int* wait) {
  if (K < 1 || epb < 1 || !conn_host || !nchunks || !chunk_tiles || !up || !order || !ready0 ||
      !wait)
    return BB_ERR_ARG;
  HostPlan P;
  try {
    plan_schedule(K, epb, conn_host, &P);
  } catch (const std::bad_alloc&) {
    return BB_ERR_NOMEM;
  }
  const int C = P.C, M = BB_HOST_MAX_CHUNKS;
  *nchunks = C;
  for (int c = 0; c <= C; ++c) chunk_tiles[c] = P.tb[c];
  for (int i = 0; i < C; ++i) {
    up[i] = P.up[i];
    ready0[i] = P.ready0[i];
    for (int st = 0; st < 5; ++st) {
      order[st * M + i] = P.order[st][i];
      wait[st * M + i] = P.wait[st][i];
    }
  }
  return BB_OK;
}

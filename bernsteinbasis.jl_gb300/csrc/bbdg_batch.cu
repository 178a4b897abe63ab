// Batched persistent stage kernel: many independent wave / Maxwell problems of uneven
// degree N and element count K advance together.
//
// FP32 problems with a degree-specialised stage kernel for their (N, physics) and element
// count ("fast lanes") run that kernel, each problem its own persistent launch per stage on
// one of several side streams, so that small problems share the GPU. The other problems run
// the batched generic kernel: work items are (problem, element tile) pairs, numbered problem
// by problem; the blocks of a persistent grid draw items from a device counter (one 64-bit
// atomicAdd per item, no spinning) and run the generic stage tile (bbdg_stage_generic.cuh)
// for that problem, reloading the degree tables into shared memory only when the problem
// changes. Each problem keeps its own time step, tile shape, trace buffers and state; a step
// (5 stages of every lane + the counter reset, forked and joined by events) is replayed from
// a CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bbdg_internal.cuh"
#include "bbdg_stage_fast.cuh"
#include "bbdg_stage_generic.cuh"

namespace {

constexpr int kBatchThreads = 256;
constexpr int kSideStreams = 8;  // streams the fast lanes are spread over
const double kA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                      -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double kB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                      1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                      2277821191437.0 / 14882151754819.0};

template <class T>
struct BatchDesc {
  StageParams<T> P;      // rkA/rkB/trace pointers are filled in per stage by the kernel
  T* trace[2];
  int64_t tile_begin;    // first global work item of this problem
  int physics;
};

template <class T>
__global__ void __launch_bounds__(kBatchThreads, 3)
    batch_stage_kernel(const BatchDesc<T>* __restrict__ descs, int nprob, int64_t total,
                       unsigned long long* counter, int par, T rkA, T rkB) {
  extern __shared__ __align__(16) unsigned char smem[];
  // the current problem's parameters live in shared memory, not in registers
  __shared__ StageParams<T> sP;
  __shared__ TileLayout sL;
  __shared__ long long s_item, s_begin;
  __shared__ int s_prob, s_phys, s_reload;
  if (threadIdx.x == 0) s_prob = -1;
  while (true) {
    __syncthreads();  // every thread is done with the previous tile (and its tables)
    if (threadIdx.x == 0) {
      const long long item = (long long)atomicAdd(counter, 1ull);
      s_item = item;
      s_reload = 0;
      if (item < total) {
        int p = s_prob < 0 ? 0 : s_prob;  // items only grow, so the problem index only grows
        while (p + 1 < nprob && item >= descs[p + 1].tile_begin) ++p;
        if (p != s_prob) {
          const BatchDesc<T>& d = descs[p];
          sP = d.P;
          sP.rkA = rkA;
          sP.rkB = rkB;
          sP.trace_in = d.trace[par];
          sP.trace_out = d.trace[par ^ 1];
          s_phys = d.physics;
          s_begin = d.tile_begin;
          const int NF = physics_nf(d.physics);
          sL = tile_layout_for(d.P.tab.N, NF, NF, sizeof(T), d.P.tab.nwords, d.P.epb,
                               kBatchChainLiftBytes);
          s_prob = p;
          s_reload = 1;
        }
      }
    }
    __syncthreads();
    const int64_t item = s_item;
    if (item >= total) break;
    uint32_t* stab = reinterpret_cast<uint32_t*>(smem + sL.tab_bytes);
    if (s_reload) load_tables(sP.tab, sP.gtab, stab);
    const SmemTables st = tables_view(sP.tab, stab);
    if (s_phys == BB_WAVE)
      generic_stage_tile<T, BB_WAVE>(sP, sL, st, item - s_begin);  // starts with a barrier
    else if (s_phys == BB_MAXWELL)
      generic_stage_tile<T, BB_MAXWELL>(sP, sL, st, item - s_begin);
    else
      generic_stage_tile<T, BB_ADVECTION>(sP, sL, st, item - s_begin);
  }
}

template <class T, int NF>
__global__ void batch_extract_kernel(DegTables tab, const uint32_t* __restrict__ gtab, int64_t K,
                                     const T* __restrict__ q, T* __restrict__ tr) {
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

}  // namespace

struct bb_batch {
  bb_ctx* ctx = nullptr;
  int dtype = 0;
  std::vector<bb_batch_problem> probs;
  std::vector<const DegTables*> tabs;
  std::vector<int> epb;          // per problem
  std::vector<int> fast;         // per problem: specialised variant, -1 = generic kernel
  int nfast = 0, ngeneric = 0;
  std::vector<void*> trace;      // 2 per problem
  void* d_desc = nullptr;
  unsigned long long* d_counter = nullptr;  // 5 stage counters
  int* d_status = nullptr;
  int64_t total = 0;
  size_t smem = 0;
  int grid = 0;
  bool dirty = true;             // descriptors need rebuilding
  cudaStream_t cap = nullptr;
  cudaStream_t side[kSideStreams] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kSideStreams] = {};
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int64_t g_epoch = -1;  // the context's config_epoch the graphs were captured under
};

namespace {

int batch_tile_default(int N, int nf, int dtype) {
  // largest of 6, 4, 2, 1 elements whose generic tile fits in 100 KB of shared memory
  const int cands[4] = {6, 4, 2, 1};
  for (int e : cands) {
    const TileLayout L =
        tile_layout_for(N, nf, nf, dtype_size(dtype), deg_table_words(N), e, kBatchChainLiftBytes);
    if (L.total <= 100 * 1024) return e;
  }
  return 1;
}

void drop_batch_graphs(bb_batch* b) {
  for (auto& g : b->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

template <class T>
int build_desc(bb_batch* b) {
  bb_ctx* ctx = b->ctx;
  const int np = (int)b->probs.size();
  auto a16 = [](const void* x) { return ((uintptr_t)x & 15) == 0; };
  b->fast.assign(np, -1);
  b->nfast = b->ngeneric = 0;
  for (int p = 0; p < np; ++p) {
    const bb_batch_problem& pr = b->probs[p];
    if (sizeof(T) == 4 && a16(pr.q) && a16(pr.res) && a16(pr.geo) && a16(pr.conn)) {
      const int idx = bb_fast_find(pr.N, pr.physics, 0, 0, pr.K);
      int e = 0, th = 0;
      size_t sm = 0;
      if (idx >= 0 && bb_fast_variant_info(idx, &e, &th, &sm) == BB_OK && sm <= ctx->smem_optin)
        b->fast[p] = idx;
    }
    if (b->fast[p] >= 0) ++b->nfast;
  }
  std::vector<BatchDesc<T>> h;
  int64_t begin = 0;
  size_t smem = 0;
  for (int p = 0; p < np; ++p) {
    if (b->fast[p] >= 0) continue;
    const bb_batch_problem& pr = b->probs[p];
    const DegTables* t = b->tabs[p];
    h.push_back(BatchDesc<T>{});  // every field zero (the degree tables' own defaults)
    BatchDesc<T>& d = h.back();
    d.P.tab = *t;
    d.P.gtab = t->d_words;
    d.P.K = pr.K;
    d.P.epb = b->epb[p];
    d.P.mode = 1;
    d.P.dt = T(pr.dt);
    d.P.tau = T(pr.tau);
    d.P.q = (T*)pr.q;
    d.P.res = (T*)pr.res;
    d.P.geo = (const T*)pr.geo;
    d.P.conn = pr.conn;
    d.P.status = b->d_status;
    d.trace[0] = (T*)b->trace[2 * p];
    d.trace[1] = (T*)b->trace[2 * p + 1];
    d.tile_begin = begin;
    d.physics = pr.physics;
    begin += (pr.K + b->epb[p] - 1) / b->epb[p];
    const int nf = physics_nf(pr.physics);
    const TileLayout L = tile_layout_for(pr.N, nf, nf, sizeof(T), t->nwords, b->epb[p],
                                         kBatchChainLiftBytes);
    smem = std::max(smem, L.total);
  }
  b->ngeneric = (int)h.size();
  b->total = begin;
  b->smem = smem;
  if (h.empty()) {
    b->dirty = false;
    return BB_OK;
  }
  if (smem > ctx->smem_optin) return bb_fail(ctx, BB_ERR_ARG, "batch tiles exceed shared memory");
  if (!b->d_desc) {
    BB_CUDA(ctx, cudaMalloc(&b->d_desc, sizeof(BatchDesc<T>) * np));
  }
  BB_CUDA(ctx, cudaMemcpy(b->d_desc, h.data(), sizeof(BatchDesc<T>) * h.size(), cudaMemcpyHostToDevice));
  BB_CUDA(ctx, cudaFuncSetAttribute(batch_stage_kernel<T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  BB_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_stage_kernel<T>,
                                                             kBatchThreads, smem));
  if (per_sm < 1) return bb_fail(ctx, BB_ERR_ARG, "batch tile does not fit on an SM");
  b->grid = (int)std::min<int64_t>((int64_t)per_sm * ctx->num_sms, std::max<int64_t>(b->total, 1));
  b->dirty = false;
  return BB_OK;
}

// Stage s of a fast-lane problem: its specialised kernel, traces in buffer (par + s) & 1.
int launch_fast_lane(bb_batch* b, int p, int s, int par, cudaStream_t st) {
  const bb_batch_problem& pr = b->probs[p];
  const DegTables& t = *b->tabs[p];
  FastStageParams P{};
  P.gtab = t.d_words;
  P.o_node3 = t.o_node3;
  P.o_node3m1 = t.o_node3m1;
  P.o_fvol = t.o_fvol;
  P.o_fperm = t.o_fperm;
  P.o_sslot = t.o_sslot;
  P.K = pr.K;
  P.mode = 1;
  P.rkA = float(kA[s]);
  P.rkB = float(kB[s]);
  P.dt = float(pr.dt);
  P.tau = float(pr.tau);
  P.q = (float*)pr.q;
  P.res = (float*)pr.res;
  P.rhs = nullptr;
  const int in = (par + s) & 1;
  P.trace_in = (const float*)b->trace[2 * p + in];
  P.trace_out = (float*)b->trace[2 * p + (in ^ 1)];
  P.geo = (const float*)pr.geo;
  P.conn = pr.conn;
  P.status = b->d_status;
  FastLaunch fl;
  fl.num_sms = b->ctx->num_sms;
  fl.device = b->ctx->device;
  fl.wait_iters = b->ctx->wait_iters;
  fl.fault = b->ctx->test_fault;
  const int rc = bb_fast_launch(b->fast[p], fl, P, st);
  if (rc) return bb_fail(b->ctx, rc, "stage_fast_kernel launch: %s", cudaGetErrorString(cudaGetLastError()));
  b->ctx->launches++;
  return BB_OK;
}

template <class T>
int enqueue_batch_step(bb_batch* b, int par, cudaStream_t st) {
  bb_ctx* ctx = b->ctx;
  const int nside = std::min(b->nfast, kSideStreams);
  if (nside > 0) {  // fork: the fast lanes start with the step
    BB_CUDA(ctx, cudaEventRecord(b->fork_ev, st));
    for (int i = 0; i < nside; ++i) BB_CUDA(ctx, cudaStreamWaitEvent(b->side[i], b->fork_ev, 0));
    int j = 0;
    for (size_t p = 0; p < b->probs.size(); ++p) {
      if (b->fast[p] < 0) continue;
      cudaStream_t ss = b->side[j++ % nside];
      for (int s = 0; s < 5; ++s) {
        const int rc = launch_fast_lane(b, (int)p, s, par, ss);
        if (rc) return rc;
      }
    }
  }
  if (b->ngeneric > 0) {
    BB_CUDA(ctx, cudaMemsetAsync(b->d_counter, 0, 5 * sizeof(unsigned long long), st));
    for (int s = 0; s < 5; ++s) {
      batch_stage_kernel<T><<<b->grid, kBatchThreads, b->smem, st>>>(
          (const BatchDesc<T>*)b->d_desc, b->ngeneric, b->total, b->d_counter + s,
          (par + s) & 1, T(kA[s]), T(kB[s]));
      int rc = bb_check_launch(ctx, "batch_stage_kernel");
      if (rc) return rc;
    }
  }
  for (int i = 0; i < nside; ++i) {  // join
    BB_CUDA(ctx, cudaEventRecord(b->join_ev[i], b->side[i]));
    BB_CUDA(ctx, cudaStreamWaitEvent(st, b->join_ev[i], 0));
  }
  return BB_OK;
}

template <class T>
int batch_extract(bb_batch* b, cudaStream_t st) {
  for (size_t p = 0; p < b->probs.size(); ++p) {
    const bb_batch_problem& pr = b->probs[p];
    const DegTables& t = *b->tabs[p];
    const int nf = physics_nf(pr.physics);
    int64_t grid = (pr.K * 4 * nf * t.Nfp + 255) / 256;
    grid = std::min<int64_t>(std::max<int64_t>(grid, 1), (int64_t)b->ctx->num_sms * 8);
    if (nf == 4)
      batch_extract_kernel<T, 4><<<(int)grid, 256, 0, st>>>(t, t.d_words, pr.K, (const T*)pr.q,
                                                            (T*)b->trace[2 * p]);
    else if (nf == 1)
      batch_extract_kernel<T, 1><<<(int)grid, 256, 0, st>>>(t, t.d_words, pr.K, (const T*)pr.q,
                                                            (T*)b->trace[2 * p]);
    else
      batch_extract_kernel<T, 6><<<(int)grid, 256, 0, st>>>(t, t.d_words, pr.K, (const T*)pr.q,
                                                            (T*)b->trace[2 * p]);
    int rc = bb_check_launch(b->ctx, "batch_extract_kernel");
    if (rc) return rc;
  }
  return BB_OK;
}

template <class T>
int batch_run_t(bb_batch* b, int nsteps, int use_graph, cudaStream_t st) {
  bb_ctx* ctx = b->ctx;
  if (b->g_epoch != ctx->config_epoch) {
    drop_batch_graphs(b);
    b->g_epoch = ctx->config_epoch;
  }
  if (b->dirty) {
    drop_batch_graphs(b);
    int rc = build_desc<T>(b);
    if (rc) return rc;
  }
  int rc = batch_extract<T>(b, st);
  if (rc) return rc;
  if (!use_graph) {
    for (int step = 0; step < nsteps; ++step) {
      rc = enqueue_batch_step<T>(b, step & 1, st);
      if (rc) return rc;
    }
  } else {
    for (int par = 0; par < 2; ++par)
      if (!b->graph[par]) {
        cudaGraph_t g = nullptr;
        BB_CUDA(ctx, cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_batch_step<T>(b, par, b->cap);
        cudaError_t e = cudaStreamEndCapture(b->cap, &g);
        if (rc) {
          if (g) cudaGraphDestroy(g);
          return rc;
        }
        if (e != cudaSuccess) return bb_fail(ctx, BB_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph[par], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bb_fail(ctx, BB_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
      }
    for (int step = 0; step < nsteps; ++step) {
      BB_CUDA(ctx, cudaGraphLaunch(b->graph[step & 1], st));
      ctx->launches += 5;
    }
  }
  return BB_OK;
}

void free_batch(bb_batch* b) {
  drop_batch_graphs(b);
  for (void* p : b->trace) cudaFree(p);
  cudaFree(b->d_desc);
  cudaFree(b->d_counter);
  cudaFree(b->d_status);
  if (b->cap) cudaStreamDestroy(b->cap);
  for (int i = 0; i < kSideStreams; ++i) {
    if (b->side[i]) cudaStreamDestroy(b->side[i]);
    if (b->join_ev[i]) cudaEventDestroy(b->join_ev[i]);
  }
  if (b->fork_ev) cudaEventDestroy(b->fork_ev);
  delete b;
}

}  // namespace

extern "C" int bb_batch_create(bb_ctx* ctx, int nprob, const bb_batch_problem* probs, int dtype,
                               bb_batch** out) {
  if (!ctx || !out) return BB_ERR_ARG;
  *out = nullptr;
  if (nprob < 1 || !probs) return bb_fail(ctx, BB_ERR_ARG, "need at least one problem");
  if (!valid_dtype(dtype)) return bb_fail(ctx, BB_ERR_ARG, "bad dtype");
  int rc = bb_set_device(ctx);
  if (rc) return rc;
  bb_batch* b = new (std::nothrow) bb_batch();
  if (!b) return BB_ERR_NOMEM;
  b->ctx = ctx;
  b->dtype = dtype;
  for (int p = 0; p < nprob; ++p) {
    const bb_batch_problem& pr = probs[p];
    if (physics_nf(pr.physics) == 0 || pr.physics == BB_ADVECTION3 || !valid_degree(pr.N) || pr.K < 1 ||
        pr.K >= (int64_t(1) << 27) || !pr.conn || !pr.geo || !pr.q || !pr.res ||
        !std::isfinite(pr.dt) || !std::isfinite(pr.tau)) {
      free_batch(b);
      return bb_fail(ctx, BB_ERR_ARG, "bad problem %d", p);
    }
    const DegTables* t = bb_tables(ctx, pr.N);
    if (!t) {
      free_batch(b);
      return bb_fail(ctx, BB_ERR_NOMEM, "table allocation failed");
    }
    b->probs.push_back(pr);
    b->tabs.push_back(t);
    const int nf = physics_nf(pr.physics);
    b->epb.push_back(batch_tile_default(pr.N, nf, dtype));
    const size_t bytes = (size_t)pr.K * 4 * nf * t->Nfp * dtype_size(dtype);
    for (int k = 0; k < 2; ++k) {
      void* ptr = nullptr;
      if (cudaMalloc(&ptr, bytes) != cudaSuccess) {
        free_batch(b);
        return bb_fail(ctx, BB_ERR_NOMEM, "trace allocation failed");
      }
      b->trace.push_back(ptr);
    }
  }
  if (cudaMalloc(&b->d_counter, 5 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&b->d_status, sizeof(int)) != cudaSuccess ||
      cudaMemset(b->d_status, 0, sizeof(int)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) != cudaSuccess) {
    free_batch(b);
    return bb_fail(ctx, BB_ERR_NOMEM, "batch allocation failed");
  }
  for (int i = 0; i < kSideStreams; ++i)
    if (cudaStreamCreateWithFlags(&b->side[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join_ev[i], cudaEventDisableTiming) != cudaSuccess) {
      free_batch(b);
      return bb_fail(ctx, BB_ERR_NOMEM, "batch stream allocation failed");
    }
  *out = b;
  return BB_OK;
}

extern "C" int bb_batch_destroy(bb_batch* b) {
  if (!b) return BB_ERR_ARG;
  cudaSetDevice(b->ctx->device);
  free_batch(b);
  return BB_OK;
}

extern "C" int bb_batch_set_tile(bb_batch* b, int physics, int N, int elems_per_block) {
  if (!b) return BB_ERR_ARG;
  if (elems_per_block < 1 || elems_per_block > 64)
    return bb_fail(b->ctx, BB_ERR_ARG, "elements per block must be 1..64");
  const int nf = physics_nf(physics);
  if (!valid_degree(N) || nf == 0) return bb_fail(b->ctx, BB_ERR_ARG, "bad physics or degree");
  const TileLayout L = tile_layout_for(N, nf, nf, dtype_size(b->dtype), deg_table_words(N),
                                       elems_per_block, kBatchChainLiftBytes);
  if (L.total > b->ctx->smem_optin)
    return bb_fail(b->ctx, BB_ERR_ARG, "tile of %d elements exceeds shared memory", elems_per_block);
  int hits = 0;
  for (size_t p = 0; p < b->probs.size(); ++p)
    if (b->probs[p].physics == physics && b->probs[p].N == N) {
      b->epb[p] = elems_per_block;
      ++hits;
    }
  if (hits) b->dirty = true;
  return BB_OK;
}

extern "C" int bb_batch_get_tile(const bb_batch* b, int physics, int N, int* elems_per_block) {
  if (!b || !elems_per_block) return BB_ERR_ARG;
  for (size_t p = 0; p < b->probs.size(); ++p)
    if (b->probs[p].physics == physics && b->probs[p].N == N) {
      *elems_per_block = b->epb[p];
      return BB_OK;
    }
  return BB_ERR_ARG;
}

extern "C" int bb_batch_run(bb_batch* b, int nsteps, int use_graph, void* stream) {
  if (!b) return BB_ERR_ARG;
  if (nsteps < 0) return bb_fail(b->ctx, BB_ERR_ARG, "nsteps must be >= 0");
  int rc = bb_set_device(b->ctx);
  if (rc) return rc;
  if (nsteps == 0) return BB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  rc = b->dtype == BB_F64 ? batch_run_t<double>(b, nsteps, use_graph, st)
                          : batch_run_t<float>(b, nsteps, use_graph, st);
  if (rc) return rc;
  int h = 0;
  BB_CUDA(b->ctx, cudaMemcpyAsync(&h, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  BB_CUDA(b->ctx, cudaStreamSynchronize(st));
  if (h) {
    cudaMemsetAsync(b->d_status, 0, sizeof(int), st);
    return bb_device_status_error(b->ctx, h);
  }
  return BB_OK;
}

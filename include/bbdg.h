/*
 * bbdg.h -- C ABI of the GB300 (sm_103a) Bernstein DG hot path.
 *
 * Drop-in boundary for vincentxwang/BernsteinBasis.jl: the Julia operator types
 * (BernsteinDerivativeMatrix_3D_{r,s,t}, BernsteinLift) keep their mul! API and dispatch to
 * these entry points by ccall for device arrays; the examples' rhs_matvec! and time loop map
 * onto the solver entry points. Every function returns a bb_status (0 = success) and never
 * aborts; bb_ctx_last_error() describes the most recent failure on a context.
 *
 * Conventions
 *   - Array arguments are DEVICE pointers owned by the caller unless a name ends in _host.
 *   - Matrix operands keep the reference layout: one column per element, column-major,
 *     i.e. element e's Np (or 4*Nfp) coefficients are contiguous at offset e*Np.
 *   - Solver state is field-major structure-of-arrays: q[field][element][node], i.e. each
 *     field is the reference's Np x K matrix; fields are (p,u,v,w) for the wave equation and
 *     (Hx,Hy,Hz,Ex,Ey,Ez) for Maxwell, as in examples/3d_wave.jl and examples/3d_maxwell.jl.
 *   - dtype selects FP32 (BB_F32) or FP64 (BB_F64) storage and arithmetic.
 *   - Calls are ordered on the given cudaStream_t (passed as void*; NULL = legacy stream).
 *   - A context holds scratch, tables and CUDA graphs; use one context per host thread.
 */
#ifndef BBDG_H
#define BBDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  BB_OK = 0,
  BB_ERR_ARG = 1,       /* invalid argument (degree, size, null pointer, alignment, ...) */
  BB_ERR_CUDA = 2,      /* a CUDA runtime call failed */
  BB_ERR_TIMEOUT = 3,   /* a device-side bounded wait ran out */
  BB_ERR_NONFINITE = 4, /* NaN or Inf detected by a checked reduction */
  BB_ERR_STATE = 5,     /* call not valid in the object's current state */
  BB_ERR_NOMEM = 6,     /* device or host allocation failed */
  BB_ERR_DEVICE = 7     /* device-side check failed (corrupt connectivity, bad index) */
} bb_status;

typedef enum { BB_F32 = 0, BB_F64 = 1 } bb_dtype;
/* BB_WAVE: examples/3d_wave.jl (p, u, v, w); BB_MAXWELL: examples/3d_maxwell.jl
 * (Hx, Hy, Hz, Ex, Ey, Ez); BB_ADVECTION: examples/3d_advec_scalar.jl (u, du/dt + du/dx = 0,
 * upwind flux with the face Jacobian; tau does not enter, the generic kernel runs it);
 * BB_ADVECTION3: examples/3d_advec.jl (u, v, w with fx = (u, 0, 0): the same interface flux
 * on all three components, the volume term on u only; generic kernel, single solvers only,
 * not in batches). */
typedef enum { BB_WAVE = 0, BB_MAXWELL = 1, BB_ADVECTION = 2, BB_ADVECTION3 = 3 } bb_physics;
typedef enum { BB_AXIS_R = 0, BB_AXIS_S = 1, BB_AXIS_T = 2 } bb_axis;

#define BB_MAX_DEGREE 20
/* Per-element geometry record (bb_solver_create): rxJ sxJ txJ ryJ syJ tyJ rzJ szJ tzJ,
 * 1/J, J, (unused), nxJ[4], nyJ[4], nzJ[4] -- StartUpDG's md fields for affine tets. */
#define BB_GEO_STRIDE 24

typedef struct bb_ctx bb_ctx;
typedef struct bb_solver bb_solver;

/* ---- context ------------------------------------------------------------------------ */
int bb_version(void);
int bb_ctx_create(int device, bb_ctx** out);
int bb_ctx_destroy(bb_ctx* ctx);
const char* bb_ctx_last_error(const bb_ctx* ctx);
/* Number of kernels this context has launched (for launch accounting). */
int64_t bb_ctx_launch_count(const bb_ctx* ctx);

/* ---- reference-element operators, matrix form (one column per element) -------------- */

/* out = D x for D in {Dr, Ds, Dt} (axis 0/1/2).
 * Replaces LinearAlgebra.mul!(out, D::BernsteinDerivativeMatrix_3D_{r,s,t}, x::Matrix),
 * src/BernsteinDerivativeMatrix_3D.jl:222-231 (vector form :134,:176,:218 is K = 1). */
int bb_deriv_apply(bb_ctx* ctx, int axis, int N, int64_t K, int dtype, const void* x,
                   void* out, void* stream);

/* dr, ds, dt = Dr x, Ds x, Dt x from one read of x (fused form of the three calls above). */
int bb_grad_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x, void* dr,
                  void* ds, void* dt, void* stream);

/* out = L x with L the Bernstein lift [L1|L2|L3|L4]; x holds 4*Nfp face coefficients per
 * element (faces s=-1, r+s+t=-1, r=-1, t=-1).
 * Replaces LinearAlgebra.mul!(out, L::BernsteinLift, x), src/BernsteinLift.jl:191-220 and
 * the matrix form :264-269. */
int bb_lift_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* faces, void* out,
                  void* stream);

/* Single-face lift (Nfp -> Np per column). Replaces face_lift_multiply!,
 * src/BernsteinLift.jl:139-164 and its matrix form :174-179. */
int bb_face_lift_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x, void* out,
                       void* stream);

/* 2D degree elevation N -> N+1 and reduction N -> N-1, one column per face.
 * Replace elevation_multiply! (src/BernsteinLift.jl:100-125) and reduction_multiply!
 * (src/BernsteinLift.jl:66-90). */
int bb_elevation_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x, void* out,
                       void* stream);
int bb_reduction_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x, void* out,
                       void* stream);

/* Fused operator pass: dr, ds, dt = D{r,s,t} x and lift = L faces. In FP32 with N <= 15
 * this is two launches, the gradient kernel and then the lift kernel, whose results equal
 * bb_grad_apply and bb_lift_apply bitwise; otherwise (FP64, N > 15) one launch of the
 * table-driven fused kernel. */
int bb_fused_apply(bb_ctx* ctx, int N, int64_t K, int dtype, const void* x,
                   const void* faces, void* dr, void* ds, void* dt, void* lift, void* stream);

/* ---- DG solver (examples/3d_wave.jl, examples/3d_maxwell.jl) ------------------------- */

/* conn: K*4 int32, conn[e*4+f] = nbr << 5 | nbr_face << 3 | orientation (device).
 * geo:  K*BB_GEO_STRIDE values of the solver dtype (device).
 * tau <= 0: the examples' interface flux exactly as written; tau > 0: the same upwind
 * flux with its penalty scaled by the face Jacobian |nJ| (stable at dt ~ h/(N+1)^2).
 * Both arrays must stay alive and unchanged while the solver exists. */
int bb_solver_create(bb_ctx* ctx, int physics, int N, int64_t K, int dtype,
                     const int32_t* conn, const void* geo, double tau, bb_solver** out);
int bb_solver_destroy(bb_solver* s);
/* Elements per thread block and threads per block of the stage kernels (0 = default).
 * FP32 solvers of some degrees have degree-specialised kernels (whole lift chains in
 * registers, bulk-copy pipelined tiles); those need K to be a multiple of the tile. */
int bb_solver_set_tile(bb_solver* s, int elems_per_block, int threads);
int bb_solver_get_tile(const bb_solver* s, int* elems_per_block, int* threads);
/* Shared memory of one generic-kernel tile of epb elements (and whether it runs the
 * chain-per-thread lift), for tile choosers. */
int bb_stage_tile_bytes(int physics, int N, int dtype, int epb, int64_t* bytes, int* chain);
/* The idx-th compiled degree-specialised FP32 stage-kernel variant (idx = 0, 1, ...): its
 * degree, physics, elements per block and threads per block, for tile choosers; BB_ERR_ARG
 * past the last one. No counterpart in the reference (a tuning aid). */
int bb_fast_variant(int idx, int* N, int* physics, int* elems_per_block, int* threads);
/* kind 0: use a degree-specialised kernel when one exists (default); 1: generic kernel. */
int bb_solver_set_kernel(bb_solver* s, int kind);
/* 0 if a degree-specialised kernel is in use, 1 for the generic kernel. */
int bb_solver_get_kernel(const bb_solver* s);

/* rhs = RHS(q): one evaluation of rhs_matvec! (examples/3d_wave.jl:36-84,
 * examples/3d_maxwell.jl:36-93). */
int bb_rhs(bb_solver* s, const void* q, void* rhs, void* stream);

/* nsteps steps of 5-stage 4th-order low-storage Runge-Kutta, q and res updated in place.
 * res must start at zero or hold the previous step's residual (its first stage ignores it).
 * use_graph != 0 replays each step from a CUDA graph. */
int bb_lsrk_run(bb_solver* s, double dt, int nsteps, void* q, void* res, int use_graph,
                void* stream);

/* Reads and clears the solver's device status word (synchronises the stream): BB_OK, or
 * BB_ERR_TIMEOUT when a bounded device-side wait of its kernels ran out, BB_ERR_DEVICE when
 * a kernel found corrupt connectivity. bb_rhs checks it itself; bb_lsrk_run does not wait. */
int bb_solver_check(bb_solver* s, void* stream);

/* The same with host state: copies q_host_in to q_dev, advances, copies back to
 * q_host_out. Pipelined over up to 24 element ranges ("chunks") on solver-owned streams: one
 * for the uploads, one per LSRK stage, one for the downloads. A chunk's traces are extracted
 * as it lands, each stage runs on a chunk once the previous stage has finished on the chunks
 * holding its neighbours (read once from conn), and a chunk goes down as soon as its last
 * stage is done, so both copy directions overlap the compute; with several steps the middle
 * ones run as whole launches on `stream`. One step with use_graph set and page-locked host
 * buffers is captured into a graph on first use and replayed while the buffers, dt and tile
 * stay the same. The results are those of bb_lsrk_run. The call is
 * stream-ordered: `stream` waits for the last download. The host buffers must stay valid
 * until then; pinned host memory is needed for the copies to overlap. q_host_in and
 * q_host_out may be the same buffer. */
int bb_lsrk_run_host(bb_solver* s, double dt, int nsteps, const void* q_host_in,
                     void* q_host_out, void* q_dev, void* res_dev, int use_graph,
                     void* stream);

/* The chunk schedule of bb_lsrk_run_host for K elements in tiles of epb elements, from a
 * host copy of the packed connectivity (as bb_solver_create); host-only, no CUDA call.
 * *nchunks = C <= BB_HOST_MAX_CHUNKS. chunk_tiles[0..C]: chunk c is tiles
 * [chunk_tiles[c], chunk_tiles[c+1]). up[p]: the chunk uploaded p-th. order[s*BB_HOST_MAX_CHUNKS
 * + i]: the chunk LSRK stage s launches i-th. ready0[i]: the last upload position
 * order[0][i] needs (its traces extracted). wait[s*BB_HOST_MAX_CHUNKS + i] (s >= 1): the
 * launch index of stage s-1 that order[s][i] waits for (launches of one stage run in order;
 * -1 for s = 0). For a test or a tool that checks the schedule's dependencies. */
#define BB_HOST_MAX_CHUNKS 24
int bb_host_schedule(int64_t K, int epb, const int32_t* conn_host, int* nchunks,
                     int64_t* chunk_tiles, int* up, int* order, int* ready0, int* wait);

/* ---- StartUpDG MeshData import (host functions, no device work) -------------------------
 * conn_out[e*4+f] (the packed connectivity of bb_solver_create) from StartUpDG's
 * rd.Fmask (4*Nfp volume indices, faces in reference order) and md.mapP (K*4*Nfp global
 * face-node indices, element-major), both 0-based. Returns BB_ERR_ARG if a face side's nodes
 * do not all meet one partner face through one of the six face symmetries. */
int bb_conn_from_mapP(int N, int64_t K, const int32_t* Fmask, const int64_t* mapP,
                      int32_t* conn_out);
/* The geometry records of bb_solver_create (dtype BB_F32 or BB_F64, K*BB_GEO_STRIDE) from
 * per-element affine metric terms rst9[e*9 + m] = (rxJ, sxJ, txJ, ryJ, syJ, tyJ, rzJ, szJ,
 * tzJ)[m], face-constant scaled normals nJ[(e*4 + f)*3 + c] = (nxJ, nyJ, nzJ)[c] and J[e]. */
int bb_geo_from_meshdata(int64_t K, int dtype, const double* rst9, const double* nJ,
                         const double* J, void* geo_out);

/* ---- degree reduction --------------------------------------------------------------
 * FP64 L2 projection of degree-N Bernstein coefficients to degree M < N, per element and
 * field: c_M = M_MM^{-1} E_{M->N}^T M_NN c_N (Bernstein mass matrices of the reference
 * tetrahedron, E the degree elevation). in: [nf][K][Np(N)], out: [nf][K][Np(M)]; either
 * may be FP32 or FP64, arithmetic is FP64. No counterpart in the reference. */
int bb_project(bb_ctx* ctx, int N, int M, int64_t K, int nf, int dtype_in, const void* in,
               int dtype_out, void* out, void* stream);

/* ---- batched uneven solves ------------------------------------------------------------
 * Many independent wave / Maxwell problems of different degree N and element count K advance
 * together, each step replayed from a CUDA graph. FP32 problems with a degree-specialised
 * stage kernel for their (N, physics, K) run it on side streams (one persistent launch per
 * problem and stage); the others share one persistent launch per stage whose blocks draw
 * (problem, element tile) work items from a device counter. Each problem keeps its own time
 * step and penalty; the generic tile shape is chosen per (physics, N). No counterpart in
 * the reference, which solves one problem per script (examples/3d_wave.jl,
 * examples/3d_maxwell.jl). Arrays are device pointers in the batch dtype and must outlive
 * the batch object. */
typedef struct {
  int physics;          /* BB_WAVE, BB_MAXWELL or BB_ADVECTION */
  int N;                /* degree, 1..BB_MAX_DEGREE */
  int64_t K;            /* elements */
  const int32_t* conn;  /* K*4 packed connectivity (as bb_solver_create) */
  const void* geo;      /* K*BB_GEO_STRIDE geometry records */
  void* q;              /* [nf][K][Np] state, updated in place */
  void* res;            /* [nf][K][Np] LSRK register */
  double dt;            /* this problem's time step */
  double tau;           /* penalty mode, as bb_solver_create */
} bb_batch_problem;

typedef struct bb_batch bb_batch;
int bb_batch_create(bb_ctx* ctx, int nprob, const bb_batch_problem* probs, int dtype,
                    bb_batch** out);
int bb_batch_destroy(bb_batch* b);
/* Elements per work item for every problem with this physics and degree. */
int bb_batch_set_tile(bb_batch* b, int physics, int N, int elems_per_block);
int bb_batch_get_tile(const bb_batch* b, int physics, int N, int* elems_per_block);
/* nsteps LSRK steps of every problem; synchronises the stream to check device status. */
int bb_batch_run(bb_batch* b, int nsteps, int use_graph, void* stream);

/* ---- reductions (FP64 accumulation, warp-shuffle trees) ------------------------------ */

/* For each field f of nf fields laid out as [nf][K][Np]:
 *   out_host[3f+0] = sum a^2, out_host[3f+1] = sum (a-b)^2, out_host[3f+2] = sum b^2
 * (b may be NULL: then the last two are 0). Returns BB_ERR_NONFINITE if any sum is not
 * finite. Synchronises the stream. */
int bb_norms(bb_ctx* ctx, int N, int64_t K, int nf, int dtype, const void* a, const void* b,
             double* out_host, void* stream);

/* The sums of bb_norms written to a caller-provided DEVICE buffer out_dev (3*nf doubles,
 * same order), with no allocation and no context. It is for callers that cannot allocate
 * device memory: a host runtime whose device memory all belongs to its own pool allocator
 * (CUDA.jl's pool, PyTorch's caching allocator), where a hidden cudaMalloc competes with the
 * pool, and time-stepping loops that must not stall, since cudaFree synchronises the device.
 * No counterpart in the reference. Its scratch is a fixed file-scope device array
 * (512 blocks x 8 fields x 3 doubles = 96 KiB) that every GPU loading this library keeps
 * until exit; nf > 8 returns BB_ERR_ARG. The first call on a device (and the first after a
 * cudaDeviceReset) looks up that array's device address with cudaGetSymbolAddress, so make
 * that call before any stream capture. All calls share the array: calls that overlap on the
 * GPU (different streams, no ordering between them) race. Stream-ordered; does not
 * synchronise. A launch error it returns is its own, never one left by an earlier call. */
int bb_norms_noalloc(int N, int64_t K, int nf, int dtype, const void* a, const void* b,
                     double* out_dev, void* stream);

/* Mass-matrix energy: out_host[f] = sum_e J_e (a_e^T M a_e) with M the Bernstein mass
 * matrix of the reference tetrahedron; with b != NULL the quadratic form of (a - b).
 * J is read from the geometry records (stride BB_GEO_STRIDE, solver dtype). */
int bb_mass_norms(bb_ctx* ctx, int N, int64_t K, int nf, int dtype, const void* a,
                  const void* b, const void* geo, double* out_host, void* stream);

/* ---- learned per-element closure: BF16 tensor-core GEMM and MLP ---------------------
 * No counterpart in the reference. Matrices are row-major device arrays. */

/* C = alpha * A[M x K] * B[N x K]^T on the tensor cores (BF16 operands, FP32 accumulation),
 * then, per output element v (row r, column c):
 *   v += bias[c];  act 1: pre[r][c] = v (if pre), v = GELU(v);  act 2: v *= GELU'(pre[r][c])
 *   C_f32[r][c] = v; C_bf16[r][c] = bf16(v); CT_bf16[c][r] = bf16(v); bias_grad[c] += sum_r v
 * (every output optional, at least one given). A, B 16-byte aligned, K % 8 == 0; row-major
 * outputs use ldc >= N, the transposed one ldt >= M. kt_per > 0 splits K into chunks of
 * kt_per x 64 computed by different CTAs and added into C_f32 atomically (the caller zeroes it;
 * no other output allowed); 0 = no split. Stream-ordered; a pipeline wait that runs out sets
 * the context's device status word (bb_device_status). */
int bb_gemm_bf16(bb_ctx* ctx, int64_t M, int N, int K, const void* A, const void* B,
                 float alpha, const float* bias, int act, float* pre, float* C_f32,
                 void* C_bf16, void* CT_bf16, float* bias_grad, int ldc, int ldt, int kt_per,
                 void* stream);

/* Reads and clears the context's device status word (synchronises the stream); *out = 0 when
 * no kernel reported a problem, bit 0 = a corrupt connectivity entry, bit 1 = a wait ran out. */
int bb_device_status(bb_ctx* ctx, void* stream, int* out);

/* ---- bounded device-side waits ------------------------------------------------------
 * No counterpart in the reference (its loops run on the CPU). The bulk-copy pipelines of the
 * degree-specialised stage kernels, the FP32 lift and the tensor-core GEMM wait on mbarriers;
 * every such wait gives up after a bounded number of polls, sets a status bit, lets the
 * kernel's own copies in flight land (bounded) and returns, so the context stays usable. */

/* Polls before a device-side wait gives up, for kernels launched afterwards on this context
 * (captured solver and batch graphs are rebuilt); 0 = the default, 2^24 polls (about a
 * second). */
int bb_ctx_set_wait_limit(bb_ctx* ctx, uint32_t polls);
/* Test only: mode 1 makes the stage kernels' and the GEMM's copy issuers arm the barrier of
 * one bulk copy (the stage kernel: the copy issued during each block's second tile; the GEMM:
 * the second operand stage) without issuing it, so that the bounded wait on it runs out and
 * the time-out path can be checked; 0 = off (the default). Applies to launches made
 * afterwards. */
int bb_ctx_set_test_fault(bb_ctx* ctx, int mode);

/* out[c][r] = in[r][c] for a BF16 [rows x cols] matrix. */
int bb_transpose_bf16(bb_ctx* ctx, int64_t rows, int cols, const void* in, void* out,
                      void* stream);

/* MLP nin -> h1 -> h2 -> nout with GELU after the hidden layers (all widths multiples of 8),
 * BF16 weights and activations, FP32 accumulation, FP32 master parameters and Adam state.
 * Parameters are one flat FP32 vector: W1[h1][nin], b1[h1], W2[h2][h1], b2[h2],
 * W3[nout][h2], b3[nout]; weights start uniform in +-1/sqrt(fan_in) from `seed`, biases 0. */
typedef struct bb_mlp bb_mlp;
int bb_mlp_create(bb_ctx* ctx, int nin, int h1, int h2, int nout, int64_t max_batch,
                  uint64_t seed, bb_mlp** out);
int bb_mlp_destroy(bb_mlp* m);
int64_t bb_mlp_num_params(const bb_mlp* m);
int bb_mlp_set_params(bb_mlp* m, const float* host, void* stream);  /* resets Adam state */
int bb_mlp_get_params(bb_mlp* m, float* host, void* stream);
int bb_mlp_get_grads(bb_mlp* m, float* host, void* stream);
/* Y[B][nout] (FP32) = MLP(X[B][nin] BF16). train != 0 keeps the activations for bb_mlp_bwd
 * and needs XT = X^T ([nin][B] BF16, kept by the caller until bb_mlp_bwd) and B % 8 == 0. */
int bb_mlp_fwd(bb_mlp* m, int64_t B, const void* X, const void* XT, float* Y, int train,
               void* stream);
/* Gradients of L = 1/(B nout) sum (Y - T)^2 for the last training bb_mlp_fwd; writes L to
 * loss_dev (one device double). */
int bb_mlp_bwd(bb_mlp* m, int64_t B, const float* Y, const float* T, double* loss_dev,
               void* stream);
/* One Adam step (bias-corrected) with the stored gradients. */
int bb_mlp_step(bb_mlp* m, float lr, float beta1, float beta2, float eps, void* stream);

/* Closure features of every element of a degree-N, nf-field state q ([nf][K][Np], dtype):
 * X[e] = scale * ( q[0..nf)[e][0..Np) , for faces f = 0..3: the neighbour's nf x Nfp
 * coefficients on face f in this element's face ordering ) as BF16, nin = nf Np + 4 nf Nfp
 * (840 for Maxwell at N = 5); XT (optional) receives X^T. conn as bb_solver_create. */
int bb_closure_features(bb_ctx* ctx, int N, int64_t K, int nf, const int32_t* conn,
                        int dtype, const void* q, float scale, void* X, void* XT,
                        void* stream);
/* q[f][e][p] += alpha * Y[e][f Np + p] (Y FP32 [K][nf Np]). */
int bb_closure_apply(bb_ctx* ctx, int N, int64_t K, int nf, int dtype, float alpha,
                     const float* Y, void* q, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* BBDG_H */

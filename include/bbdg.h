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
typedef enum { BB_WAVE = 0, BB_MAXWELL = 1 } bb_physics;
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

/* Fused operator pass: dr, ds, dt = D{r,s,t} x and lift = L faces in one launch. */
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

/* The same with host state: copies q_host_in to q_dev, advances, copies back to
 * q_host_out (pinned host memory recommended). */
int bb_lsrk_run_host(bb_solver* s, double dt, int nsteps, const void* q_host_in,
                     void* q_host_out, void* q_dev, void* res_dev, int use_graph,
                     void* stream);

/* ---- degree reduction --------------------------------------------------------------
 * FP64 L2 projection of degree-N Bernstein coefficients to degree M < N, per element and
 * field: c_M = M_MM^{-1} E_{M->N}^T M_NN c_N (Bernstein mass matrices of the reference
 * tetrahedron, E the degree elevation). in: [nf][K][Np(N)], out: [nf][K][Np(M)]; either
 * may be FP32 or FP64, arithmetic is FP64. No counterpart in the reference. */
int bb_project(bb_ctx* ctx, int N, int M, int64_t K, int nf, int dtype_in, const void* in,
               int dtype_out, void* out, void* stream);

/* ---- batched uneven solves ------------------------------------------------------------
 * Many independent wave / Maxwell problems of different degree N and element count K advance
 * together: one persistent launch per LSRK stage whose blocks draw (problem, element tile)
 * work items from a device counter, each step replayed from a CUDA graph. Each problem keeps
 * its own time step and penalty; the tile shape is chosen per (physics, N). No counterpart in
 * the reference, which solves one problem per script (examples/3d_wave.jl,
 * examples/3d_maxwell.jl). Arrays are device pointers in the batch dtype and must outlive
 * the batch object. */
typedef struct {
  int physics;          /* BB_WAVE or BB_MAXWELL */
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
 * same order), without allocating anything and without a context: for callers that must not
 * allocate device memory -- code running while a CUDA graph is being captured on its stream,
 * runtimes whose device memory belongs to their own pool allocator, latency-bound loops.
 * No counterpart in the reference. Its scratch is a fixed file-scope device array
 * (512 blocks x 8 fields x 3 doubles = 96 KiB) that every GPU loading this library keeps
 * until exit; nf > 8 returns BB_ERR_ARG. The first call on a device looks up that array's
 * device address (cudaGetSymbolAddress), so make it before any stream capture. All calls
 * share the array: calls that overlap on the GPU (different streams, no ordering) race.
 * Stream-ordered; does not synchronise. */
int bb_norms_noalloc(int N, int64_t K, int nf, int dtype, const void* a, const void* b,
                     double* out_dev, void* stream);

/* Mass-matrix energy: out_host[f] = sum_e J_e (a_e^T M a_e) with M the Bernstein mass
 * matrix of the reference tetrahedron; with b != NULL the quadratic form of (a - b).
 * J is read from the geometry records (stride BB_GEO_STRIDE, solver dtype). */
int bb_mass_norms(bb_ctx* ctx, int N, int64_t K, int nf, int dtype, const void* a,
                  const void* b, const void* geo, double* out_host, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* BBDG_H */

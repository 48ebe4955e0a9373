/*
 * xpbd_gb300.h -- C ABI of the GB300-native RDC-XPBD substep (libxpbd_gb300.so).
 *
 * The reference (RaymondMcGuire/rdc-xpbd-taichi) exposes this path as the
 * Python class XPBDNeoHookeanSolver (xpbd_gpu/neohookean_solver.py:16-587)
 * over Taichi kernels; it has no FFI of its own.  Each entry point below
 * replaces one method of that class (cited beside it), so a Python host
 * binds them with ctypes and keeps the class interface.
 *
 * Conventions
 *  - Every function returns an int status (XPBD_OK == 0).
 *  - Device buffers are allocated by the caller (e.g. torch CUDA tensors) and
 *    passed as raw pointers; the library never frees them.  The library owns
 *    only a small per-solver block of device state (SDF table, FP64 Chebyshev
 *    state, per-iteration history), released by xpbd_destroy.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default
 *    stream.  All work is stream-ordered; no entry point synchronises unless
 *    it says so.
 *  - A handle is not thread-safe; separate handles are independent.
 *  - Vertex arrays are float4 per vertex: (x, y, z, w).  In x, p0 and p1 the w
 *    lane carries inv_m; in dx it carries the constraint count.
 */
#ifndef XPBD_GB300_H
#define XPBD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XPBD_ABI_VERSION 3

enum xpbd_status {
  XPBD_OK = 0,
  XPBD_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad enum */
  XPBD_ERR_CUDA = 2,             /* a CUDA runtime call failed */
  XPBD_ERR_NONFINITE = 3,        /* the residual reduction saw NaN/Inf */
  XPBD_ERR_NO_SDF = 4,           /* xpbd_base.py:66-67 raises ValueError */
  XPBD_ERR_BAD_MESH = 5,         /* index out of range / empty mesh */
  XPBD_ERR_HISTORY_FULL = 6,     /* more iterations than the history holds */
  XPBD_ERR_TIMEOUT = 7           /* a bounded device-side wait gave up */
};

/* sdf.py:60-124 */
enum xpbd_sdf_kind { XPBD_SDF_PLANE = 0, XPBD_SDF_SPHERE = 1, XPBD_SDF_CUBE = 2 };

/* Scatter variants of the Jacobi accumulation.
 *  ATOMIC: one thread per tet, four red.global.add.v4.f32 per tet.
 *  GATHER: per-corner contributions, then a deterministic vertex->tet CSR sum.
 *  PATCH:  one CTA per patch of P consecutive tets; the patch's vertex
 *          neighbourhood is staged in shared memory once.  Each thread
 *          projects tets_per_thread consecutive tets and merges the corners
 *          they share in registers before red.global.add.v4.f32 (or, with
 *          patch_reduce, contributions are summed per patch vertex in shared
 *          memory and one reduction is issued per patch vertex). */
enum xpbd_scatter { XPBD_SCATTER_ATOMIC = 0, XPBD_SCATTER_GATHER = 1, XPBD_SCATTER_PATCH = 2 };

/* One SDF obstacle (sdf.py:7-124).  48 bytes. */
typedef struct xpbd_sdf {
  int32_t kind;  /* xpbd_sdf_kind */
  int32_t fixed; /* SdfModel.fixed (sdf.py:10-11) */
  float a[3];    /* plane: point; sphere, cube: center */
  float b[3];    /* plane: unit normal; sphere: (radius, 0, 0); cube: half size */
  float vel[3];  /* SdfModel.vel (sdf.py:9); zero in the reference */
  float pad;
} xpbd_sdf;

/* Solver constants (neohookean_solver.py:18-77, xpbd_base.py:26-39). */
typedef struct xpbd_params {
  float lame_mu;                /* calc_second_lame (neohookean_solver.py:11-12) */
  float lame_lambda;            /* calc_first_lame (neohookean_solver.py:7-8) */
  float gravity[3];             /* xpbd_base.py:33-34 */
  float damping;                /* xpbd_base.py:35 */
  float hydrostatic_relaxation; /* split mode only (neohookean_solver.py:243) */
  float deviatoric_relaxation;  /* split mode only (neohookean_solver.py:183) */
  float cheb_gamma;             /* neohookean_solver.py:135 */
  int32_t cheb_enable;
  int32_t cheb_warmup;
  int32_t block_mode;           /* 1: block 2x2 solve, 0: split hydro + dev */
  int32_t constraints_iter;     /* Jacobi iterations per substep */
  int32_t monitor;              /* record mean |det F - 1|, |tr F^T F - 3| */
  int32_t precise_hydro;        /* 1: cancellation-free det F - 1, tr F^T F - 3 */
  int32_t scatter;              /* xpbd_scatter */
  int32_t use_graph;            /* 1: xpbd_solve replays a cached CUDA graph */
  int32_t sweep_order;          /* PATCH only: 1 = residual visits patches last-to-first */
  int32_t patch_pipeline;       /* PATCH only: 0 = one CTA per patch, 1 = persistent CTAs
                                   streaming tet records with cp.async.bulk */
  int32_t patch_reduce;         /* PATCH, pipeline 0: 1 = reduce per patch vertex in shared
                                   memory before the global reduction */
  int32_t tets_per_thread;      /* PATCH, pipeline 0, reduce 0: 0/1 = one tet per thread;
                                   2 or 4 = that many consecutive tets per thread, corners
                                   shared along the chain summed in registers */
  double rho_min, rho_max, rho_beta; /* neohookean_solver.py:66-68 */
  /* Stop mode (off when both are 0, the reference's fixed iteration count,
   * neohookean_solver.py:474): a substep ends after the first iteration k
   * whose residual (compute_xpbd_residual, :298-329) satisfies
   *   r_hat_k <= target_rel_residual * r_hat_0  or  r_hat_k <= residual_floor,
   * and after constraints_iter iterations at the most.  The positions are
   * those of a fixed-count run of k + 1 iterations.  Under xpbd_solve's
   * graph the remaining iterations launch nothing (a conditional WHILE node
   * of the frame graph loops over pairs of iterations); direct launches run
   * the cap and the kernels of stopped iterations return at once.  The
   * adjoint entry points reject it. */
  double target_rel_residual;
  double residual_floor;
} xpbd_params;

/* Caller-owned device buffers of one body (already in solver vertex/tet order). */
typedef struct xpbd_body {
  int32_t n_verts;
  int32_t n_tets;
  float* x;              /* [V][4] positions, w = inv_m */
  float* v;              /* [V][4] velocities */
  float* p0;             /* [V][4] predicted positions (ping), w = inv_m */
  float* p1;             /* [V][4] predicted positions (pong), w = inv_m */
  float* dx;             /* [V][4] Jacobi accumulator; must be zero at create */
  const int32_t* tets;   /* [T][4] vertex ids */
  const float* dm_a;     /* [T][4] inv_Dm[0][0..2], inv_Dm[1][0] */
  const float* dm_b;     /* [T][4] inv_Dm[1][1..2], inv_Dm[2][0..1] */
  const float* dm_c;     /* [T] inv_Dm[2][2] */
  const float* v0;       /* [T] rest volume V0 */
  float* lam;            /* [T][2] lambda_D, lambda_H */
  /* optional per-tet materials (ATOMIC / GATHER variants): 1 / mu and
   * 1 / lambda of every tet; NULL = the uniform lame_mu / lame_lambda */
  const float* tet_inv_mu;     /* [T] */
  const float* tet_inv_lambda; /* [T] */
  /* deterministic gather variant (XPBD_SCATTER_GATHER); may be NULL otherwise */
  const int32_t* v2t_offsets; /* [V+1] CSR row offsets */
  const int32_t* v2t_slots;   /* [4T] tet*4+corner, ascending per vertex */
  float* corner_dx;           /* [4T][4] per-corner contributions */
  /* solver vertex i is the caller's vertex vert_perm[i]; NULL = identity */
  const int32_t* vert_perm;   /* [V] */
  /* tile variant (XPBD_SCATTER_PATCH); may be NULL / 0 otherwise.  With it,
   * dm_a, dm_b, dm_c, lam and tet_lid hold n_patches * patch_tets entries
   * (zero padded past n_tets) so that every patch is copied whole.  Patch p is
   * tets [p*patch_tets, min((p+1)*patch_tets, T)); its vertices are
   * patch_verts[patch_voff[p] .. patch_voff[p+1]) (at most 256), and byte q of
   * tet_lid[t] is the patch-local index of corner q. */
  int32_t n_patches;
  int32_t patch_tets;         /* 64, 128 or 256 */
  const uint32_t* tet_lid;    /* [T] */
  const int32_t* patch_voff;  /* [n_patches+1] */
  const int32_t* patch_verts; /* [patch_voff[n_patches]] */
  /* patch-local vertex -> corner lists (xpbd_build_patch_csr): the corners of
   * patch vertex k are slots[p*4P + pv_start[k] .. next start) with slot =
   * 4 * (tet - p*P) + corner, ascending. */
  const uint16_t* pv_start;   /* [patch_voff[n_patches]] */
  const uint16_t* pv_slots;   /* [4 * n_patches * patch_tets] */
  /* 1: the tets were laid out by xpbd_pair_tets (two-tet units at positions
   * (2k, 2k+1), face pairs with aligned corners); the two-tets-per-thread
   * kernels then merge a face pair's shared corners without comparisons and
   * flush the other units' corners unmerged */
  int32_t tet_pairs;
} xpbd_body;

/* Vertex fields addressable by xpbd_import_vec3 / xpbd_export_vec3. */
enum xpbd_field { XPBD_FIELD_X = 0, XPBD_FIELD_V = 1, XPBD_FIELD_PRED_X = 2 };

int xpbd_abi_version(void);
const char* xpbd_status_string(int status);

/* Message of the last failure on the calling thread ("" if none). */
const char* xpbd_last_error(void);

/* Number of CUDA-visible devices (0 when none); never fails. */
int xpbd_device_count(void);

/* Constructor (neohookean_solver.py:18-77 after the mesh is on the device).
 * Copies the SDF list (xpbd_base.py:60-70) and allocates the solver state.
 * `max_records` = iterations the per-frame history can hold. */
int xpbd_create(const xpbd_params* params, const xpbd_body* body, const xpbd_sdf* sdfs,
                int32_t n_sdf, int32_t max_records, void** out_handle);
int xpbd_destroy(void* handle);

/* Replace the SDF table contents (same count as at create); synchronises
 * `stream` first so that no queued kernel sees a partial table. */
int xpbd_set_sdfs(void* handle, const xpbd_sdf* sdfs, int32_t n_sdf, void* stream);

/* Replace constants (e.g. after the host changed damping); resets cached graphs. */
int xpbd_set_params(void* handle, const xpbd_params* params);

/* apply_external_forces (xpbd_base.py:139-146): p = x + (v += g dt) dt. */
int xpbd_apply_external_forces(void* handle, float dt, void* stream);

/* solve_sdf_collision (xpbd_base.py:162-178) on the predicted positions. */
int xpbd_solve_sdf_collision(void* handle, float dt, void* stream);

/* solve_step (neohookean_solver.py:453-560): lambda reset, SDF projection,
 * constraints_iter Jacobi iterations with residual-driven Chebyshev.
 * Per-iteration records go to history rows [record_base, record_base+iters). */
int xpbd_solve_step(void* handle, float dt, int32_t record_base, void* stream);

/* advance (xpbd_base.py:148-160). */
int xpbd_advance(void* handle, float dt, float damping, void* stream);

/* One substep = apply_external_forces + solve_step + advance, with predict and
 * SDF projection fused into one vertex pass (neohookean_solver.py:577-579). */
int xpbd_substep(void* handle, float dt, int32_t record_base, void* stream);

/* solve (neohookean_solver.py:562-587): one frame, chunked by dt in float64,
 * replayed from a cached CUDA graph. */
int xpbd_solve(void* handle, double frame_dt, double dt, int32_t substeps, void* stream);

/* Copy history rows [0, n) as {r_hat, omega, hydro_error, dev_error} doubles
 * to host memory; synchronises `stream`. */
int xpbd_read_history(void* handle, double* host_out, int32_t n, void* stream);

/* Jacobi iterations run by substeps [0, n) of the last frame (or, for
 * xpbd_substep / xpbd_solve_step, by the substep whose record_base is
 * s * constraints_iter); n <= 256.  `total` (may be NULL) receives the
 * iterations run since xpbd_create by the substeps that summed a residual
 * (Chebyshev, monitoring or stop mode).  Synchronises `stream`.  No
 * counterpart in the reference, whose iteration count is fixed. */
int xpbd_read_iterations(void* handle, int32_t* host_out, int32_t n, int64_t* total, void* stream);

/* Spectral-radius estimate rho_hat (neohookean_solver.py:65, persists across
 * substeps); get synchronises `stream`. */
int xpbd_get_rho_hat(void* handle, double* out, void* stream);
int xpbd_set_rho_hat(void* handle, double value, void* stream);

/* Device-to-device transfer of a vertex field in the caller's vertex order
 * ([V][3] floats), permuting through vert_perm: the Taichi field accessors
 * mesh.verts.<f>.from_numpy / .to_numpy (xpbd_base.py:54, renderer.py:49).
 * Importing XPBD_FIELD_X keeps inv_m in the w lane. */
int xpbd_import_vec3(void* handle, int32_t field, const float* src, void* stream);
int xpbd_export_vec3(void* handle, int32_t field, float* dst, void* stream);

/* Kernel classes for xpbd_read_profile. */
enum xpbd_kernel_class {
  XPBD_K_BEGIN = 0,    /* predict + SDF (V) */
  XPBD_K_PROJECT = 1,  /* Neo-Hookean projection + Jacobi scatter (T) */
  XPBD_K_GATHER = 2,   /* deterministic vertex gather (V) */
  XPBD_K_RESIDUAL = 3, /* residual / monitoring sweep + FP64 scalars (T) */
  XPBD_K_UPDATE = 4,   /* post_solve + Chebyshev mix (V) */
  XPBD_K_END = 5,      /* advance (V) */
  XPBD_K_COUNT = 6
};

/* Profiling: with `enable`, every kernel launch is bracketed by CUDA events
 * on its stream.  With use_graph, xpbd_solve replays a frame graph that
 * carries those events as event record nodes, and waits for the previous
 * profiled replay before launching the next; without it the launches are
 * direct.  (The reference's counterpart is the host perf_counter brackets of
 * solve_step, neohookean_solver.py:454-560.) */
int xpbd_set_profiling(void* handle, int32_t enable);

/* L2 eviction policy of the read-only tet records in the tile (PATCH)
 * sweeps.  mode -1: automatic, the default: evict_last when the records and
 * the per-iteration state fit in 80% of the device's L2, else plain loads;
 * 0: plain loads; 1: evict_last.  `active` (may be NULL) receives the
 * policy in force (0 or 1).  Results do not depend on it.  No counterpart in
 * the reference (Taichi leaves caching to the hardware). */
int xpbd_set_l2_hint(void* handle, int32_t mode, int32_t* active);

/* Accumulated device milliseconds and launch counts per kernel class
 * (arrays of n <= XPBD_K_COUNT); synchronises `stream`; `reset` clears. */
int xpbd_read_profile(void* handle, double* ms, int64_t* launches, int32_t n, int32_t reset, void* stream);

/* Stream-ordered device-to-device copies of the FP64 rho_hat to / from a
 * caller's device double (checkpoints of a differentiable forward). */
int xpbd_save_rho_hat(void* handle, double* dst_device, void* stream);
int xpbd_load_rho_hat(void* handle, const double* src_device, void* stream);

/* Sticky device error flags (XPBD_OK, XPBD_ERR_NONFINITE or XPBD_ERR_TIMEOUT);
 * synchronises. */
int xpbd_check_status(void* handle, void* stream);

/* ------------------------------------------------------------------------
 * Differentiation of one substep (block mode, ATOMIC or GATHER variant,
 * per-tet materials).  No counterpart in the reference, which has no
 * gradients; the adjoint follows the forward of neohookean_solver.py:453-587.
 * Contact sets and the pivot branch are piecewise constant.  The Chebyshev
 * omega is a stop-gradient unless the tape carries `posts` and `rho_in` and
 * the adjoint an `omega_state`: then the adjoint also runs back through
 * omega_k -> rho_hat_k -> r_hat_k -> the post-Jacobi positions, multipliers
 * and compliances (:298-329, :495-546), the derivative of the forward as it
 * runs; the clamp of the rho ratio and the warm-up are piecewise constant.
 * ------------------------------------------------------------------------ */
typedef struct xpbd_tape {
  float* xs;      /* [(K+1)][V][4] predicted positions entering every iteration */
  float* lams;    /* [K][T][2] multipliers entering every iteration; with posts
                     [K+1][T][2], the last being those after the substep */
  float* xpre;    /* [V][4] predicted positions before the SDF list */
  float* v1;      /* [V][4] velocities after gravity */
  float* posts;   /* [K][V][4] post-Jacobi positions of every iteration, or NULL
                     (omega then is a stop-gradient) */
  double* rho_in; /* [bodies] rho_hat entering the substep (with posts) */
  double* hist;   /* [bodies][K][4] the substep's history rows (r_hat, omega,
                     ...), copied by the tape call, or NULL: the adjoint then
                     reads the solver's own rows 0..K-1, which the next
                     substep overwrites.  With it, the tapes of many substeps
                     can be recorded in the forward and reversed later. */
} xpbd_tape;

typedef struct xpbd_adjoint {
  float* gx;            /* [V][4] in: dL/dx after the substep; out: before it */
  float* gv;            /* [V][4] likewise for v */
  double* g_inv_mu;     /* [T] += dL/d(1/mu) of every tet */
  double* g_inv_lambda; /* [T] += dL/d(1/lambda) */
  float* work0;         /* [V][4] scratch */
  float* work1;         /* [V][4] scratch */
  float* ybar;          /* [V][4] scratch */
  float* dxbar;         /* [V][4] scratch */
  float* lambar;        /* [T][2] scratch */
  const float* cnt;     /* [V] constraints per vertex (vertex valence) */
  double* omega_state;  /* [bodies][8 + 6 K] the omega chain's state and the
                           substep's chain coefficients, or NULL (omega is a
                           stop-gradient); zero it before the first substep
                           adjoint of a backward pass (it carries the adjoint of
                           rho_hat, which persists across substeps, backwards) */
  float* work_res_tet;  /* [T][4] scratch of the batched omega chain (NULL for a
                           single body) */
} xpbd_adjoint;

/* One substep (as xpbd_substep) that records `tape`; history rows [0, K)
 * receive its omegas for xpbd_substep_adjoint. */
int xpbd_substep_tape(void* handle, float dt, const xpbd_tape* tape, void* stream);

/* Reverse of the substep recorded on `tape` by xpbd_substep_tape: the last
 * one run, or, when the tape holds its history rows (`hist`), any recorded
 * substep, with the solver's materials and SDFs as they were then. */
int xpbd_substep_adjoint(void* handle, float dt, const xpbd_tape* tape, const xpbd_adjoint* adj, void* stream);

/* Residual sweep that allocates nothing.  No counterpart in the reference.
 * For callers that may not allocate device memory -- an engine or plugin host
 * that owns every device allocation and hands this library only its buffers,
 * or a frame loop that cannot afford cudaMalloc's implicit device
 * synchronisation -- this computes, over the tets of `body` at the post-Jacobi
 * positions pred_x + dx / count, the three FP64 means
 *   out[0] = r_hat  (compute_xpbd_residual, neohookean_solver.py:298-329),
 *   out[1] = mean |det F - 1|, out[2] = mean |tr F^T F - 3|
 * into the caller's device array `out` (3 doubles), using only body->tets,
 * dm_a, dm_b, dm_c, v0, lam, dx and, when set, tet_inv_mu / tet_inv_lambda
 * (then the compliances are per tet and lame_mu / lame_lambda are unused),
 * and pred_x ([V][4]).  Every scatter variant's body works: tets, inv_Dm, V0
 * and lambda are per tet in the same solver order in all of them (the tile
 * variant's padding records past n_tets are not read).  Tet ids are not
 * re-checked, so pass a body that xpbd_create has validated.
 * It calls no cudaMalloc, cudaFree or allocating library routine:
 * its scratch is a static device array of (3 * 8192 + 1) doubles (192 KiB)
 * that every GPU loading the library keeps until the process exits, so one
 * call handles at most 8192 * 256 = 2,097,152 tets; larger meshes get
 * XPBD_ERR_INVALID_ARGUMENT.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  The address is that of the runtime's
 * primary context: it is not looked up again after cudaDeviceReset, and
 * contexts created through the driver API are not supported.  All calls share the array and it
 * keeps the last call's contents (the call clears the ticket it needs), so
 * calls that overlap on the GPU -- on different streams, or from different
 * threads -- race and must be serialised by the caller. */
int xpbd_residual_noalloc(const xpbd_body* body, const float* pred_x, float dt, float lame_mu, float lame_lambda,
                          int32_t precise_hydro, double* out, void* stream);

/* Host mesh preprocessing (replaces the patcher's reorder, xpbd_base.py:42).
 * Permutations perm[new] = old: tets in Morton (Z-order) order of their
 * centroids; vertices in order of first use by the sorted tets (unused
 * vertices last, in Morton order).  Either output may be NULL. */
int xpbd_morton_order(const double* pts, int32_t n_verts, const int32_t* tets, int32_t n_tets,
                      int32_t* vert_perm, int32_t* tet_perm);

/* Patches of `patch_tets` consecutive tets for the tile variant: fills
 * patch_voff [ceil(T/P)+1], patch_verts (capacity 4T; ids ascending per
 * patch) and tet_lid, and returns the largest patch vertex count in
 * *max_patch_verts (the layout is usable only if it is <= 256). */
int xpbd_build_patches(const int32_t* tets, int32_t n_tets, int32_t n_verts, int32_t patch_tets,
                       int32_t* patch_voff, int32_t* patch_verts, uint32_t* tet_lid, int32_t* max_patch_verts);

/* Patch-local vertex -> corner lists for the tile variant, from the layout of
 * xpbd_build_patches: pv_start [patch_voff[n_patches]], pv_slots
 * [4 * ceil(T/P) * P] (unused tail entries are 0xffff). */
int xpbd_build_patch_csr(const int32_t* patch_voff, const uint32_t* tet_lid, int32_t n_tets, int32_t patch_tets,
                         uint16_t* pv_start, uint16_t* pv_slots);

/* Pairs of face-adjacent tets for the two-tets-per-thread tile kernels (the
 * reference's patcher has no counterpart; it only orders the mesh,
 * xpbd_base.py:42).  tets: [T][4] in the solver's order.  Writes order[T]
 * (position i of the new order holds old tet order[i]) and corner_perm[T]
 * (corner c of the new tet is old corner (corner_perm >> 2c) & 3), and the
 * number of face pairs in *n_pairs.  A tet pairs with its nearest face
 * neighbour within 48 positions of the old order (which should be a
 * space-filling order, e.g. xpbd_morton_order's), so the new order keeps its
 * locality.  The new order is made of two-tet units at positions (2k, 2k+1)
 * sorted by their first tet: the face pairs, and the other tets two by two in
 * their old order with unchanged corners (an odd count leaves one last tet).
 * A face pair (a, b) with shared face {u, v, w} becomes a = (u, v, w, a*) and
 * b = (v, u, w, b*), each an even permutation of its old corner order, so
 * every tet keeps its signed rest volume; the kernels then merge the three
 * shared corners in registers without comparing vertex ids. */
int xpbd_pair_tets(const int32_t* tets, int32_t n_tets, int32_t n_verts, int32_t* order, uint8_t* corner_perm,
                   int32_t* n_pairs);

/* Vertex -> (tet*4+corner) CSR for the gather variant, slots ascending. */
int xpbd_build_vertex_csr(const int32_t* tets, int32_t n_tets, int32_t n_verts,
                          int32_t* offsets /* [V+1] */, int32_t* slots /* [4T] */);

/* ------------------------------------------------------------------------
 * Batched form: many independent bodies of uneven size in one set of
 * launches.  The reference steps one body per solver object
 * (neohookean_solver.py:16-587); a batch replaces a list of such solvers that
 * share the SDF list, time step and iteration settings, each body keeping its
 * own Lame parameters and Chebyshev state (rho_hat persists per body).
 * Every body's tets are padded to a multiple of 256 (one patch = 256 tets of
 * one body) and its vertices to a multiple of 256 (one vertex block = 256
 * vertices of one body); padding vertices have inv_m = 0 and vert_perm = -1.
 * ------------------------------------------------------------------------ */
typedef struct xpbd_batch {
  int32_t n_bodies;
  int32_t n_verts;            /* padded total, multiple of 256 */
  int32_t n_tets;             /* padded total = 256 * n_patches */
  int32_t n_patches;
  int32_t n_patch_verts;      /* patch_voff[n_patches] */
  int32_t n_out_verts;        /* caller vertices (sum of real vertex counts) */
  float* x;                   /* [V][4] w = inv_m */
  float* v;                   /* [V][4] */
  float* p0;                  /* [V][4] */
  float* p1;                  /* [V][4] */
  float* dx;                  /* [V][4] zero at create */
  const float* dm_a;          /* [T][4] */
  const float* dm_b;          /* [T][4] */
  const float* dm_c;          /* [T] */
  float* lam;                 /* [T][2] */
  const uint32_t* tet_lid;    /* [T] 4 u8 patch-local corner ids */
  const int32_t* patch_voff;  /* [n_patches+1] */
  const int32_t* patch_verts; /* [n_patch_verts] */
  const int32_t* patch_body;  /* [n_patches] */
  const int32_t* patch_ntets; /* [n_patches] real tets of the patch */
  const int32_t* vblock_body; /* [V/256] */
  const float* body_inv_mu;   /* [n_bodies] 1 / mu */
  const float* body_inv_lambda; /* [n_bodies] 1 / lambda */
  const int32_t* body_n_patches; /* [n_bodies] */
  const int32_t* body_n_tets; /* [n_bodies] real tets (r_hat = sum / n) */
  const int32_t* vert_perm;   /* [V] caller vertex of each solver vertex, -1 for padding */
  /* optional per-tet materials: 1 / mu and 1 / lambda of every tet slot
   * (padding slots unused); NULL = the body's body_inv_mu / body_inv_lambda */
  const float* tet_inv_mu;    /* [T] */
  const float* tet_inv_lambda; /* [T] */
  int32_t tet_pairs;          /* 1: every body's tets laid out by xpbd_pair_tets (see xpbd_body) */
} xpbd_batch;

/* Message of the last batch failure on the calling thread. */
const char* xpbd_batch_last_error(void);

/* Create a batch (params: lame_mu / lame_lambda unused, per body instead). */
int xpbd_batch_create(const xpbd_params* params, const xpbd_batch* batch, const xpbd_sdf* sdfs, int32_t n_sdf,
                      int32_t max_records, void** out_handle);
int xpbd_batch_destroy(void* handle);

/* One substep of every body (neohookean_solver.py:577-579). */
int xpbd_batch_substep(void* handle, float dt, int32_t record_base, void* stream);

/* One frame of every body (neohookean_solver.py:562-587), cached CUDA graph.
 * In stop mode (xpbd_params) every body stops at its own residual target; the
 * frame graph loops while any body still iterates, and the kernels skip the
 * patches and vertex blocks of the bodies that have stopped. */
int xpbd_batch_solve(void* handle, double frame_dt, double dt, int32_t substeps, void* stream);

/* History rows [0, n) of every body, host layout [n_bodies][n][4]; synchronises. */
int xpbd_batch_read_history(void* handle, double* host_out, int32_t n, void* stream);

/* Jacobi iterations every body ran in substeps [0, n) of the last frame,
 * host layout [n_bodies][n], n <= 256 (stop mode: xpbd_params); synchronises.
 * No counterpart in the reference, whose iteration count is fixed. */
int xpbd_batch_read_iterations(void* handle, int32_t* host_out, int32_t n, void* stream);

/* rho_hat of every body (host [n_bodies]); synchronises. */
int xpbd_batch_get_rho_hat(void* handle, double* host_out, void* stream);

int xpbd_batch_check_status(void* handle, void* stream);
int xpbd_batch_import_vec3(void* handle, int32_t field, const float* src, void* stream);
int xpbd_batch_export_vec3(void* handle, int32_t field, float* dst, void* stream);
int xpbd_batch_set_profiling(void* handle, int32_t enable);
int xpbd_batch_read_profile(void* handle, double* ms, int64_t* launches, int32_t n, int32_t reset, void* stream);

/* Replace the batch's constants between frames (attribute changes of the
 * solver objects a batch replaces, neohookean_solver.py:18-77); drops the
 * cached frame graph when they differ.  Used by the launch autotuner to
 * switch tets_per_thread in place. */
int xpbd_batch_set_params(void* handle, const xpbd_params* params);

/* Stream-ordered copy of every body's rho_hat (neohookean_solver.py:65) to /
 * from a device array of n_bodies doubles (per-substep adjoint checkpoints). */
int xpbd_batch_save_rho_hat(void* handle, double* dst_device, void* stream);
int xpbd_batch_load_rho_hat(void* handle, const double* src_device, void* stream);

/* Batched differentiation (no counterpart in the reference, which has no
 * gradients): xpbd_substep_tape / xpbd_substep_adjoint for every body of the
 * batch at once, block mode only.  Tape and adjoint buffers are sized by the
 * padded batch (V = n_verts, T = n_tets of xpbd_batch); history rows [0, K)
 * of every body receive the substep's omegas, so max_records >= K.  Per-tet
 * material adjoints are written per tet slot (dL/d(1/mu), dL/d(1/lambda) of
 * the tet's own material with tet_inv_mu, else of its body's). */
int xpbd_batch_substep_tape(void* handle, float dt, const xpbd_tape* tape, void* stream);
int xpbd_batch_substep_adjoint(void* handle, float dt, const xpbd_tape* tape, const xpbd_adjoint* adj,
                               void* stream);

#ifdef __cplusplus
}
#endif

#endif /* XPBD_GB300_H */

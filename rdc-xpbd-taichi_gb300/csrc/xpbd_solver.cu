// GB300 (sm_103a) kernels and C ABI of the RDC-XPBD substep.
//
// One substep of XPBDNeoHookeanSolver (neohookean_solver.py:453-587,
// xpbd_base.py:139-178) runs as
//   begin   (V): predict + sequential SDF projection            xpbd_base.py:139-178
//   per Jacobi iteration:
//     project (T): block 2x2 (or split) Neo-Hookean projection,
//                  Jacobi scatter of dx + constraint count       neohookean_solver.py:144-254,358-451
//     [gather](V): deterministic CSR sum of per-corner dx (gather variant only)
//     residual(T): r_hat / monitoring sums at post-Jacobi positions,
//                  FP64 block reduction into the sweep's sums    :298-329, :492-504
//     update  (V): rho_hat / omega from those sums (per CTA),
//                  post_solve + Chebyshev mix, dx reset          :115-142, :537-549
//   end     (V): velocity update                                xpbd_base.py:148-160
// The predicted positions ping-pong between p0/p1: the Chebyshev mix writes
// x_{k+1} over y_{k-1} in place, so no buffer copies are needed
// (neohookean_solver.py:121-142 copies three buffers instead).

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "xpbd_device.cuh"

namespace xpbd {

constexpr int kBlock = 256;
constexpr int kUpdateVerts = 2;  // vertices per thread in k_update

// FP64 solver state that lives on the device (neohookean_solver.py:59-69).
// Chebyshev state entering one Jacobi iteration of a substep.
struct SweepSlot {
  double rho_hat;
  double prev_r_hat;
  double inv_prev;  // 1 / (prev_r_hat + 1e-12)
  double omega;     // omega of the previous iteration of this substep
  double r0;        // r_hat of the substep's first iteration (stop mode)
  int has_prev;     // prev_r_hat is not None
  int it;           // index of the iteration this slot enters
  int active;       // stop mode: 0 once the substep has stopped iterating
};

// Substeps of one frame whose iteration counts are kept (DevState::iters).
constexpr int kMaxCountedSubsteps = 256;

// Iteration k's residual sweep adds into acc[k & 1]; iteration k's update
// reads slot[k & 1] and acc[k & 1], and its first CTA writes slot[(k+1) & 1]
// and clears acc[(k+1) & 1], so no kernel reads what it writes.
struct DevState {
  double acc[2][3];     // residual sum, |C_H| sum, |C_D| sum of a sweep
  SweepSlot slot[2];
  double rho_hat;       // persists across substeps and frames
  int nonfinite;        // sticky: a residual sum was NaN/Inf
  int bad_mesh;         // set by the index validation kernel
  int timeout;          // sticky: a bounded mbarrier wait gave up
  int pos_cur;          // buffer p[] holding the predicted positions after
                        // the last iteration that ran (stop mode)
  int iters[kMaxCountedSubsteps];  // iterations run by substep s of the frame
  unsigned long long total_iters;  // iterations run since create (residual sweeps ended)
};

struct Dev {
  int V, T;
  float4* x;
  float4* v;
  float4* p[2];
  float4* dx;
  const int4* tets;
  const float4* dm_a;
  const float4* dm_b;
  const float* dm_c;
  const float* v0;
  float2* lam;
  const float* tinv_mu;  // per-tet 1 / mu (nullptr: uniform)
  const float* tinv_la;  // per-tet 1 / lambda
  const int* v2t_off;
  const int* v2t_slot;
  float4* corner;
  const int* perm;  // solver vertex i <- caller vertex perm[i] (nullptr = identity)
  int paired;       // tets laid out by xpbd_pair_tets
  int l2_keep;      // tile sweeps load the tet records evict_last
  // tile variant: patch p = tets [p*P, (p+1)*P), vertices verts[voff[p]..voff[p+1])
  int n_patches, P, n_pverts;
  const uint32_t* lid;
  const int* voff;
  const int* pverts;
  const uint16_t* pv_start;
  const uint16_t* pv_slots;
  const xpbd_sdf* sdfs;
  int n_sdf;
  DevState* st;
  double* hist;
  // stop mode (xpbd_params.target_rel_residual > 0): the `active` flag of the
  // slot entering the launched iteration; nullptr = always run
  const int* act;
  int dyn_end;  // stop mode: advance and the vertex-field accessors read p[st->pos_cur]
  float2* lam_tape;  // taping (ATOMIC / GATHER projection): the multipliers entering the iteration (nullptr: none)
};

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// Stop mode: the iteration this launch belongs to is not run (the substep
// already met its residual target or iteration cap).  Every CTA reads the
// same flag, which an earlier kernel wrote.
__device__ __forceinline__ bool stopped(const Dev& d) {
  return d.act != nullptr && *reinterpret_cast<const volatile int*>(d.act) == 0;
}

// ---------------------------------------------------------------------------
// vertex kernels
// ---------------------------------------------------------------------------

// kPredict: apply_external_forces (xpbd_base.py:139-146) writes p[dst].
// kSdf: solve_step's start (neohookean_solver.py:457-463): prev_r_hat = None,
//       omega = 1, then sequential SDF projection of p[dst] (xpbd_base.py:162-178).
template <bool kPredict, bool kSdf>
__global__ void __launch_bounds__(kBlock) k_begin(Dev d, float dt, float gx, float gy, float gz, int dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (kSdf && i == 0) {
    SweepSlot& s0 = d.st->slot[0];
    s0.rho_hat = d.st->rho_hat;
    s0.prev_r_hat = 0.0;
    s0.inv_prev = 0.0;
    s0.omega = 1.0;
    s0.has_prev = 0;
    s0.r0 = 0.0;
    s0.it = 0;
    s0.active = 1;
    d.st->pos_cur = dst;
    d.st->acc[0][0] = d.st->acc[0][1] = d.st->acc[0][2] = 0.0;
  }
  if (i >= d.V) return;
  const float4 xi = d.x[i];
  float4 vi = d.v[i];
  const float w = xi.w;
  float3 p;
  if (kPredict) {
    if (w > 0.f) {
      vi.x += gx * dt;
      vi.y += gy * dt;
      vi.z += gz * dt;
      d.v[i] = vi;
    }
    p = make_float3(xi.x + vi.x * dt, xi.y + vi.y * dt, xi.z + vi.z * dt);
  } else {
    const float4 q = d.p[dst][i];
    p = make_float3(q.x, q.y, q.z);
  }
  if (kSdf && w > 0.f) sdf_project_all(d.sdfs, d.n_sdf, p, make_float3(vi.x, vi.y, vi.z));
  d.p[dst][i] = make_float4(p.x, p.y, p.z, w);
}

// advance (xpbd_base.py:148-160) from p[cur] (stop mode: from the buffer the
// last iteration that ran left the positions in).
__global__ void __launch_bounds__(kBlock) k_end(Dev d, int cur, float dt, float damping) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
  if (d.dyn_end) cur = d.st->pos_cur;
  const float4 xi = d.x[i];
  if (xi.w <= 0.f) {
    d.p[cur][i] = xi;  // fixed vertices do not move
    return;
  }
  const float4 pi = d.p[cur][i];
  const float e = expf(-dt * damping);
  const float4 vi = d.v[i];
  d.v[i] = make_float4((pi.x - xi.x) / dt * e, (pi.y - xi.y) / dt * e, (pi.z - xi.z) / dt * e, vi.w);
  d.x[i] = make_float4(pi.x, pi.y, pi.z, xi.w);
}

// Deterministic gather: dx[v] = sum of its corner contributions in ascending
// (tet, corner) order, i.e. the order of a sequential scatter.
__global__ void __launch_bounds__(kBlock) k_gather(Dev d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V || stopped(d)) return;
  const int b = d.v2t_off[i], e = d.v2t_off[i + 1];
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k = b; k < e; ++k) {
    const float4 c = d.corner[d.v2t_slot[k]];
    s.x += c.x;
    s.y += c.y;
    s.z += c.z;
    s.w += c.w;
  }
  d.dx[i] = s;
}

// post_solve (neohookean_solver.py:115-119) fused with the Chebyshev mix
// (:131-142, :548-549).  x_post = p[cur] + dx / count; with kCheb the result
//   y_prev + omega * (gamma * (x_post - y_curr) + y_curr - y_prev)
// is written to p[1-cur] (which held y_prev), else x_post goes to p[cur].
// What the update of one iteration needs to finish its residual sweep.  The
// iteration's index comes from the slot it enters (slot[par]), so the same
// launch can be replayed by a loop in the frame graph.
struct UpdArgs {
  int par;       // slot parity of the iteration (its index & 1)
  int rec_base;  // history row of the substep's iteration 0 (-1: no records)
  int K;         // iterations per substep (stop mode: the cap)
  int warmup;
  int res, mon;  // Chebyshev recurrence / monitoring means
  int stop;      // stop mode: end the substep at the residual target
  int sub;       // substep index for DevState::iters (-1: not counted)
  int cur_next;  // buffer holding the positions after this iteration
  int use_cond;  // set the frame graph's loop condition (cond)
  cudaGraphConditionalHandle cond;
  float4* post_out;  // taping through omega: the post-Jacobi positions (nullptr: none)
  float4* xs_out;    // taping: the positions entering the next iteration (nullptr: none)
  int pre;           // a residual sweep ran between the projection and this update
  double inv_n;  // 1 / tet count (0 for an empty mesh)
  double rho_min, rho_max, rho_beta;
  double target, floor;  // stop at r_hat <= target * r_hat_0 or r_hat <= floor
};

// The end of a residual sweep (neohookean_solver.py:495-504, :537-546): r_hat
// from the sweep's sums, the rho_hat recurrence and omega of the iteration.
// Every CTA of the update evaluates it (thread 0); CTA 0 also stores the
// state entering the next iteration, clears the next sweep's accumulators,
// writes history row rec_base + it = {r_hat, omega, hydro, dev}, and after
// the substep's last iteration the persistent rho_hat.  Every CTA runs one
// FP64 division (omega); r_hat / n and r_hat / prev_r_hat are products with
// reciprocals that the host (1 / n) and the previous iteration's CTA 0
// (1 / prev) computed.
// Stop mode: the substep ends after iteration k once r_hat_k <= target *
// r_hat_0 or r_hat_k <= floor (or at the cap); the remaining iterations'
// kernels return at once, and CTA 0 sets the frame graph's loop condition.
__device__ __forceinline__ float sweep_step(const Dev& d, const UpdArgs& u) {
  DevState* st = d.st;
  const SweepSlot c = st->slot[u.par];
  const double* acc = st->acc[u.par];
  const double S = acc[0], Hs = acc[1], Ds = acc[2];
  const double n = (double)d.T;
  const int it = c.it;
  SweepSlot nx = c;
  double r_hat = 0.0, omega = 1.0;
  if (u.res || u.stop) r_hat = S * u.inv_n;
  if (u.res) {
    if (c.has_prev && c.prev_r_hat > 1e-12) {
      double rho_inst = r_hat * c.inv_prev;
      rho_inst = fmax(u.rho_min, fmin(u.rho_max, rho_inst));
      nx.rho_hat = (1.0 - u.rho_beta) * c.rho_hat + u.rho_beta * rho_inst;
    }
    nx.prev_r_hat = r_hat;
    nx.has_prev = 1;
    const double rho2 = nx.rho_hat * nx.rho_hat;
    if (it < u.warmup) omega = 1.0;
    else if (it == u.warmup) omega = 2.0 / (2.0 - rho2);
    else omega = 4.0 / (4.0 - rho2 * c.omega);
    nx.omega = omega;
  }
  bool more = it + 1 < u.K;
  if (u.stop) {
    if (it == 0) nx.r0 = r_hat;
    if (r_hat <= u.target * nx.r0 || r_hat <= u.floor) more = false;
  }
  nx.it = it + 1;
  nx.active = more ? 1 : 0;
  if (blockIdx.x == 0) {
    if ((u.res || u.stop) && !isfinite(S)) st->nonfinite = 1;
    if (u.res) nx.inv_prev = 1.0 / (r_hat + 1e-12);
    st->slot[u.par ^ 1] = nx;
    double* an = st->acc[u.par ^ 1];
    an[0] = an[1] = an[2] = 0.0;
    if (!more) st->rho_hat = nx.rho_hat;
    if (u.rec_base >= 0) {
      double* h = d.hist + 4 * ((size_t)u.rec_base + it);
      h[0] = r_hat;
      h[1] = omega;
      h[2] = u.mon && d.T > 0 ? Hs / n : 0.0;
      h[3] = u.mon && d.T > 0 ? Ds / n : 0.0;
    }
    if (u.stop) st->pos_cur = u.cur_next;
    if (u.sub >= 0 && u.sub < kMaxCountedSubsteps) st->iters[u.sub] = it + 1;
    st->total_iters += 1ull;
    if (u.use_cond) cudaGraphSetConditional(u.cond, more ? 1u : 0u);
  }
  return (float)omega;
}

// Stop mode, an iteration that does not run: CTA 0 carries the slot (and its
// `active` = 0) over to the next parity and keeps the graph's loop closed.
__device__ __forceinline__ void skip_step(const Dev& d, const UpdArgs& u) {
  DevState* st = d.st;
  SweepSlot nx = st->slot[u.par];
  nx.it += 1;
  st->slot[u.par ^ 1] = nx;
  if (u.use_cond) cudaGraphSetConditional(u.cond, 0u);
}

// Compiled for 4 resident CTAs per SM (64 registers, no spill; 71 without the
// bound, where thread 0's FP64 omega step sets every thread's count): the
// 64^3 cube's 537 CTAs then run in one wave, and the launch takes 9.5 us
// instead of 10.7.
template <bool kCheb, bool kFirstIt, bool kResetDx>
__global__ void __launch_bounds__(kBlock, 4) k_update(Dev d, int cur, float gamma, UpdArgs u) {
  // kUpdateVerts vertices per thread, kBlock apart: all of a thread's loads
  // are in flight together, and the grid is a quarter of a one-per-vertex one
  const int base = blockIdx.x * (kBlock * kUpdateVerts) + threadIdx.x;
  // every load is issued before the first store: as far as the compiler
  // knows the buffers may alias, so a load after a store would wait for it
  float4 pc[kUpdateVerts], D[kUpdateVerts], yp[kUpdateVerts];
  // after a residual sweep the positions and Jacobi sums were written two or
  // more kernels back; straight after the projection the sums are not yet
  if (!u.pre) pdl_wait();
#pragma unroll
  for (int k = 0; k < kUpdateVerts; ++k) {
    const int i = base + k * kBlock;
    if (i < d.V) {
      pc[k] = d.p[cur][i];
      D[k] = d.dx[i];
      yp[k] = (kCheb && !kFirstIt) ? d.p[cur ^ 1][i] : pc[k];
    }
  }
  if (u.pre) pdl_wait();  // the residual's sums (sweep_step), and the stores below
  pdl_trigger();
  __shared__ float s_om;
  __shared__ int s_run;
  if (threadIdx.x == 0) {
    const bool run = !stopped(d);
    s_run = run;
    if (run) s_om = (u.res || u.mon || u.stop) ? sweep_step(d, u) : 1.f;
    else if (blockIdx.x == 0) skip_step(d, u);
  }
  __syncthreads();
  if (!s_run) return;
  const float om = kCheb ? s_om : 1.f;
#pragma unroll
  for (int k = 0; k < kUpdateVerts; ++k) {
    const int i = base + k * kBlock;
    if (i >= d.V) break;
    if (kResetDx) d.dx[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    float3 xp = make_float3(pc[k].x, pc[k].y, pc[k].z);
    if (D[k].w > 0.f) {
      xp.x += D[k].x / D[k].w;
      xp.y += D[k].y / D[k].w;
      xp.z += D[k].z / D[k].w;
    }
    if (u.post_out) u.post_out[i] = make_float4(xp.x, xp.y, xp.z, pc[k].w);
    float4 xo;
    if (kCheb) {
      const float nx = gamma * (xp.x - pc[k].x) + pc[k].x;
      const float ny = gamma * (xp.y - pc[k].y) + pc[k].y;
      const float nz = gamma * (xp.z - pc[k].z) + pc[k].z;
      xo = make_float4(yp[k].x + om * (nx - yp[k].x), yp[k].y + om * (ny - yp[k].y),
                       yp[k].z + om * (nz - yp[k].z), pc[k].w);
      d.p[cur ^ 1][i] = xo;
    } else {
      xo = make_float4(xp.x, xp.y, xp.z, pc[k].w);
      d.p[cur][i] = xo;
    }
    if (u.xs_out) u.xs_out[i] = xo;
  }
}

// ---------------------------------------------------------------------------
// tet kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ void load_tet(const Dev& d, int t, int4& id, Tet& tt) {
  id = __ldg(d.tets + t);
  const float4 a = __ldg(d.dm_a + t);
  const float4 b = __ldg(d.dm_b + t);
  tt.dm[0] = a.x; tt.dm[1] = a.y; tt.dm[2] = a.z;
  tt.dm[3] = a.w; tt.dm[4] = b.x; tt.dm[5] = b.y;
  tt.dm[6] = b.z; tt.dm[7] = b.w; tt.dm[8] = __ldg(d.dm_c + t);
  tt.V0 = __ldg(d.v0 + t);
}

template <bool kGather>
__device__ __forceinline__ void emit(const Dev& d, int t, int corner, int vid, float3 dp, float cnt) {
  if (kGather) {
    d.corner[t * 4 + corner] = make_float4(dp.x, dp.y, dp.z, cnt);
  } else {
    red_add_v4(d.dx + vid, dp.x, dp.y, dp.z, cnt);
  }
}

// solve_neohookean_block (neohookean_solver.py:358-451) for kBlock, else the
// split pair solve_hydrostatic + solve_deviatoric (:196-254, :144-194), both
// reading the same predicted positions.  kFirst: lambda == 0 (the reset at
// :458-459), so lambda is not read.
// One thread per tet; scatter by vector atomics or into the per-corner buffer.
// kFirst: lambda == 0 (the reset at neohookean_solver.py:458-459), not read.
// cD, cH = 1 / (mu dt^2), 1 / (lambda dt^2): aD = alpha_D / dt^2 = cD / V0.
template <bool kBlockMode, bool kFirst, bool kPrecise, bool kGather>
__global__ void __launch_bounds__(kBlock) k_project(Dev d, int cur, float cD, float cH, float relax_h, float relax_d) {
  if (stopped(d)) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.T) return;
  int4 id;
  Tet tt;
  load_tet(d, t, id, tt);
  const float4* P = d.p[cur];
  tt.p[0] = ldg4(P + id.x);
  tt.p[1] = ldg4(P + id.y);
  tt.p[2] = ldg4(P + id.z);
  tt.p[3] = ldg4(P + id.w);
  float2 L = kFirst ? make_float2(0.f, 0.f) : d.lam[t];
  if (d.lam_tape) d.lam_tape[t] = L;
  const int vid[4] = {id.x, id.y, id.z, id.w};
  float3 dp[4];
  float cnt;
  const float inv_v0 = 1.f / tt.V0;
  float aD = cD * inv_v0, aH = cH * inv_v0;
  if (d.tinv_mu) {  // per-tet materials: cD = cH = 1 / dt^2
    aD *= __ldg(d.tinv_mu + t);
    aH *= __ldg(d.tinv_la + t);
  }
  project_tet<kBlockMode, kPrecise>(tt, aD, aH, relax_h, relax_d, L, dp, cnt);
  d.lam[t] = L;
#pragma unroll
  for (int c = 0; c < 4; ++c) emit<kGather>(d, t, c, vid[c], dp[c], cnt);
}

// ---------------------------------------------------------------------------
// Tile variant.  Patch p = kP consecutive tets of the solver order (arrays padded to a
// multiple of the patch size) whose <= 256 vertices are listed in
// pverts[voff[p] .. voff[p+1]).  Persistent CTAs walk the patches; one thread
// streams the next patch's tet records (48 bytes per tet: 4 u8 local corner
// ids, inv_Dm, lambda) into shared memory with cp.async.bulk while the CTA
// works on the current patch, whose vertex neighbourhood is staged in shared
// memory once and shared by all its tets.  V0 = 1 / (6 det inv_Dm).
// ---------------------------------------------------------------------------

struct __align__(16) PatchStage {
  float4 dma[256];
  float4 dmb[256];
  float2 lam[256];
  uint32_t lid[256];
  float dmc[256];
};

constexpr int kMaxPolls = 1 << 20;

// Issue the bulk copies of patch p's tet records into `st` (one thread);
// completion is tracked by the transaction count of `bar`.
template <bool kLam>
__device__ __forceinline__ void issue_records(const Dev& d, PatchStage& st, unsigned long long* barp, int p, int kP) {
  const size_t t0 = (size_t)p * kP;
  const uint32_t bytes = kP * (16u + 16u + 4u + 4u + (kLam ? 8u : 0u));
  uint64_t* bar = reinterpret_cast<uint64_t*>(barp);
  mbar_expect_tx(bar, bytes);
  bulk_g2s(st.dma, d.dm_a + t0, kP * 16u, bar);
  bulk_g2s(st.dmb, d.dm_b + t0, kP * 16u, bar);
  bulk_g2s(st.lid, d.lid + t0, kP * 4u, bar);
  bulk_g2s(st.dmc, d.dm_c + t0, kP * 4u, bar);
  if (kLam) bulk_g2s(st.lam, d.lam + t0, kP * 8u, bar);
}

__device__ __forceinline__ void stage_tet(const PatchStage& st, int i, Tet& tt, uint32_t& lid) {
  const float4 A = st.dma[i], B = st.dmb[i];
  tt.dm[0] = A.x; tt.dm[1] = A.y; tt.dm[2] = A.z;
  tt.dm[3] = A.w; tt.dm[4] = B.x; tt.dm[5] = B.y;
  tt.dm[6] = B.z; tt.dm[7] = B.w; tt.dm[8] = st.dmc[i];
  lid = st.lid[i];
}


// Shared memory of the pipelined tile kernels: two stages, each with the tet
// records of one patch (bulk copy), the positions (and for the residual the
// Jacobi accumulators) of its vertices (cp.async gathers) and their ids.
template <bool kDx>
struct __align__(16) TileSmem {
  PatchStage st[2];
  float4 sp[2][256];
  float4 sdx[2][kDx ? 256 : 1];
  int sg[2][256];
  unsigned long long bar[2];
};

// Gather the vertex tile of one patch into stage s (thread j < nv takes vertex j).
template <bool kDx>
__device__ __forceinline__ void gather_tile(const Dev& d, TileSmem<kDx>& sm, int s, const float4* P, int g) {
  const int j = threadIdx.x;
  sm.sg[s][j] = g;
  cp_async16(&sm.sp[s][j], P + g);
  if (kDx) cp_async16(&sm.sdx[s][j], d.dx + g);
}

// Patch ids of the CTA's walk; `reverse` visits them last-to-first.
__device__ __forceinline__ int walk_patch(int q, int n, bool reverse) { return reverse ? n - 1 - q : q; }

// Pipelined tile projection (256 tets per patch, one vertex per thread).
// Iteration k computes patch q_k while the records and vertex tile of
// q_{k+1} are in flight and the vertex list of q_{k+2} is being read.
template <bool kBlockMode, bool kFirst, bool kPrecise>
__global__ void __launch_bounds__(256) k_project_tile(Dev d, int cur, float cD, float cH, float relax_h,
                                                     float relax_d) {
  if (stopped(d)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem<false>& sm = *reinterpret_cast<TileSmem<false>*>(smem_raw);
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(reinterpret_cast<uint64_t*>(&sm.bar[0]), 1);
    mbar_init(reinterpret_cast<uint64_t*>(&sm.bar[1]), 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  const int n = d.n_patches, G = gridDim.x, tid = threadIdx.x;
  const float4* P = d.p[cur];
  int q = blockIdx.x;
  if (q >= n) return;
  // prologue: records + tile of q, vertex id of q + G
  if (tid == 0) issue_records<!kFirst>(d, sm.st[0], &sm.bar[0], q, 256);
  {
    const int vb = __ldg(d.voff + q), nv = __ldg(d.voff + q + 1) - vb;
    if (tid < nv) gather_tile<false>(d, sm, 0, P, __ldg(d.pverts + vb + tid));
  }
  cp_async_commit();
  int gn = -1;
  if (q + G < n) {
    const int vb = __ldg(d.voff + q + G), nv = __ldg(d.voff + q + G + 1) - vb;
    if (tid < nv) gn = __ldg(d.pverts + vb + tid);
  }
  int k = 0;
  bool issued_next = false;
  for (; q < n; q += G, ++k) {
    const int s = k & 1;
    const int qn = q + G;
    issued_next = qn < n;
    if (issued_next) {
      if (tid == 0) {
        fence_proxy_async();
        issue_records<!kFirst>(d, sm.st[s ^ 1], &sm.bar[s ^ 1], qn, 256);
      }
      if (gn >= 0) gather_tile<false>(d, sm, s ^ 1, P, gn);
    }
    cp_async_commit();
    gn = -1;
    if (qn + G < n) {
      const int vb = __ldg(d.voff + qn + G), nv = __ldg(d.voff + qn + G + 1) - vb;
      if (tid < nv) gn = __ldg(d.pverts + vb + tid);
    }
    cp_async_wait<1>();
    if (tid == 0 && !mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[s]), (k >> 1) & 1, kMaxPolls)) {
      abort_flag = 1;
      d.st->timeout = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    const int t = q * 256 + tid;
    if (t < d.T) {
      Tet tt;
      uint32_t lid;
      stage_tet(sm.st[s], tid, tt, lid);
      const int l[4] = {(int)(lid & 0xffu), (int)((lid >> 8) & 0xffu), (int)((lid >> 16) & 0xffu), (int)(lid >> 24)};
#pragma unroll
      for (int c = 0; c < 4; ++c) tt.p[c] = sm.sp[s][l[c]];
      float2 L = kFirst ? make_float2(0.f, 0.f) : sm.st[s].lam[tid];
      const float six_det = 6.f * det9(tt.dm);  // 1 / V0
      float3 dp[4];
      float cnt;
      project_tet<kBlockMode, kPrecise>(tt, six_det * cD, six_det * cH, relax_h, relax_d, L, dp, cnt);
      d.lam[t] = L;
#pragma unroll
      for (int c = 0; c < 4; ++c) red_add_v4(d.dx + sm.sg[s][l[c]], dp[c].x, dp[c].y, dp[c].z, cnt);
    }
    __syncthreads();  // stage s is refilled two iterations later
  }
  cp_async_wait<0>();
  if (abort_flag && tid == 0) {
    mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[k & 1]), (k >> 1) & 1, kMaxPolls);
    if (issued_next) mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[(k & 1) ^ 1]), ((k + 1) >> 1) & 1, kMaxPolls);
  }
}

// Gather vertex g of the patch's list position j into stage s.
__device__ __forceinline__ void gather_vertex(TileSmem<false>& sm, int s, const float4* P, int g, int j) {
  sm.sg[s][j] = g;
  cp_async16(&sm.sp[s][j], P + g);
}

// Pipelined tile projection with two consecutive tets per thread (128 threads
// per 256-tet patch): the walk, stages and copies of k_project_tile, and per
// thread the chain of k_project_patchN (the corner sums a face pair shares
// merged before the reduction).  Each thread gathers vertices j and j + 128
// of the next tile.
template <bool kBlockMode, bool kFirst, bool kPrecise>
__global__ void __launch_bounds__(128, 6) k_project_tile2(Dev d, int cur, float cD, float cH, float relax_h,
                                                         float relax_d) {
  if (stopped(d)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem<false>& sm = *reinterpret_cast<TileSmem<false>*>(smem_raw);
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(reinterpret_cast<uint64_t*>(&sm.bar[0]), 1);
    mbar_init(reinterpret_cast<uint64_t*>(&sm.bar[1]), 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  const int n = d.n_patches, G = gridDim.x, tid = threadIdx.x;
  const float4* P = d.p[cur];
  int q = blockIdx.x;
  if (q >= n) return;
  // prologue: records + tile of q, vertex ids of q + G
  if (tid == 0) issue_records<!kFirst>(d, sm.st[0], &sm.bar[0], q, 256);
  {
    const int vb = __ldg(d.voff + q), nv = __ldg(d.voff + q + 1) - vb;
    if (tid < nv) gather_vertex(sm, 0, P, __ldg(d.pverts + vb + tid), tid);
    if (tid + 128 < nv) gather_vertex(sm, 0, P, __ldg(d.pverts + vb + tid + 128), tid + 128);
  }
  cp_async_commit();
  int gn0 = -1, gn1 = -1;
  if (q + G < n) {
    const int vb = __ldg(d.voff + q + G), nv = __ldg(d.voff + q + G + 1) - vb;
    if (tid < nv) gn0 = __ldg(d.pverts + vb + tid);
    if (tid + 128 < nv) gn1 = __ldg(d.pverts + vb + tid + 128);
  }
  int k = 0;
  bool issued_next = false;
  const int l0 = 2 * tid;
  for (; q < n; q += G, ++k) {
    const int s = k & 1;
    const int qn = q + G;
    issued_next = qn < n;
    if (issued_next) {
      if (tid == 0) {
        fence_proxy_async();
        issue_records<!kFirst>(d, sm.st[s ^ 1], &sm.bar[s ^ 1], qn, 256);
      }
      if (gn0 >= 0) gather_vertex(sm, s ^ 1, P, gn0, tid);
      if (gn1 >= 0) gather_vertex(sm, s ^ 1, P, gn1, tid + 128);
    }
    cp_async_commit();
    gn0 = gn1 = -1;
    if (qn + G < n) {
      const int vb = __ldg(d.voff + qn + G), nv = __ldg(d.voff + qn + G + 1) - vb;
      if (tid < nv) gn0 = __ldg(d.pverts + vb + tid);
      if (tid + 128 < nv) gn1 = __ldg(d.pverts + vb + tid + 128);
    }
    cp_async_wait<1>();
    if (tid == 0 && !mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[s]), (k >> 1) & 1, kMaxPolls)) {
      abort_flag = 1;
      d.st->timeout = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    const int t0 = q * 256;
    const int nt = d.T - t0 < 256 ? d.T - t0 : 256;
    const int nk = nt - l0 < 2 ? nt - l0 : 2;
    if (nk > 0) {
      const PatchStage& st = sm.st[s];
      float4 A[2], B[2];
      float C[2];
      uint32_t lid[2];
      float2 L[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int i = j < nk ? l0 + j : l0;
        A[j] = st.dma[i];
        B[j] = st.dmb[i];
        C[j] = st.dmc[i];
        lid[j] = st.lid[i];
        L[j] = kFirst ? make_float2(0.f, 0.f) : st.lam[i];
      }
      project_chain<kBlockMode, kPrecise, 2>(A, B, C, lid, L, d.lam + t0 + l0, nk, sm.sp[s], sm.sg[s], d.dx, cD, cH,
                                             relax_h, relax_d, d.paired != 0);
    }
    __syncthreads();  // stage s is refilled two iterations later
  }
  cp_async_wait<0>();
  if (abort_flag && tid == 0) {
    mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[k & 1]), (k >> 1) & 1, kMaxPolls);
    if (issued_next) mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[(k & 1) ^ 1]), ((k + 1) >> 1) & 1, kMaxPolls);
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float3 post_position(const float4 p, const float4 D) {
  float3 r = make_float3(p.x, p.y, p.z);
  if (D.w > 0.f) {
    r.x += D.x / D.w;
    r.y += D.y / D.w;
    r.z += D.z / D.w;
  }
  return r;
}

struct SweepArgs {
  int cur;
  float cD, cH;  // 1 / (mu dt^2), 1 / (lambda dt^2)
  int par;       // accumulators acc[par] (the iteration's index & 1)
  int reverse;   // tile residual: visit patches last-to-first
};

// Block FP64 reduction of the per-thread partial sums, added into the
// sweep's accumulators.  The rho_hat / omega recurrence runs in the update
// that follows (sweep_step), so the sweep ends with its last reduction.
template <bool kRes, bool kMon>
__device__ __forceinline__ void finish_residual(const Dev& d, const SweepArgs& a, float sr, float sh, float sd) {
  __shared__ double red[3][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const double r0 = warp_sum((double)sr), r1 = warp_sum((double)sh), r2 = warp_sum((double)sd);
  if (lane == 0) {
    red[0][warp] = r0;
    red[1][warp] = r1;
    red[2][warp] = r2;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double b0 = 0.0, b1 = 0.0, b2 = 0.0;
  for (int k = 0; k < nw; ++k) {
    b0 += red[0][k];
    b1 += red[1][k];
    b2 += red[2][k];
  }
  double* acc = d.st->acc[a.par];
  if (kRes) atomicAdd(acc, b0);
  if (kMon) {
    atomicAdd(acc + 1, b1);
    atomicAdd(acc + 2, b2);
  }
}

template <bool kRes, bool kMon, bool kPrecise>
__device__ __forceinline__ void residual_terms(const Tet& tt, float2 L, float aD, float aH, float& sr, float& sh,
                                               float& sd) {
  float F[9];
  deformation_gradient(tt, F);
  float C_D, C_H;
  invariants<kPrecise>(F, C_D, C_H);
  if (kRes) {
    const float rD = C_D + aD * L.x;
    const float rH = C_H + aH * L.y;
    sr += sqrtf(rD * rD + rH * rH);
  }
  if (kMon) {
    sh += fabsf(C_H);
    sd += fabsf(C_D);
  }
}

// compute_xpbd_residual (neohookean_solver.py:298-329) and the monitoring
// errors (:256-296) at the post-Jacobi positions p[cur] + dx/count, i.e.
// before the Chebyshev mix (:490-494).  Grid-stride over tets with per-thread
// FP32 partials, then finish_residual.
template <bool kRes, bool kMon, bool kPrecise>
__global__ void __launch_bounds__(kBlock) k_residual(Dev d, SweepArgs a) {
  if (stopped(d)) return;
  float sr = 0.f, sh = 0.f, sd = 0.f;
  const float4* P = d.p[a.cur];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < d.T; t += gridDim.x * blockDim.x) {
    int4 id;
    Tet tt;
    load_tet(d, t, id, tt);
    const int vid[4] = {id.x, id.y, id.z, id.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float3 q = post_position(ldg4(P + vid[c]), ldg4(d.dx + vid[c]));
      tt.p[c] = make_float4(q.x, q.y, q.z, 0.f);
    }
    const float2 L = kRes ? d.lam[t] : make_float2(0.f, 0.f);
    const float inv_v0 = 1.f / tt.V0;
    float aD = a.cD * inv_v0, aH = a.cH * inv_v0;
    if (d.tinv_mu) {
      aD *= __ldg(d.tinv_mu + t);
      aH *= __ldg(d.tinv_la + t);
    }
    residual_terms<kRes, kMon, kPrecise>(tt, L, aD, aH, sr, sh, sd);
  }
  finish_residual<kRes, kMon>(d, a, sr, sh, sd);
}

// Pipelined tile residual: the same walk as k_project_tile (optionally
// last-to-first, so that the records the projection touched last are still
// in L2); the tile carries positions and Jacobi accumulators, converted to
// post-Jacobi positions in shared memory before the tets use them.
template <bool kRes, bool kMon, bool kPrecise>
__global__ void __launch_bounds__(256) k_residual_tile(Dev d, SweepArgs a) {
  if (stopped(d)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem<true>& sm = *reinterpret_cast<TileSmem<true>*>(smem_raw);
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(reinterpret_cast<uint64_t*>(&sm.bar[0]), 1);
    mbar_init(reinterpret_cast<uint64_t*>(&sm.bar[1]), 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  float sr = 0.f, sh = 0.f, sd = 0.f;
  const int n = d.n_patches, G = gridDim.x, tid = threadIdx.x;
  const bool rev = a.reverse != 0;
  const float4* P = d.p[a.cur];
  int q = blockIdx.x;
  int k = 0;
  bool issued_next = false;
  if (q < n) {
    const int p0 = walk_patch(q, n, rev);
    if (tid == 0) issue_records<kRes>(d, sm.st[0], &sm.bar[0], p0, 256);
    const int vb = __ldg(d.voff + p0), nv = __ldg(d.voff + p0 + 1) - vb;
    if (tid < nv) gather_tile<true>(d, sm, 0, P, __ldg(d.pverts + vb + tid));
  }
  cp_async_commit();
  int gn = -1;
  if (q + G < n) {
    const int p1 = walk_patch(q + G, n, rev);
    const int vb = __ldg(d.voff + p1), nv = __ldg(d.voff + p1 + 1) - vb;
    if (tid < nv) gn = __ldg(d.pverts + vb + tid);
  }
  for (; q < n; q += G, ++k) {
    const int s = k & 1;
    const int p = walk_patch(q, n, rev);
    const int qn = q + G;
    issued_next = qn < n;
    if (issued_next) {
      if (tid == 0) {
        fence_proxy_async();
        issue_records<kRes>(d, sm.st[s ^ 1], &sm.bar[s ^ 1], walk_patch(qn, n, rev), 256);
      }
      if (gn >= 0) gather_tile<true>(d, sm, s ^ 1, P, gn);
    }
    cp_async_commit();
    gn = -1;
    if (qn + G < n) {
      const int p2 = walk_patch(qn + G, n, rev);
      const int vb = __ldg(d.voff + p2), nv = __ldg(d.voff + p2 + 1) - vb;
      if (tid < nv) gn = __ldg(d.pverts + vb + tid);
    }
    cp_async_wait<1>();
    if (tid == 0 && !mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[s]), (k >> 1) & 1, kMaxPolls)) {
      abort_flag = 1;
      d.st->timeout = 1;
    }
    __syncthreads();
    if (abort_flag) break;
    {
      const int nv = __ldg(d.voff + p + 1) - __ldg(d.voff + p);
      if (tid < nv) {
        const float3 x = post_position(sm.sp[s][tid], sm.sdx[s][tid]);
        sm.sp[s][tid] = make_float4(x.x, x.y, x.z, 0.f);
      }
    }
    __syncthreads();
    const int t = p * 256 + tid;
    if (t < d.T) {
      Tet tt;
      uint32_t lid;
      stage_tet(sm.st[s], tid, tt, lid);
      tt.p[0] = sm.sp[s][lid & 0xffu];
      tt.p[1] = sm.sp[s][(lid >> 8) & 0xffu];
      tt.p[2] = sm.sp[s][(lid >> 16) & 0xffu];
      tt.p[3] = sm.sp[s][lid >> 24];
      const float six_det = 6.f * det9(tt.dm);
      const float2 L = kRes ? sm.st[s].lam[tid] : make_float2(0.f, 0.f);
      residual_terms<kRes, kMon, kPrecise>(tt, L, six_det * a.cD, six_det * a.cH, sr, sh, sd);
    }
    __syncthreads();
  }
  cp_async_wait<0>();
  if (abort_flag && tid == 0) {
    mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[k & 1]), (k >> 1) & 1, kMaxPolls);
    if (issued_next) mbar_wait(reinterpret_cast<uint64_t*>(&sm.bar[(k & 1) ^ 1]), ((k + 1) >> 1) & 1, kMaxPolls);
  }
  // every CTA adds its sums, even after a timeout; the sticky timeout flag
  // marks the sweep invalid for the host
  finish_residual<kRes, kMon>(d, a, sr, sh, sd);
}

// Tile variant, one CTA per patch: the tet records are loaded straight into
// registers and the vertex neighbourhood into shared memory; many resident
// CTAs per SM overlap each other's load and compute phases.  The corner
// contributions are reduced per patch vertex in shared memory, in the fixed
// order of the patch's vertex -> corner lists, so that one
// red.global.add.v4 per patch vertex (instead of one per tet corner) reaches
// the L2.
// kReduce: reduce per patch vertex before the global reduction (else one
// red.global.add.v4 per tet corner).
template <bool kBlockMode, bool kFirst, bool kPrecise, int kP, bool kReduce>
__global__ void __launch_bounds__(kP) k_project_patch1(Dev d, int cur, float cD, float cH, float relax_h,
                                                      float relax_d) {
  if (stopped(d)) return;
  __shared__ float4 sp[256];
  __shared__ int sg[256];
  __shared__ float4 sdp[kReduce ? 4 * kP : 1];
  __shared__ __align__(16) uint16_t sslot[kReduce ? 4 * kP : 8];
  __shared__ uint16_t sstart[kReduce ? 257 : 1];
  const int p = blockIdx.x;
  const int vb = __ldg(d.voff + p);
  const int nv = __ldg(d.voff + p + 1) - vb;
  const int t0 = p * kP;
  const int nt = d.T - t0 < kP ? d.T - t0 : kP;
  const int t = t0 + threadIdx.x;
  const bool has = threadIdx.x < nt;
  Tet tt;
  uint32_t lid = 0;
  float2 L = make_float2(0.f, 0.f);
  if (has) {
    const float4 A = __ldg(d.dm_a + t), B = __ldg(d.dm_b + t);
    tt.dm[0] = A.x; tt.dm[1] = A.y; tt.dm[2] = A.z;
    tt.dm[3] = A.w; tt.dm[4] = B.x; tt.dm[5] = B.y;
    tt.dm[6] = B.z; tt.dm[7] = B.w; tt.dm[8] = __ldg(d.dm_c + t);
    lid = __ldg(d.lid + t);
    if (!kFirst) L = d.lam[t];
  }
  // the patch's vertex -> corner lists: 4 kP u16 slots (16-byte chunks) + starts
  if (kReduce) {
    const uint4* src = reinterpret_cast<const uint4*>(d.pv_slots + (size_t)4 * kP * p);
    uint4* dst = reinterpret_cast<uint4*>(sslot);
    for (int k = threadIdx.x; k < kP / 2; k += kP) dst[k] = __ldg(src + k);
    if (threadIdx.x == 0) sstart[nv] = (uint16_t)(4 * nt);
  }
  const float4* P = d.p[cur];
  for (int j = threadIdx.x; j < nv; j += kP) {
    const int g = __ldg(d.pverts + vb + j);
    sg[j] = g;
    if (kReduce) sstart[j] = __ldg(d.pv_start + vb + j);
    sp[j] = ldg4(P + g);
  }
  __syncthreads();
  if (has) {
    const int l[4] = {(int)(lid & 0xffu), (int)((lid >> 8) & 0xffu), (int)((lid >> 16) & 0xffu), (int)(lid >> 24)};
#pragma unroll
    for (int c = 0; c < 4; ++c) tt.p[c] = sp[l[c]];
    const float six_det = 6.f * det9(tt.dm);
    float3 dp[4];
    float cnt;
    project_tet<kBlockMode, kPrecise>(tt, six_det * cD, six_det * cH, relax_h, relax_d, L, dp, cnt);
    d.lam[t] = L;
    if (kReduce) {
#pragma unroll
      for (int c = 0; c < 4; ++c) sdp[4 * threadIdx.x + c] = make_float4(dp[c].x, dp[c].y, dp[c].z, cnt);
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c) red_add_v4(d.dx + sg[l[c]], dp[c].x, dp[c].y, dp[c].z, cnt);
    }
  }
  if (!kReduce) return;
  __syncthreads();
  for (int j = threadIdx.x; j < nv; j += kP) {
    const int s0 = sstart[j], s1 = sstart[j + 1];
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = s0; k < s1; ++k) {
      const float4 c = sdp[sslot[k]];
      acc.x += c.x;
      acc.y += c.y;
      acc.z += c.z;
      acc.w += c.w;
    }
    red_add_v4(d.dx + sg[j], acc.x, acc.y, acc.z, acc.w);
  }
}

// Tile variant, one CTA per patch, kTPT consecutive tets per thread;
// corners shared along a thread's chain are summed in registers before the
// global reduction (project_chain).
template <bool kBlockMode, bool kFirst, bool kPrecise, int kP, int kTPT>
__global__ void __launch_bounds__(kP / kTPT, project_min_blocks(kTPT)) k_project_patchN(Dev d, int cur, float cD, float cH, float relax_h,
                                                             float relax_d) {
  if (stopped(d)) return;
  constexpr int kThreads = kP / kTPT;
  __shared__ float4 sp[256];
  __shared__ int sg[256];
  const int p = blockIdx.x;
  const int vb = __ldg(d.voff + p);
  const int nv = __ldg(d.voff + p + 1) - vb;
  const int t0 = p * kP;
  const int nt = d.T - t0 < kP ? d.T - t0 : kP;
  const int l0 = kTPT * threadIdx.x;
  float4 A[kTPT], B[kTPT];
  float C[kTPT];
  uint32_t lid[kTPT];
  float2 L[kTPT];
  const uint64_t pol = l2_policy(d.l2_keep != 0);
  if (kTPT == 2 && l0 + 1 < nt) {  // a full pair: one load per record array
    const int t = t0 + l0;
    ldg_pair(d.dm_a + t, pol, A[0], A[1]);
    ldg_pair(d.dm_b + t, pol, B[0], B[1]);
    const float2 c = ldg_pair(d.dm_c + t, pol);
    const uint2 li = ldg_pair(d.lid + t, pol);
    C[0] = c.x;
    C[1] = c.y;
    lid[0] = li.x;
    lid[1] = li.y;
    if (!kFirst) {
      const float4 l2 = *reinterpret_cast<const float4*>(d.lam + t);
      L[0] = make_float2(l2.x, l2.y);
      L[1] = make_float2(l2.z, l2.w);
    } else {
      L[0] = L[1] = make_float2(0.f, 0.f);
    }
  } else {
#pragma unroll
    for (int k = 0; k < kTPT; ++k) {
      A[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      B[k] = A[k];
      C[k] = 0.f;
      lid[k] = 0u;
      L[k] = make_float2(0.f, 0.f);
      if (l0 + k < nt) {
        A[k] = ldg_hint(d.dm_a + t0 + l0 + k, pol);
        B[k] = ldg_hint(d.dm_b + t0 + l0 + k, pol);
        C[k] = ldg_hint(d.dm_c + t0 + l0 + k, pol);
        lid[k] = ldg_hint(d.lid + t0 + l0 + k, pol);
        if (!kFirst) L[k] = d.lam[t0 + l0 + k];
      }
    }
  }
  // the records and multipliers above were written two kernels back; the
  // positions come from the update that precedes this launch
  pdl_wait();
  pdl_trigger();
  const float4* P = d.p[cur];
  for (int j = threadIdx.x; j < nv; j += kThreads) {
    const int g = ldg_hint(d.pverts + vb + j, pol);
    sg[j] = g;
    sp[j] = ldg4(P + g);
  }
  __syncthreads();
  const int n = nt - l0 < kTPT ? nt - l0 : kTPT;
  project_chain<kBlockMode, kPrecise, kTPT>(A, B, C, lid, L, d.lam + t0 + l0, n, sp, sg, d.dx, cD, cH, relax_h,
                                            relax_d, d.paired != 0);
}

template <bool kRes, bool kMon, bool kPrecise, int kP>
__global__ void __launch_bounds__(kP) k_residual_patch1(Dev d, SweepArgs a) {
  if (stopped(d)) return;
  __shared__ float4 sp[256];
  float sr = 0.f, sh = 0.f, sd = 0.f;
  const float4* P = d.p[a.cur];
  const int n = d.n_patches;
  for (int q = blockIdx.x; q < n; q += gridDim.x) {
    const int p = a.reverse ? n - 1 - q : q;
    const int vb = __ldg(d.voff + p);
    const int nv = __ldg(d.voff + p + 1) - vb;
    const int t = p * kP + threadIdx.x;
    const bool has = t < d.T;
    Tet tt;
    uint32_t lid = 0;
    float2 L = make_float2(0.f, 0.f);
    if (has) {
      const float4 A = __ldg(d.dm_a + t), B = __ldg(d.dm_b + t);
      tt.dm[0] = A.x; tt.dm[1] = A.y; tt.dm[2] = A.z;
      tt.dm[3] = A.w; tt.dm[4] = B.x; tt.dm[5] = B.y;
      tt.dm[6] = B.z; tt.dm[7] = B.w; tt.dm[8] = __ldg(d.dm_c + t);
      lid = __ldg(d.lid + t);
      if (kRes) L = d.lam[t];
    }
    __syncthreads();  // the previous patch's readers are done with sp
    for (int j = threadIdx.x; j < nv; j += kP) {
      const int g = __ldg(d.pverts + vb + j);
      const float3 x = post_position(ldg4(P + g), ldg4(d.dx + g));
      sp[j] = make_float4(x.x, x.y, x.z, 0.f);
    }
    __syncthreads();
    if (has) {
      tt.p[0] = sp[lid & 0xffu];
      tt.p[1] = sp[(lid >> 8) & 0xffu];
      tt.p[2] = sp[(lid >> 16) & 0xffu];
      tt.p[3] = sp[lid >> 24];
      const float six_det = 6.f * det9(tt.dm);
      residual_terms<kRes, kMon, kPrecise>(tt, L, six_det * a.cD, six_det * a.cH, sr, sh, sd);
    }
  }
  finish_residual<kRes, kMon>(d, a, sr, sh, sd);
}

// Residual over patches with kTPT consecutive tets per thread (one CTA per
// patch at a time, kP / kTPT threads).  Loading the patch's records before
// the vertex tile lets both sets of loads be in flight together.
template <bool kRes, bool kMon, bool kPrecise, int kP, int kTPT>
__global__ void __launch_bounds__(kP / kTPT) k_residual_patchN(Dev d, SweepArgs a) {
  pdl_wait();  // the Jacobi sums and multipliers of the projection before it
  pdl_trigger();
  if (stopped(d)) return;
  constexpr int kThreads = kP / kTPT;
  __shared__ float4 sp[256];
  float sr = 0.f, sh = 0.f, sd = 0.f;
  const float4* P = d.p[a.cur];
  const int n = d.n_patches;
  const int l0 = kTPT * threadIdx.x;
  const uint64_t pol = l2_policy(d.l2_keep != 0);
  for (int q = blockIdx.x; q < n; q += gridDim.x) {
    const int p = a.reverse ? n - 1 - q : q;
    const int vb = __ldg(d.voff + p);
    const int nv = __ldg(d.voff + p + 1) - vb;
    const int t0 = p * kP + l0;
    float4 A[kTPT], B[kTPT];
    float C[kTPT];
    uint32_t lid[kTPT];
    float2 L[kTPT];
    if (kTPT == 2 && t0 + 1 < d.T) {  // a full pair: one load per record array
      ldg_pair(d.dm_a + t0, pol, A[0], A[1]);
      ldg_pair(d.dm_b + t0, pol, B[0], B[1]);
      const float2 c = ldg_pair(d.dm_c + t0, pol);
      const uint2 li = ldg_pair(d.lid + t0, pol);
      C[0] = c.x;
      C[1] = c.y;
      lid[0] = li.x;
      lid[1] = li.y;
      L[0] = L[1] = make_float2(0.f, 0.f);
      if (kRes) {
        const float4 l2 = *reinterpret_cast<const float4*>(d.lam + t0);
        L[0] = make_float2(l2.x, l2.y);
        L[1] = make_float2(l2.z, l2.w);
      }
    } else {
#pragma unroll
      for (int k = 0; k < kTPT; ++k) {
        if (t0 + k < d.T) {
          A[k] = ldg_hint(d.dm_a + t0 + k, pol);
          B[k] = ldg_hint(d.dm_b + t0 + k, pol);
          C[k] = ldg_hint(d.dm_c + t0 + k, pol);
          lid[k] = ldg_hint(d.lid + t0 + k, pol);
          L[k] = kRes ? d.lam[t0 + k] : make_float2(0.f, 0.f);
        }
      }
    }
    __syncthreads();  // the previous patch's readers are done with sp
    for (int j = threadIdx.x; j < nv; j += kThreads) {
      const int g = ldg_hint(d.pverts + vb + j, pol);
      const float3 x = post_position(ldg4(P + g), ldg4(d.dx + g));
      sp[j] = make_float4(x.x, x.y, x.z, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kTPT; ++k) {
      if (t0 + k >= d.T) break;
      Tet tt;
      tt.dm[0] = A[k].x; tt.dm[1] = A[k].y; tt.dm[2] = A[k].z;
      tt.dm[3] = A[k].w; tt.dm[4] = B[k].x; tt.dm[5] = B[k].y;
      tt.dm[6] = B[k].z; tt.dm[7] = B[k].w; tt.dm[8] = C[k];
      tt.p[0] = sp[lid[k] & 0xffu];
      tt.p[1] = sp[(lid[k] >> 8) & 0xffu];
      tt.p[2] = sp[(lid[k] >> 16) & 0xffu];
      tt.p[3] = sp[lid[k] >> 24];
      const float six_det = 6.f * det9(tt.dm);
      residual_terms<kRes, kMon, kPrecise>(tt, L[k], six_det * a.cD, six_det * a.cH, sr, sh, sd);
    }
  }
  finish_residual<kRes, kMon>(d, a, sr, sh, sd);
}

// Field transfer in caller vertex order (mesh.verts.<f>.from_numpy / to_numpy).
// f == nullptr: the predicted positions of stop mode, p[st->pos_cur].
__global__ void __launch_bounds__(kBlock) k_import(Dev d, float4* f, const float* __restrict__ src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
  if (!f) f = d.p[d.st->pos_cur];
  const int j = d.perm ? d.perm[i] : i;
  float4 o = f[i];
  o.x = src[3 * (size_t)j];
  o.y = src[3 * (size_t)j + 1];
  o.z = src[3 * (size_t)j + 2];
  f[i] = o;
}

__global__ void __launch_bounds__(kBlock) k_export(Dev d, const float4* f, float* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
  if (!f) f = d.p[d.st->pos_cur];
  const int j = d.perm ? d.perm[i] : i;
  const float4 o = f[i];
  dst[3 * (size_t)j] = o.x;
  dst[3 * (size_t)j + 1] = o.y;
  dst[3 * (size_t)j + 2] = o.z;
}

// Index validation: every tet corner (and CSR slot) must address a vertex.
__global__ void k_validate(Dev d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < d.T) {
    const int4 id = d.tets[t];
    if ((unsigned)id.x >= (unsigned)d.V || (unsigned)id.y >= (unsigned)d.V || (unsigned)id.z >= (unsigned)d.V ||
        (unsigned)id.w >= (unsigned)d.V)
      d.st->bad_mesh = 1;
  }
  if (d.v2t_off != nullptr && t <= d.V) {
    const int o = d.v2t_off[t];
    if (o < 0 || o > 4 * d.T) d.st->bad_mesh = 1;
  }
  if (d.lid != nullptr && t < d.T) {
    const int p = t / d.P;
    const int nv = d.voff[p + 1] - d.voff[p];
    const uint32_t l = d.lid[t];
    if ((int)(l & 0xffu) >= nv || (int)((l >> 8) & 0xffu) >= nv || (int)((l >> 16) & 0xffu) >= nv ||
        (int)(l >> 24) >= nv)
      d.st->bad_mesh = 1;
  }
  if (d.voff != nullptr && t < d.n_patches) {
    const int a = d.voff[t], b = d.voff[t + 1];
    if (a < 0 || b < a || b > d.n_pverts || b - a > 256) d.st->bad_mesh = 1;
    if (t == 0 && a != 0) d.st->bad_mesh = 1;
    if (t == d.n_patches - 1 && b != d.n_pverts) d.st->bad_mesh = 1;
    if (!d.st->bad_mesh) {
      // local vertex -> corner lists: starts nondecreasing in [0, 4 nt], slots < 4 nt
      const int nt = d.T - t * d.P < d.P ? d.T - t * d.P : d.P;
      int prev = 0;
      for (int k = a; k < b; ++k) {
        const int st = d.pv_start[k];
        if (st < prev || st > 4 * nt) d.st->bad_mesh = 1;
        prev = st;
      }
      const uint16_t* sl = d.pv_slots + (size_t)4 * d.P * t;
      for (int k = 0; k < 4 * nt; ++k)
        if (sl[k] >= 4 * nt) d.st->bad_mesh = 1;
    }
  }
  if (d.pverts != nullptr) {
    for (int k = t; k < d.n_pverts; k += gridDim.x * blockDim.x)
      if ((unsigned)d.pverts[k] >= (unsigned)d.V) d.st->bad_mesh = 1;
  }
  if (d.perm != nullptr && t < d.V) {
    if ((unsigned)d.perm[t] >= (unsigned)d.V) d.st->bad_mesh = 1;
  }
  if (d.v2t_slot != nullptr) {
    for (int k = t; k < 4 * d.T; k += gridDim.x * blockDim.x) {
      const int s = d.v2t_slot[k];
      if ((unsigned)s >= (unsigned)(4 * d.T)) d.st->bad_mesh = 1;
    }
  }
}

// ---------------------------------------------------------------------------
// Residual sweep that allocates nothing (xpbd_residual_noalloc).
//
// Its scratch -- one FP64 partial triple per CTA and the CTA ticket -- lives in
// the file-scope array below, which every GPU that loads the library holds
// until the process exits.  One CTA covers 256 tets, so a call handles at most
// kNoAllocMaxBlocks * 256 tets.  The last CTA sums the partials in CTA order,
// so the result does not depend on which CTAs finish first.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxBlocks = 8192;
constexpr long long kNoAllocMaxTets = (long long)kNoAllocMaxBlocks * kBlock;  // 2,097,152
constexpr int kNoAllocTicket = 3 * kNoAllocMaxBlocks;  // slot of the CTA ticket (as a u64)
static __device__ __align__(256) double g_noalloc_scratch[3 * kNoAllocMaxBlocks + 1];

template <bool kPrecise>
__global__ void __launch_bounds__(kBlock) k_residual_noalloc(Dev d, float cD, float cH, double* scratch,
                                                             double* out) {
  __shared__ double red[3][kBlock / 32];
  __shared__ bool last;
  const int t = blockIdx.x * kBlock + threadIdx.x;
  float sr = 0.f, sh = 0.f, sd = 0.f;
  if (t < d.T) {
    int4 id;
    Tet tt;
    load_tet(d, t, id, tt);
    const int vid[4] = {id.x, id.y, id.z, id.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float3 q = post_position(ldg4(d.p[0] + vid[c]), ldg4(d.dx + vid[c]));
      tt.p[c] = make_float4(q.x, q.y, q.z, 0.f);
    }
    const float inv_v0 = 1.f / tt.V0;
    float aD = cD * inv_v0, aH = cH * inv_v0;
    if (d.tinv_mu) {  // per-tet materials: cD = cH = 1 / dt^2
      aD *= __ldg(d.tinv_mu + t);
      aH *= __ldg(d.tinv_la + t);
    }
    residual_terms<true, true, kPrecise>(tt, d.lam[t], aD, aH, sr, sh, sd);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double r0 = warp_sum((double)sr), r1 = warp_sum((double)sh), r2 = warp_sum((double)sd);
  if (lane == 0) {
    red[0][warp] = r0;
    red[1][warp] = r1;
    red[2][warp] = r2;
  }
  __syncthreads();
  unsigned long long* ticket = reinterpret_cast<unsigned long long*>(scratch + kNoAllocTicket);
  if (threadIdx.x == 0) {
    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
    for (int k = 0; k < kBlock / 32; ++k) {
      b0 += red[0][k];
      b1 += red[1][k];
      b2 += red[2][k];
    }
    scratch[3 * blockIdx.x + 0] = b0;
    scratch[3 * blockIdx.x + 1] = b1;
    scratch[3 * blockIdx.x + 2] = b2;
    __threadfence();
    last = atomicAdd(ticket, 1ull) == (unsigned long long)(gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // fixed-order sum of the CTA partials: thread j takes CTAs j, j + 256, ...
  const volatile double* part = scratch;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += kBlock) {
    a0 += part[3 * k + 0];
    a1 += part[3 * k + 1];
    a2 += part[3 * k + 2];
  }
  __syncthreads();
  const double w0 = warp_sum(a0), w1 = warp_sum(a1), w2 = warp_sum(a2);
  if (lane == 0) {
    red[0][warp] = w0;
    red[1][warp] = w1;
    red[2][warp] = w2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0, H = 0.0, D = 0.0;
    for (int k = 0; k < kBlock / 32; ++k) {
      S += red[0][k];
      H += red[1][k];
      D += red[2][k];
    }
    const double n = (double)d.T;
    out[0] = S / n;
    out[1] = H / n;
    out[2] = D / n;
    *ticket = 0ull;
  }
}

}  // namespace xpbd

namespace xpbd {

// Accessors of the single-body layout for the adjoint kernels.
__device__ __forceinline__ int adj_verts(const Dev& d) { return d.V; }
__device__ __forceinline__ int adj_tets(const Dev& d) { return d.T; }
__device__ __forceinline__ float adj_omega(const Dev& d, int, int k) { return (float)d.hist[4 * k + 1]; }
__device__ __forceinline__ int adj_nbodies(const Dev&) { return 1; }
__device__ __forceinline__ int adj_vbody(const Dev&, int) { return 0; }
__device__ __forceinline__ double adj_hist(const Dev& d, int, int k, int c) { return d.hist[4 * (size_t)k + c]; }
__device__ __forceinline__ double adj_body_tets(const Dev& d, int) { return (double)d.T; }
__device__ __forceinline__ bool adj_load_tet(const Dev& d, int t, int (&vid)[4], Tet& tt, float& inv_v0, float& m_mu,
                                             float& m_la) {
  int4 id;
  load_tet(d, t, id, tt);
  vid[0] = id.x;
  vid[1] = id.y;
  vid[2] = id.z;
  vid[3] = id.w;
  inv_v0 = 1.f / tt.V0;
  m_mu = d.tinv_mu ? __ldg(d.tinv_mu + t) : 1.f;
  m_la = d.tinv_mu ? __ldg(d.tinv_la + t) : 1.f;
  return true;
}

}  // namespace xpbd

#include "xpbd_adjoint.cuh"

// ===========================================================================
// C ABI
// ===========================================================================

using namespace xpbd;

namespace {

thread_local std::string g_last_error;

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

// On failure the runtime's per-thread last error is cleared as well, so that a
// later cudaGetLastError check does not report this call again.
#define XPBD_CUDA(call)                                                            \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      cudaGetLastError();                                                          \
      return fail(XPBD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    }                                                                              \
  } while (0)

struct GraphKey {
  double frame_dt = -1.0, dt = -1.0;
  int substeps = -1;
};

struct Solver {
  // profiling (xpbd_set_profiling): event pairs per kernel class
  bool profiling = false;
  // programmatic dependent launch of the iteration's kernels (off with
  // XPBD_NO_PDL=1 in the environment at creation); pdl_now: the launch being
  // issued may overlap its predecessor
  bool pdl = true;
  bool pdl_now = false;
  int l2_auto = 0;  // automatic L2 policy of the tile sweeps (xpbd_set_l2_hint)
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[XPBD_K_COUNT];
  double prof_ms[XPBD_K_COUNT] = {0, 0, 0, 0, 0, 0};
  long long prof_n[XPBD_K_COUNT] = {0, 0, 0, 0, 0, 0};
  xpbd_params prm{};
  Dev d{};
  int device = 0;
  int sm_count = 0;
  int res_grid = 0;        // grid of the grid-stride residual kernels
  int patch_grid = 0;      // grid of the persistent tile kernels
  int patch2_grid = 0;     // grid of the persistent two-tets-per-thread tile projection
  int patch1_grid = 0;     // grid of the one-CTA-per-patch residual
  int patchN_grid = 0;     // grid of the two-tets-per-thread residual
  int tile_res_grid = 0;   // grid of the pipelined tile residual
  int max_records = 0;
  int cur = 0;  // buffer holding the current predicted positions
  cudaStream_t cap = nullptr;
  cudaStream_t cap_body = nullptr;  // captures the body of a stop-mode loop node
  float4* tape_post = nullptr;      // taping through omega: where the update writes post-Jacobi positions
  float4* tape_xs = nullptr;        // taping: where the update writes the next iteration's positions
  cudaGraphExec_t exec = nullptr;
  GraphKey key;
  // profiling with use_graph: the frame graph carries an event record node
  // before and after every launch; the events belong to that graph
  cudaGraphExec_t pexec = nullptr;
  GraphKey pkey;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> gpairs[XPBD_K_COUNT];
  bool greplay = false;    // a replay of pexec whose times are not yet added
  bool capturing = false;  // a frame is being captured on cap
};

inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

cudaEvent_t take_event(Solver* s) {
  if (!s->pool.empty()) {
    cudaEvent_t e = s->pool.back();
    s->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Brackets one launch with events when profiling is on.
struct Prof {
  Solver* s;
  int cls;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  Prof(Solver* s_, int cls_, cudaStream_t st_) : s(s_), cls(cls_), st(st_) {
    if (s->profiling) {
      a = take_event(s);
      if (a) record(a);
    }
  }
  ~Prof() {
    if (!a) return;
    cudaEvent_t b = take_event(s);
    if (!b) return;
    record(b);
    s->pending[cls].push_back({a, b});
  }
  // under stream capture an event record becomes a graph event record node
  // only with cudaEventRecordExternal (otherwise it marks a capture dependency)
  void record(cudaEvent_t e) const {
    if (s->capturing) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    else cudaEventRecord(e, st);
  }
};

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }


int check_params(const xpbd_params* p) {
  if (!p) return fail(XPBD_ERR_INVALID_ARGUMENT, "params is NULL");
  if (p->constraints_iter < 0) return fail(XPBD_ERR_INVALID_ARGUMENT, "constraints_iter < 0");
  if (p->scatter != XPBD_SCATTER_ATOMIC && p->scatter != XPBD_SCATTER_GATHER && p->scatter != XPBD_SCATTER_PATCH)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown scatter variant");
  if (p->tets_per_thread != 0 && p->tets_per_thread != 1 && p->tets_per_thread != 2 && p->tets_per_thread != 4)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "tets_per_thread must be 0, 1, 2 or 4");
  if (!(p->lame_mu != 0.f) || !(p->lame_lambda != 0.f))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "Lame parameters must be non-zero");
  if (!(p->target_rel_residual >= 0.0) || !(p->residual_floor >= 0.0))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "target_rel_residual and residual_floor must be >= 0");
  return XPBD_OK;
}

// Stop mode: each substep iterates until its residual target (or the cap).
inline bool stop_mode(const xpbd_params& p) { return p.target_rel_residual > 0.0 || p.residual_floor > 0.0; }

// ---- launch helpers (all stream-ordered, no sync) --------------------------

int launch_begin(Solver* s, bool predict, bool sdf, float dt, cudaStream_t st) {
  Prof prof(s, XPBD_K_BEGIN, st);
  const int g = blocks_for(s->d.V);
  const float* gr = s->prm.gravity;
  if (predict && sdf) k_begin<true, true><<<g, kBlock, 0, st>>>(s->d, dt, gr[0], gr[1], gr[2], s->cur);
  else if (predict) k_begin<true, false><<<g, kBlock, 0, st>>>(s->d, dt, gr[0], gr[1], gr[2], s->cur);
  else if (sdf) k_begin<false, true><<<g, kBlock, 0, st>>>(s->d, dt, gr[0], gr[1], gr[2], s->cur);
  return XPBD_OK;
}

template <bool kBlockMode, bool kFirst, bool kPrecise>
void launch_project_t(Solver* s, float cD, float cH, cudaStream_t st) {
  const int g = blocks_for(s->d.T);
  const xpbd_params& p = s->prm;
  if (p.scatter == XPBD_SCATTER_GATHER)
    k_project<kBlockMode, kFirst, kPrecise, true><<<g, kBlock, 0, st>>>(s->d, s->cur, cD, cH, p.hydrostatic_relaxation,
                                                                        p.deviatoric_relaxation);
  else
    k_project<kBlockMode, kFirst, kPrecise, false><<<g, kBlock, 0, st>>>(s->d, s->cur, cD, cH, p.hydrostatic_relaxation,
                                                                         p.deviatoric_relaxation);
}

template <bool kBlockMode, bool kFirst, bool kPrecise, int kP>
void launch_project_patch_p(Solver* s, float cD, float cH, cudaStream_t st) {
  const xpbd_params& p = s->prm;
  if (p.patch_pipeline == 1 && kP == 256 && p.tets_per_thread == 2) {
    const int g = s->d.n_patches < s->patch2_grid ? s->d.n_patches : s->patch2_grid;
    k_project_tile2<kBlockMode, kFirst, kPrecise><<<g, 128, sizeof(TileSmem<false>), st>>>(
        s->d, s->cur, cD, cH, p.hydrostatic_relaxation, p.deviatoric_relaxation);
  } else if (p.patch_pipeline == 1 && kP == 256) {
    const int g = s->d.n_patches < s->patch_grid ? s->d.n_patches : s->patch_grid;
    k_project_tile<kBlockMode, kFirst, kPrecise><<<g, 256, sizeof(TileSmem<false>), st>>>(
        s->d, s->cur, cD, cH, p.hydrostatic_relaxation, p.deviatoric_relaxation);
  } else if (p.tets_per_thread == 2 && !p.patch_reduce) {
    launch_k(k_project_patchN<kBlockMode, kFirst, kPrecise, kP, 2>, s->d.n_patches, kP / 2, 0, st, s->pdl_now,
             s->d, s->cur, cD, cH, p.hydrostatic_relaxation, p.deviatoric_relaxation);
  } else if (p.tets_per_thread == 4 && !p.patch_reduce) {
    k_project_patchN<kBlockMode, kFirst, kPrecise, kP, 4><<<s->d.n_patches, kP / 4, 0, st>>>(
        s->d, s->cur, cD, cH, p.hydrostatic_relaxation, p.deviatoric_relaxation);
  } else {
    if (p.patch_reduce)
      k_project_patch1<kBlockMode, kFirst, kPrecise, kP, true><<<s->d.n_patches, kP, 0, st>>>(
          s->d, s->cur, cD, cH, p.hydrostatic_relaxation, p.deviatoric_relaxation);
    else
      k_project_patch1<kBlockMode, kFirst, kPrecise, kP, false><<<s->d.n_patches, kP, 0, st>>>(
          s->d, s->cur, cD, cH, p.hydrostatic_relaxation, p.deviatoric_relaxation);
  }
}

template <bool kBlockMode, bool kFirst, bool kPrecise>
void launch_project_patch_t(Solver* s, float cD, float cH, cudaStream_t st) {
  switch (s->d.P) {
    case 256: launch_project_patch_p<kBlockMode, kFirst, kPrecise, 256>(s, cD, cH, st); break;
    case 128: launch_project_patch_p<kBlockMode, kFirst, kPrecise, 128>(s, cD, cH, st); break;
    default: launch_project_patch_p<kBlockMode, kFirst, kPrecise, 64>(s, cD, cH, st); break;
  }
}

// 1 / (mu dt^2) and 1 / (lambda dt^2), rounded once from double; with per-tet
// materials both are 1 / dt^2 and the kernels multiply by the tet's 1 / mu, 1 / lambda
inline void compliance_factors(const Solver* s, float dt, float& cD, float& cH) {
  const double dt2 = (double)dt * (double)dt;
  if (s->d.tinv_mu) {
    cD = cH = (float)(1.0 / dt2);
    return;
  }
  cD = (float)(1.0 / ((double)s->prm.lame_mu * dt2));
  cH = (float)(1.0 / ((double)s->prm.lame_lambda * dt2));
}

template <bool kBlockMode, bool kFirst, bool kPrecise>
void launch_project_any(Solver* s, float cD, float cH, cudaStream_t st) {
  if (s->prm.scatter == XPBD_SCATTER_PATCH) launch_project_patch_t<kBlockMode, kFirst, kPrecise>(s, cD, cH, st);
  else launch_project_t<kBlockMode, kFirst, kPrecise>(s, cD, cH, st);
}

void launch_project(Solver* s, bool first, float dt, cudaStream_t st) {
  Prof prof(s, XPBD_K_PROJECT, st);
  const bool blk = s->prm.block_mode != 0, pr = s->prm.precise_hydro != 0;
  float cD, cH;
  compliance_factors(s, dt, cD, cH);
  if (blk) {
    if (first) pr ? launch_project_any<true, true, true>(s, cD, cH, st) : launch_project_any<true, true, false>(s, cD, cH, st);
    else pr ? launch_project_any<true, false, true>(s, cD, cH, st) : launch_project_any<true, false, false>(s, cD, cH, st);
  } else {
    if (first) pr ? launch_project_any<false, true, true>(s, cD, cH, st) : launch_project_any<false, true, false>(s, cD, cH, st);
    else pr ? launch_project_any<false, false, true>(s, cD, cH, st) : launch_project_any<false, false, false>(s, cD, cH, st);
  }
}

template <bool kRes, bool kMon, bool kPrecise, int kP>
void launch_residual_patch_p(Solver* s, const SweepArgs& a, cudaStream_t st) {
  const int n = s->d.n_patches;
  if (s->prm.patch_pipeline == 1 && kP == 256) {
    const int g = n < s->tile_res_grid ? n : s->tile_res_grid;
    k_residual_tile<kRes, kMon, kPrecise><<<g, 256, sizeof(TileSmem<true>), st>>>(s->d, a);
  } else if (s->prm.tets_per_thread == 2 && !s->prm.patch_reduce) {
    const int g = n < s->patchN_grid ? n : s->patchN_grid;
    launch_k(k_residual_patchN<kRes, kMon, kPrecise, kP, 2>, g, kP / 2, 0, st, s->pdl_now, s->d, a);
  } else {
    const int g = n < s->patch1_grid ? n : s->patch1_grid;
    k_residual_patch1<kRes, kMon, kPrecise, kP><<<g, kP, 0, st>>>(s->d, a);
  }
}

template <bool kRes, bool kMon, bool kPrecise>
void launch_residual_patch_t(Solver* s, const SweepArgs& a, cudaStream_t st) {
  switch (s->d.P) {
    case 256: launch_residual_patch_p<kRes, kMon, kPrecise, 256>(s, a, st); break;
    case 128: launch_residual_patch_p<kRes, kMon, kPrecise, 128>(s, a, st); break;
    default: launch_residual_patch_p<kRes, kMon, kPrecise, 64>(s, a, st); break;
  }
}

template <bool kRes, bool kMon>
void launch_residual_t(Solver* s, const SweepArgs& a, int grid, cudaStream_t st) {
  if (s->prm.scatter == XPBD_SCATTER_PATCH) {
    if (s->prm.precise_hydro) launch_residual_patch_t<kRes, kMon, true>(s, a, st);
    else launch_residual_patch_t<kRes, kMon, false>(s, a, st);
    return;
  }
  if (s->prm.precise_hydro) k_residual<kRes, kMon, true><<<grid, kBlock, 0, st>>>(s->d, a);
  else k_residual<kRes, kMon, false><<<grid, kBlock, 0, st>>>(s->d, a);
}

SweepArgs sweep_args(Solver* s, int par, float dt) {
  const xpbd_params& p = s->prm;
  SweepArgs a;
  a.cur = s->cur;
  compliance_factors(s, dt, a.cD, a.cH);
  a.par = par;
  a.reverse = p.sweep_order == 1 ? 1 : 0;
  return a;
}

void launch_residual(Solver* s, const SweepArgs& a, cudaStream_t st) {
  // residuals are summed for the Chebyshev recurrence and for stop mode
  const bool res = s->prm.cheb_enable != 0 || stop_mode(s->prm), mon = s->prm.monitor != 0;
  int grid = blocks_for(s->d.T);
  if (grid > s->res_grid) grid = s->res_grid;
  if (grid < 1) grid = 1;
  Prof prof(s, XPBD_K_RESIDUAL, st);
  if (res && mon) launch_residual_t<true, true>(s, a, grid, st);
  else if (res) launch_residual_t<true, false>(s, a, grid, st);
  else launch_residual_t<false, true>(s, a, grid, st);
}

// One Jacobi iteration (neohookean_solver.py:474-556).  `first`: the
// substep's iteration 0 (lambda reset); `par`: its index & 1; `sub`: the
// substep's index in the frame (for the iteration counts, -1: none); `cond`:
// the loop condition a stop-mode frame graph iterates on (nullptr: none).
void launch_iteration(Solver* s, bool first, int par, float dt, int rec_base, int sub, cudaStream_t st,
                      const cudaGraphConditionalHandle* cond) {
  const xpbd_params& p = s->prm;
  const bool stop = stop_mode(p);
  s->d.act = stop ? &s->d.st->slot[par].active : nullptr;
  // the fixed-count tile path (two tets per thread) launches its kernels so
  // that each may start while its predecessor drains
  s->pdl_now = s->pdl && !stop && !s->profiling && p.scatter == XPBD_SCATTER_PATCH && p.tets_per_thread == 2 &&
               !p.patch_pipeline && !p.patch_reduce;
  launch_project(s, first, dt, st);
  if (p.scatter == XPBD_SCATTER_GATHER) {
    Prof prof(s, XPBD_K_GATHER, st);
    k_gather<<<blocks_for(s->d.V), kBlock, 0, st>>>(s->d);
  }
  const bool cheb = p.cheb_enable != 0, mon = p.monitor != 0;
  if (cheb || mon || stop) launch_residual(s, sweep_args(s, par, dt), st);
  const int g = (s->d.V + kBlock * kUpdateVerts - 1) / (kBlock * kUpdateVerts);
  const bool reset = p.scatter != XPBD_SCATTER_GATHER;
  UpdArgs u{};
  u.par = par;
  u.rec_base = rec_base;
  u.K = p.constraints_iter;
  u.warmup = p.cheb_warmup;
  u.res = cheb;
  u.mon = mon;
  u.stop = stop;
  u.sub = sub;
  u.cur_next = cheb ? s->cur ^ 1 : s->cur;
  u.use_cond = cond != nullptr;
  if (cond) u.cond = *cond;
  u.post_out = s->tape_post;
  u.xs_out = s->tape_xs;
  u.pre = cheb || mon || stop;
  u.inv_n = s->d.T > 0 ? 1.0 / (double)s->d.T : 0.0;
  u.rho_min = p.rho_min;
  u.rho_max = p.rho_max;
  u.rho_beta = p.rho_beta;
  u.target = p.target_rel_residual;
  u.floor = p.residual_floor;
  Prof prof(s, XPBD_K_UPDATE, st);
  const bool o = s->pdl_now;
  if (cheb) {
    if (first) {
      if (reset) launch_k(k_update<true, true, true>, g, kBlock, 0, st, o, s->d, s->cur, p.cheb_gamma, u);
      else launch_k(k_update<true, true, false>, g, kBlock, 0, st, o, s->d, s->cur, p.cheb_gamma, u);
    } else {
      if (reset) launch_k(k_update<true, false, true>, g, kBlock, 0, st, o, s->d, s->cur, p.cheb_gamma, u);
      else launch_k(k_update<true, false, false>, g, kBlock, 0, st, o, s->d, s->cur, p.cheb_gamma, u);
    }
    s->cur ^= 1;
  } else {
    if (reset) launch_k(k_update<false, false, true>, g, kBlock, 0, st, o, s->d, s->cur, p.cheb_gamma, u);
    else launch_k(k_update<false, false, false>, g, kBlock, 0, st, o, s->d, s->cur, p.cheb_gamma, u);
  }
  s->pdl_now = false;
  s->d.act = nullptr;
}

// Stop mode under capture: iterations 0 and 1 as plain nodes, then a WHILE
// conditional node whose body is iterations of parity 0 and 1.  The update of
// every iteration from 1 on sets the loop condition (CTA 0, after the
// residual target test), so the graph launches no kernel of a substep that
// has stopped, except the rest of a body pass that started before it stopped;
// those kernels return at once.
int capture_stop_loop(Solver* s, float dt, int record_base, int sub, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  XPBD_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  if (cs != cudaStreamCaptureStatusActive || !g) return fail(XPBD_ERR_CUDA, "stop-mode loop outside a capture");
  cudaGraphConditionalHandle h = 0;
  XPBD_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
  launch_iteration(s, true, 0, dt, record_base, sub, st, nullptr);
  launch_iteration(s, false, 1, dt, record_base, sub, st, &h);
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nd = 0;
  XPBD_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &nd));
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  XPBD_CUDA(cudaGraphAddNode(&node, g, deps, edges, nd, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  XPBD_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  XPBD_CUDA(cudaStreamBeginCaptureToGraph(s->cap_body, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  launch_iteration(s, false, 0, dt, record_base, sub, s->cap_body, &h);
  launch_iteration(s, false, 1, dt, record_base, sub, s->cap_body, &h);
  cudaGraph_t out = nullptr;
  XPBD_CUDA(cudaStreamEndCapture(s->cap_body, &out));
  return XPBD_OK;
}

int launch_iterations(Solver* s, int K, float dt, int record_base, cudaStream_t st) {
  const int sub = record_base >= 0 && K > 0 ? record_base / K : -1;
  if (stop_mode(s->prm) && s->capturing && !s->profiling && K > 2)
    return capture_stop_loop(s, dt, record_base, sub, st);
  for (int it = 0; it < K; ++it) launch_iteration(s, it == 0, it & 1, dt, record_base, sub, st, nullptr);
  return XPBD_OK;
}

int do_solve_step(Solver* s, float dt, int record_base, cudaStream_t st) {
  const int K = s->prm.constraints_iter;
  if (record_base >= 0 && record_base + K > s->max_records)
    return fail(XPBD_ERR_HISTORY_FULL, "history holds " + std::to_string(s->max_records) + " records");
  launch_begin(s, false, true, dt, st);
  return launch_iterations(s, K, dt, record_base, st);
}

int do_substep(Solver* s, float dt, int record_base, cudaStream_t st) {
  const int K = s->prm.constraints_iter;
  if (record_base >= 0 && record_base + K > s->max_records)
    return fail(XPBD_ERR_HISTORY_FULL, "history holds " + std::to_string(s->max_records) + " records");
  s->cur = 0;
  launch_begin(s, true, true, dt, st);
  int r = launch_iterations(s, K, dt, record_base, st);
  if (r != XPBD_OK) return r;
  {
    Prof prof(s, XPBD_K_END, st);
    k_end<<<blocks_for(s->d.V), kBlock, 0, st>>>(s->d, s->cur, dt, s->prm.damping);
  }
  return XPBD_OK;
}

int enqueue_frame(Solver* s, double frame_dt, double dt, int substeps, cudaStream_t st) {
  // neohookean_solver.py:562-587: chunks of min(dt, left) in float64
  double left = frame_dt;
  int rec = 0;
  while (left > 0.0) {
    const double dt0 = dt < left ? dt : left;
    left -= dt0;
    const float sub_dt = (float)(dt0 / substeps);
    for (int k = 0; k < substeps; ++k) {
      const int base = rec + s->prm.constraints_iter <= s->max_records ? rec : -1;
      int r = do_substep(s, sub_dt, base, st);
      if (r != XPBD_OK) return r;
      rec += s->prm.constraints_iter;
    }
  }
  return XPBD_OK;
}

// Adds the event times of the last profiled graph replay (waits for it).
int accumulate_graph_profile(Solver* s) {
  if (!s->greplay) return XPBD_OK;
  s->greplay = false;
  for (int k = 0; k < XPBD_K_COUNT; ++k)
    for (auto& pr : s->gpairs[k]) {
      float t = 0.f;
      XPBD_CUDA(cudaEventSynchronize(pr.second));
      XPBD_CUDA(cudaEventElapsedTime(&t, pr.first, pr.second));
      s->prof_ms[k] += t;
      s->prof_n[k] += 1;
    }
  return XPBD_OK;
}

void drop_graph(Solver* s) {
  if (s->exec) cudaGraphExecDestroy(s->exec);
  s->exec = nullptr;
  s->key = GraphKey();
  accumulate_graph_profile(s);
  if (s->pexec) cudaGraphExecDestroy(s->pexec);
  s->pexec = nullptr;
  s->pkey = GraphKey();
  for (auto& v : s->gpairs) {
    for (auto& pr : v) {
      s->pool.push_back(pr.first);
      s->pool.push_back(pr.second);
    }
    v.clear();
  }
}

// Captures one frame into *exec.  With profiling on, the Prof brackets become
// event record nodes and their event pairs move to gpairs.
int capture_frame(Solver* s, double frame_dt, double dt, int substeps, cudaGraphExec_t* exec) {
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> direct[XPBD_K_COUNT];
  for (int k = 0; k < XPBD_K_COUNT; ++k) direct[k].swap(s->pending[k]);
  cudaError_t e = cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    for (int k = 0; k < XPBD_K_COUNT; ++k) s->pending[k].swap(direct[k]);
    XPBD_CUDA(e);
  }
  s->capturing = true;
  int r = enqueue_frame(s, frame_dt, dt, substeps, s->cap);
  s->capturing = false;
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(s->cap, &g);
  for (int k = 0; k < XPBD_K_COUNT; ++k) {
    for (auto& pr : s->pending[k]) s->gpairs[k].push_back(pr);
    s->pending[k].swap(direct[k]);
  }
  if (r != XPBD_OK) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return fail(XPBD_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    *exec = nullptr;
    return fail(XPBD_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  }
  return XPBD_OK;
}

}  // namespace

extern "C" {

int xpbd_abi_version(void) { return XPBD_ABI_VERSION; }

const char* xpbd_status_string(int status) {
  switch (status) {
    case XPBD_OK: return "ok";
    case XPBD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case XPBD_ERR_CUDA: return "CUDA error";
    case XPBD_ERR_NONFINITE: return "non-finite residual";
    case XPBD_ERR_NO_SDF: return "At least one SDF object must be provided.";
    case XPBD_ERR_BAD_MESH: return "bad mesh";
    case XPBD_ERR_HISTORY_FULL: return "history full";
    case XPBD_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

const char* xpbd_last_error(void) { return g_last_error.c_str(); }

int xpbd_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int xpbd_create(const xpbd_params* params, const xpbd_body* body, const xpbd_sdf* sdfs, int32_t n_sdf,
                int32_t max_records, void** out_handle) {
  g_last_error.clear();
  if (!out_handle || !body) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL body or handle pointer");
  *out_handle = nullptr;
  int r = check_params(params);
  if (r != XPBD_OK) return r;
  if (n_sdf <= 0 || !sdfs) return fail(XPBD_ERR_NO_SDF, "At least one SDF object must be provided.");
  for (int k = 0; k < n_sdf; ++k)
    if (sdfs[k].kind < XPBD_SDF_PLANE || sdfs[k].kind > XPBD_SDF_CUBE)
      return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown SDF kind");
  if (body->n_verts <= 0 || body->n_tets <= 0) return fail(XPBD_ERR_BAD_MESH, "empty mesh");
  if ((long long)body->n_tets * 4 >= (1ll << 31)) return fail(XPBD_ERR_BAD_MESH, "too many tets");
  if (!body->x || !body->v || !body->p0 || !body->p1 || !body->dx || !body->tets || !body->dm_a || !body->dm_b ||
      !body->dm_c || !body->v0 || !body->lam)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL body buffer");
  if (params->scatter == XPBD_SCATTER_GATHER && (!body->v2t_offsets || !body->v2t_slots || !body->corner_dx))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "gather variant needs v2t_offsets, v2t_slots and corner_dx");
  if (max_records < 0) return fail(XPBD_ERR_INVALID_ARGUMENT, "max_records < 0");
  const bool has_patch = body->tet_lid && body->patch_voff && body->patch_verts && body->pv_start && body->pv_slots;
  if (params->scatter == XPBD_SCATTER_PATCH && !has_patch)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "patch variant needs tet_lid, patch_voff, patch_verts, pv_start, pv_slots");
  if (has_patch) {
    const int P = body->patch_tets;
    if (P != 64 && P != 128 && P != 256) return fail(XPBD_ERR_INVALID_ARGUMENT, "patch_tets must be 64, 128 or 256");
    if (body->n_patches != (body->n_tets + P - 1) / P) return fail(XPBD_ERR_BAD_MESH, "n_patches != ceil(T / P)");
  }

  Solver* s = new (std::nothrow) Solver();
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "out of host memory");
  s->prm = *params;
  XPBD_CUDA(cudaGetDevice(&s->device));
  XPBD_CUDA(cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device));
  Dev& d = s->d;
  d.V = body->n_verts;
  d.T = body->n_tets;
  d.x = reinterpret_cast<float4*>(body->x);
  d.v = reinterpret_cast<float4*>(body->v);
  d.p[0] = reinterpret_cast<float4*>(body->p0);
  d.p[1] = reinterpret_cast<float4*>(body->p1);
  d.dx = reinterpret_cast<float4*>(body->dx);
  d.tets = reinterpret_cast<const int4*>(body->tets);
  d.dm_a = reinterpret_cast<const float4*>(body->dm_a);
  d.dm_b = reinterpret_cast<const float4*>(body->dm_b);
  d.dm_c = body->dm_c;
  d.v0 = body->v0;
  d.lam = reinterpret_cast<float2*>(body->lam);
  d.tinv_mu = body->tet_inv_mu;
  d.tinv_la = body->tet_inv_lambda;
  if ((d.tinv_mu == nullptr) != (d.tinv_la == nullptr)) {
    delete s;
    return fail(XPBD_ERR_INVALID_ARGUMENT, "tet_inv_mu and tet_inv_lambda must be given together");
  }
  if (d.tinv_mu && params->scatter == XPBD_SCATTER_PATCH) {
    delete s;
    return fail(XPBD_ERR_INVALID_ARGUMENT, "per-tet materials need the ATOMIC or GATHER variant");
  }
  d.v2t_off = body->v2t_offsets;
  d.v2t_slot = body->v2t_slots;
  d.corner = reinterpret_cast<float4*>(body->corner_dx);
  d.perm = body->vert_perm;
  d.paired = body->tet_pairs != 0;
  if (has_patch) {
    d.n_patches = body->n_patches;
    d.P = body->patch_tets;
    d.lid = body->tet_lid;
    d.voff = body->patch_voff;
    d.pverts = body->patch_verts;
    d.pv_start = body->pv_start;
    d.pv_slots = body->pv_slots;
  }
  d.n_sdf = n_sdf;
  s->max_records = max_records;

  auto cleanup = [&](int status) {
    if (d.sdfs) cudaFree(const_cast<xpbd_sdf*>(d.sdfs));
    if (d.st) cudaFree(d.st);
    if (d.hist) cudaFree(d.hist);
    if (s->cap) cudaStreamDestroy(s->cap);
    if (s->cap_body) cudaStreamDestroy(s->cap_body);
    delete s;
    return status;
  };
  xpbd_sdf* dsdf = nullptr;
  cudaError_t e = cudaMalloc(&dsdf, sizeof(xpbd_sdf) * n_sdf);
  if (e != cudaSuccess) return cleanup(fail(XPBD_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e)));
  d.sdfs = dsdf;
  e = cudaMemcpy(dsdf, sdfs, sizeof(xpbd_sdf) * n_sdf, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&d.st, sizeof(DevState));
  if (e == cudaSuccess) e = cudaMalloc(&d.hist, sizeof(double) * 4 * (size_t)(max_records > 0 ? max_records : 1));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cap_body, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cleanup(fail(XPBD_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e)));
  d.dyn_end = stop_mode(*params) ? 1 : 0;
  if (has_patch) {
    e = cudaMemcpy(&d.n_pverts, d.voff + d.n_patches, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cleanup(fail(XPBD_ERR_CUDA, std::string("patch offsets: ") + cudaGetErrorString(e)));
    // The tile sweeps load the read-only records (inv_Dm, local ids, patch
    // vertex lists) evict_last when they and the per-iteration state
    // (positions, previous positions, accumulators, multipliers) fit in
    // 80% of L2; past that, evict_last records would push the state out.
    int l2 = 0;
    if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, s->device) != cudaSuccess) l2 = 0;
    const double records = 40.0 * d.T + 4.0 * d.n_pverts;
    const double state = 48.0 * d.V + 8.0 * d.T;
    s->l2_auto = records + state <= 0.8 * l2;
    const char* no_pdl = std::getenv("XPBD_NO_PDL");
    s->pdl = !(no_pdl && no_pdl[0] == '1');
    d.l2_keep = s->l2_auto;
  }
  {
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_residual<true, false, false>, kBlock, 0) != cudaSuccess ||
        bps < 1)
      bps = 2;
    s->res_grid = s->sm_count * bps;
    bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_project_tile<true, false, true>, 256,
                                                      sizeof(TileSmem<false>)) != cudaSuccess ||
        bps < 1)
      bps = 2;
    s->patch_grid = s->sm_count * bps;
    bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_project_tile2<true, false, true>, 128,
                                                      sizeof(TileSmem<false>)) != cudaSuccess ||
        bps < 1)
      bps = 2;
    s->patch2_grid = s->sm_count * bps;
    bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_residual_tile<true, false, true>, 256,
                                                      sizeof(TileSmem<true>)) != cudaSuccess ||
        bps < 1)
      bps = 2;
    s->tile_res_grid = s->sm_count * bps;
    bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_residual_patch1<true, false, true, 256>, 256, 0) !=
            cudaSuccess ||
        bps < 1)
      bps = 2;
    s->patch1_grid = s->sm_count * bps;
    bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &bps, k_residual_patchN<true, false, true, 256, 2>, 128, 0) != cudaSuccess ||
        bps < 1)
      bps = 4;
    s->patchN_grid = s->sm_count * bps;
  }
  DevState h{};
  h.rho_hat = 0.999;  // neohookean_solver.py:65
  e = cudaMemcpy(d.st, &h, sizeof(h), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d.hist, 0, sizeof(double) * 4 * (size_t)(max_records > 0 ? max_records : 1));
  if (e != cudaSuccess) return cleanup(fail(XPBD_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e)));
  // validate the mesh indices once, before any kernel gathers through them
  int nval = (d.T > d.V + 1 ? d.T : d.V + 1);
  if (d.n_patches + 1 > nval) nval = d.n_patches + 1;
  k_validate<<<blocks_for(nval), kBlock>>>(d);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&h, d.st, sizeof(h), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cleanup(fail(XPBD_ERR_CUDA, std::string("validate: ") + cudaGetErrorString(e)));
  if (h.bad_mesh) return cleanup(fail(XPBD_ERR_BAD_MESH, "tet or CSR index out of range"));
  *out_handle = s;
  return XPBD_OK;
}

int xpbd_destroy(void* handle) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return XPBD_OK;
  drop_graph(s);
  for (auto& v : s->pending)
    for (auto& pr : v) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  for (cudaEvent_t e : s->pool) cudaEventDestroy(e);
  if (s->d.sdfs) cudaFree(const_cast<xpbd_sdf*>(s->d.sdfs));
  if (s->d.st) cudaFree(s->d.st);
  if (s->d.hist) cudaFree(s->d.hist);
  if (s->cap) cudaStreamDestroy(s->cap);
  if (s->cap_body) cudaStreamDestroy(s->cap_body);
  delete s;
  return XPBD_OK;
}

int xpbd_set_params(void* handle, const xpbd_params* params) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  int r = check_params(params);
  if (r != XPBD_OK) return r;
  if (params->scatter == XPBD_SCATTER_GATHER && (!s->d.v2t_off || !s->d.v2t_slot || !s->d.corner))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "gather variant needs CSR buffers given at create");
  if (params->scatter == XPBD_SCATTER_PATCH && !s->d.lid)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "patch variant needs the patch layout given at create");
  if (params->scatter == XPBD_SCATTER_PATCH && s->d.tinv_mu)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "per-tet materials need the ATOMIC or GATHER variant");
  if (std::memcmp(&s->prm, params, sizeof(xpbd_params)) != 0) drop_graph(s);
  s->prm = *params;
  s->d.dyn_end = stop_mode(*params) ? 1 : 0;
  return XPBD_OK;
}

int xpbd_set_sdfs(void* handle, const xpbd_sdf* sdfs, int32_t n_sdf, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !sdfs) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or SDF table");
  if (n_sdf != s->d.n_sdf) return fail(XPBD_ERR_INVALID_ARGUMENT, "SDF count differs from create");
  for (int k = 0; k < n_sdf; ++k)
    if (sdfs[k].kind < XPBD_SDF_PLANE || sdfs[k].kind > XPBD_SDF_CUBE)
      return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown SDF kind");
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  XPBD_CUDA(cudaMemcpy(const_cast<xpbd_sdf*>(s->d.sdfs), sdfs, sizeof(xpbd_sdf) * n_sdf, cudaMemcpyHostToDevice));
  return XPBD_OK;
}

int xpbd_apply_external_forces(void* handle, float dt, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  s->cur = 0;
  launch_begin(s, true, false, dt, S(stream));
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_solve_sdf_collision(void* handle, float dt, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  launch_begin(s, false, true, dt, S(stream));
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_solve_step(void* handle, float dt, int32_t record_base, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  int r = do_solve_step(s, dt, record_base, S(stream));
  if (r != XPBD_OK) return r;
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_advance(void* handle, float dt, float damping, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  Prof prof(s, XPBD_K_END, S(stream));
  k_end<<<blocks_for(s->d.V), kBlock, 0, S(stream)>>>(s->d, s->cur, dt, damping);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_substep(void* handle, float dt, int32_t record_base, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  int r = do_substep(s, dt, record_base, S(stream));
  if (r != XPBD_OK) return r;
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_solve(void* handle, double frame_dt, double dt, int32_t substeps, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  if (substeps <= 0 || !(dt > 0.0) || !(frame_dt >= 0.0))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "need substeps > 0, dt > 0, frame_dt >= 0");
  if (frame_dt / dt > 1e6) return fail(XPBD_ERR_INVALID_ARGUMENT, "frame_dt / dt too large");
  if (!s->prm.use_graph) {
    int r = enqueue_frame(s, frame_dt, dt, substeps, S(stream));
    if (r != XPBD_OK) return r;
    XPBD_CUDA(cudaGetLastError());
    return XPBD_OK;
  }
  if (s->profiling) {
    // the graph with timing nodes; the previous replay's times are added first
    // (a host wait per frame, only while profiling)
    if (!(s->pexec && s->pkey.frame_dt == frame_dt && s->pkey.dt == dt && s->pkey.substeps == substeps)) {
      drop_graph(s);
      int r = capture_frame(s, frame_dt, dt, substeps, &s->pexec);
      if (r != XPBD_OK) return r;
      s->pkey.frame_dt = frame_dt;
      s->pkey.dt = dt;
      s->pkey.substeps = substeps;
    }
    int r = accumulate_graph_profile(s);
    if (r != XPBD_OK) return r;
    XPBD_CUDA(cudaGraphLaunch(s->pexec, S(stream)));
    s->greplay = true;
    return XPBD_OK;
  }
  if (!(s->exec && s->key.frame_dt == frame_dt && s->key.dt == dt && s->key.substeps == substeps)) {
    drop_graph(s);
    int r = capture_frame(s, frame_dt, dt, substeps, &s->exec);
    if (r != XPBD_OK) return r;
    s->key.frame_dt = frame_dt;
    s->key.dt = dt;
    s->key.substeps = substeps;
  }
  XPBD_CUDA(cudaGraphLaunch(s->exec, S(stream)));
  return XPBD_OK;
}

int xpbd_read_history(void* handle, double* host_out, int32_t n, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !host_out || n < 0) return fail(XPBD_ERR_INVALID_ARGUMENT, "bad history read");
  if (n > s->max_records) return fail(XPBD_ERR_INVALID_ARGUMENT, "n > max_records");
  if (n == 0) return XPBD_OK;
  XPBD_CUDA(cudaMemcpyAsync(host_out, s->d.hist, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost, S(stream)));
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  return XPBD_OK;
}

int xpbd_read_iterations(void* handle, int32_t* host_out, int32_t n, int64_t* total, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || (n > 0 && !host_out) || n < 0 || n > kMaxCountedSubsteps)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "bad iteration-count read (n must be 0.." +
                                               std::to_string(kMaxCountedSubsteps) + ")");
  if (n > 0)
    XPBD_CUDA(cudaMemcpyAsync(host_out, s->d.st->iters, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost,
                              S(stream)));
  unsigned long long tot = 0;
  if (total)
    XPBD_CUDA(cudaMemcpyAsync(&tot, &s->d.st->total_iters, sizeof(tot), cudaMemcpyDeviceToHost, S(stream)));
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  if (total) *total = (int64_t)tot;
  return XPBD_OK;
}

int xpbd_get_rho_hat(void* handle, double* out, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !out) return fail(XPBD_ERR_INVALID_ARGUMENT, "bad argument");
  XPBD_CUDA(cudaMemcpyAsync(out, &s->d.st->rho_hat, sizeof(double), cudaMemcpyDeviceToHost, S(stream)));
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  return XPBD_OK;
}

int xpbd_set_rho_hat(void* handle, double value, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  // the value lives on the host stack: copy synchronously w.r.t. the stream
  XPBD_CUDA(cudaMemcpyAsync(&s->d.st->rho_hat, &value, sizeof(double), cudaMemcpyHostToDevice, S(stream)));
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  return XPBD_OK;
}

int xpbd_set_profiling(void* handle, int32_t enable) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  s->profiling = enable != 0;
  return XPBD_OK;
}

int xpbd_set_l2_hint(void* handle, int32_t mode, int32_t* active) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  if (mode < -1 || mode > 1) return fail(XPBD_ERR_INVALID_ARGUMENT, "l2 hint mode must be -1, 0 or 1");
  const int keep = mode < 0 ? s->l2_auto : mode;
  if (keep != s->d.l2_keep) {
    s->d.l2_keep = keep;
    drop_graph(s);  // the frame graph holds the kernels' Dev by value
  }
  if (active) *active = s->d.l2_keep;
  return XPBD_OK;
}

int xpbd_read_profile(void* handle, double* ms, int64_t* launches, int32_t n, int32_t reset, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || n < 0 || n > XPBD_K_COUNT) return fail(XPBD_ERR_INVALID_ARGUMENT, "bad profile read");
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  int r = accumulate_graph_profile(s);
  if (r != XPBD_OK) return r;
  for (int k = 0; k < XPBD_K_COUNT; ++k) {
    for (auto& pr : s->pending[k]) {
      float t = 0.f;
      XPBD_CUDA(cudaEventSynchronize(pr.second));
      XPBD_CUDA(cudaEventElapsedTime(&t, pr.first, pr.second));
      s->prof_ms[k] += t;
      s->prof_n[k] += 1;
      s->pool.push_back(pr.first);
      s->pool.push_back(pr.second);
    }
    s->pending[k].clear();
  }
  for (int k = 0; k < n; ++k) {
    if (ms) ms[k] = s->prof_ms[k];
    if (launches) launches[k] = s->prof_n[k];
  }
  if (reset)
    for (int k = 0; k < XPBD_K_COUNT; ++k) {
      s->prof_ms[k] = 0.0;
      s->prof_n[k] = 0;
    }
  return XPBD_OK;
}

// `known` = false for a valid field whose buffer only the device knows (the
// predicted positions in stop mode); the kernels then get nullptr.
static float4* field_ptr(Solver* s, int32_t field, bool& known) {
  known = true;
  switch (field) {
    case XPBD_FIELD_X: return s->d.x;
    case XPBD_FIELD_V: return s->d.v;
    case XPBD_FIELD_PRED_X:
      if (s->d.dyn_end) {
        known = false;
        return nullptr;
      }
      return s->d.p[s->cur];
    default: return nullptr;
  }
}

int xpbd_import_vec3(void* handle, int32_t field, const float* src, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !src) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or source");
  bool known = true;
  float4* f = field_ptr(s, field, known);
  if (!f && known) return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown field");
  k_import<<<blocks_for(s->d.V), kBlock, 0, S(stream)>>>(s->d, f, src);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_export_vec3(void* handle, int32_t field, float* dst, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !dst) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or destination");
  bool known = true;
  float4* f = field_ptr(s, field, known);
  if (!f && known) return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown field");
  k_export<<<blocks_for(s->d.V), kBlock, 0, S(stream)>>>(s->d, f, dst);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_save_rho_hat(void* handle, double* dst_device, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !dst_device) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or destination");
  XPBD_CUDA(cudaMemcpyAsync(dst_device, &s->d.st->rho_hat, sizeof(double), cudaMemcpyDeviceToDevice, S(stream)));
  return XPBD_OK;
}

int xpbd_load_rho_hat(void* handle, const double* src_device, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !src_device) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or source");
  XPBD_CUDA(cudaMemcpyAsync(&s->d.st->rho_hat, src_device, sizeof(double), cudaMemcpyDeviceToDevice, S(stream)));
  return XPBD_OK;
}

int xpbd_check_status(void* handle, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  int flag = 0;
  XPBD_CUDA(cudaMemcpyAsync(&flag, &s->d.st->nonfinite, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
  int tmo = 0;
  XPBD_CUDA(cudaMemcpyAsync(&tmo, &s->d.st->timeout, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  if (tmo) return fail(XPBD_ERR_TIMEOUT, "a bounded mbarrier wait timed out; results are invalid");
  return flag ? fail(XPBD_ERR_NONFINITE, "non-finite residual") : XPBD_OK;
}

static int check_diff(Solver* s) {
  if (!s->prm.block_mode) return fail(XPBD_ERR_INVALID_ARGUMENT, "the adjoint supports block mode only");
  if (stop_mode(s->prm)) return fail(XPBD_ERR_INVALID_ARGUMENT, "the adjoint needs a fixed iteration count");
  if (s->prm.scatter == XPBD_SCATTER_PATCH) return fail(XPBD_ERR_INVALID_ARGUMENT, "the adjoint needs ATOMIC or GATHER");
  if (!s->d.tinv_mu) return fail(XPBD_ERR_INVALID_ARGUMENT, "the adjoint needs per-tet materials");
  if (s->prm.constraints_iter > s->max_records)
    return fail(XPBD_ERR_HISTORY_FULL, "history shorter than constraints_iter");
  return XPBD_OK;
}

int xpbd_substep_tape(void* handle, float dt, const xpbd_tape* tape, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !tape || !tape->xs || !tape->lams || !tape->xpre || !tape->v1)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or tape buffer");
  int r = check_diff(s);
  if (r != XPBD_OK) return r;
  cudaStream_t st = S(stream);
  const int K = s->prm.constraints_iter, V = s->d.V, T = s->d.T;
  Tape tp{reinterpret_cast<float4*>(tape->xs), reinterpret_cast<float2*>(tape->lams),
          reinterpret_cast<float4*>(tape->xpre), reinterpret_cast<float4*>(tape->v1),
          reinterpret_cast<float4*>(tape->posts), tape->rho_in};
  if (tp.posts && !tp.rho_in) return fail(XPBD_ERR_INVALID_ARGUMENT, "a tape with posts needs rho_in");
  const float* g = s->prm.gravity;
  if (tp.posts)
    XPBD_CUDA(cudaMemcpyAsync(tp.rho_in, &s->d.st->rho_hat, sizeof(double), cudaMemcpyDeviceToDevice, st));
  k_tape_begin<Dev><<<blocks_for(V), kBlock, 0, st>>>(s->d, tp, dt, g[0], g[1], g[2]);
  s->cur = 0;
  launch_begin(s, true, true, dt, st);
  // iteration 0 enters with the predicted positions and zero multipliers; after
  // it the projection records the multipliers entering each iteration and the
  // update the positions entering the next (xs[K]: those after the last)
  XPBD_CUDA(cudaMemcpyAsync(tp.xs, s->d.p[s->cur], sizeof(float4) * V, cudaMemcpyDeviceToDevice, st));
  XPBD_CUDA(cudaMemsetAsync(tp.lams, 0, sizeof(float2) * T, st));
  for (int it = 0; it < K; ++it) {
    s->d.lam_tape = it > 0 ? tp.lams + (size_t)it * T : nullptr;
    s->tape_post = tp.posts ? tp.posts + (size_t)it * V : nullptr;
    s->tape_xs = tp.xs + (size_t)(it + 1) * V;
    launch_iteration(s, it == 0, it & 1, dt, 0, -1, st, nullptr);
    s->d.lam_tape = nullptr;
    s->tape_post = nullptr;
    s->tape_xs = nullptr;
  }
  if (tp.posts)  // the multipliers after the last iteration (the residual's lambda_K)
    XPBD_CUDA(cudaMemcpyAsync(tp.lams + (size_t)K * T, s->d.lam, sizeof(float2) * T, cudaMemcpyDeviceToDevice, st));
  if (tape->hist)
    XPBD_CUDA(cudaMemcpyAsync(tape->hist, s->d.hist, sizeof(double) * 4 * (size_t)K, cudaMemcpyDeviceToDevice, st));
  k_end<<<blocks_for(V), kBlock, 0, st>>>(s->d, s->cur, dt, s->prm.damping);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_substep_adjoint(void* handle, float dt, const xpbd_tape* tape, const xpbd_adjoint* adj, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !tape || !adj || !adj->gx || !adj->gv || !adj->g_inv_mu || !adj->g_inv_lambda || !adj->work0 ||
      !adj->work1 || !adj->ybar || !adj->dxbar || !adj->lambar || !adj->cnt)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle, tape or adjoint buffer");
  int r = check_diff(s);
  if (r != XPBD_OK) return r;
  cudaStream_t st = S(stream);
  const int K = s->prm.constraints_iter, V = s->d.V, T = s->d.T;
  Tape tp{reinterpret_cast<float4*>(tape->xs), reinterpret_cast<float2*>(tape->lams),
          reinterpret_cast<float4*>(tape->xpre), reinterpret_cast<float4*>(tape->v1),
          reinterpret_cast<float4*>(tape->posts), tape->rho_in};
  // through omega: the tape holds the post-Jacobi positions and the adjoint a chain state
  const bool through_omega = tp.posts && tp.rho_in && adj->omega_state && s->prm.cheb_enable;
  Dev dv = s->d;  // the history rows of the substep: the tape's copy, else the solver's rows 0..K-1
  if (tape->hist) dv.hist = tape->hist;
  Adj a;
  a.om = through_omega ? adj->omega_state : nullptr;
  a.om_n = om_stride(K);
  a.rtet = nullptr;  // the single-body residual adjoint adds its tet parts in place
  a.gx = reinterpret_cast<float4*>(adj->gx);
  a.gv = reinterpret_cast<float4*>(adj->gv);
  a.g_mu = adj->g_inv_mu;
  a.g_la = adj->g_inv_lambda;
  a.abuf[0] = reinterpret_cast<float4*>(adj->work0);
  a.abuf[1] = reinterpret_cast<float4*>(adj->work1);
  a.ybar = reinterpret_cast<float4*>(adj->ybar);
  a.dxbar = reinterpret_cast<float4*>(adj->dxbar);
  a.lambar = reinterpret_cast<float2*>(adj->lambar);
  a.cnt = adj->cnt;
  XPBD_CUDA(cudaMemsetAsync(a.lambar, 0, sizeof(float2) * T, st));
  const float e_over_dt = expf(-dt * s->prm.damping) / dt;
  const ChainPrm cp{K, s->prm.cheb_warmup, s->prm.rho_min, s->prm.rho_max, s->prm.rho_beta};
  if (a.om) ka_chain<Dev><<<1, 32, 0, st>>>(dv, tp, a, cp);
  ka_end<Dev><<<blocks_for(V), kBlock, 0, st>>>(dv, a, e_over_dt);
  float cD, cH;
  compliance_factors(s, dt, cD, cH);
  int src = 0;
  for (int k = K - 1; k >= 0; --k) {
    if (s->prm.cheb_enable)
      ka_cheb<Dev, true><<<blocks_for(V), kBlock, 0, st>>>(dv, tp, a, k, s->prm.cheb_gamma, src);
    else ka_cheb<Dev, false><<<blocks_for(V), kBlock, 0, st>>>(dv, tp, a, k, s->prm.cheb_gamma, src);
    const int g = (T + 127) / 128;
    if (through_omega) {
      if (s->prm.precise_hydro) ka_residual_adj<Dev, true><<<g, 128, 0, st>>>(dv, tp, a, k, cD, cH, src ^ 1);
      else ka_residual_adj<Dev, false><<<g, 128, 0, st>>>(dv, tp, a, k, cD, cH, src ^ 1);
    }
    if (s->prm.precise_hydro) ka_project<Dev, true><<<g, 128, 0, st>>>(dv, tp, a, k, cD, cH, src ^ 1);
    else ka_project<Dev, false><<<g, 128, 0, st>>>(dv, tp, a, k, cD, cH, src ^ 1);
    src ^= 1;
  }
  ka_begin<Dev><<<blocks_for(V), kBlock, 0, st>>>(dv, tp, a, src, dt);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

// Per-device address of g_noalloc_scratch, looked up once per device (with
// that device current) on the first call made on it.  The address belongs to
// the runtime's primary context of that device: the cache is not refreshed
// after cudaDeviceReset, and contexts created through the driver API are not
// supported.
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[256] = {nullptr};

int xpbd_residual_noalloc(const xpbd_body* body, const float* pred_x, float dt, float lame_mu, float lame_lambda,
                          int32_t precise_hydro, double* out, void* stream) {
  if (!body || !pred_x || !out) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL body, pred_x or out");
  if (body->n_tets <= 0 || body->n_verts <= 0) return fail(XPBD_ERR_BAD_MESH, "empty mesh");
  if ((long long)body->n_tets > kNoAllocMaxTets)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "xpbd_residual_noalloc handles at most " +
                                               std::to_string(kNoAllocMaxTets) + " tets per call, got " +
                                               std::to_string(body->n_tets));
  if (!body->tets || !body->dm_a || !body->dm_b || !body->dm_c || !body->v0 || !body->lam || !body->dx)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL body buffer");
  if ((body->tet_inv_mu == nullptr) != (body->tet_inv_lambda == nullptr))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "per-tet materials need both tet_inv_mu and tet_inv_lambda");
  const bool tet_mat = body->tet_inv_mu != nullptr;
  if (!(dt > 0.f) || (!tet_mat && (!(lame_mu != 0.f) || !(lame_lambda != 0.f))))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "need dt > 0 and non-zero Lame parameters");
  int dev = 0;
  XPBD_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return fail(XPBD_ERR_INVALID_ARGUMENT, "device ordinal out of range");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess)
        return fail(XPBD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_noalloc_ptr[dev] = static_cast<double*>(ptr);
    }
    scratch = g_noalloc_ptr[dev];
  }
  Dev d{};
  d.V = body->n_verts;
  d.T = body->n_tets;
  d.p[0] = const_cast<float4*>(reinterpret_cast<const float4*>(pred_x));
  d.dx = reinterpret_cast<float4*>(body->dx);
  d.tets = reinterpret_cast<const int4*>(body->tets);
  d.dm_a = reinterpret_cast<const float4*>(body->dm_a);
  d.dm_b = reinterpret_cast<const float4*>(body->dm_b);
  d.dm_c = body->dm_c;
  d.v0 = body->v0;
  d.lam = reinterpret_cast<float2*>(body->lam);
  d.tinv_mu = body->tet_inv_mu;
  d.tinv_la = body->tet_inv_lambda;
  // the allocating sweeps' compliance factors (compliance_factors): with
  // per-tet materials 1 / dt^2, scaled per tet by its 1 / mu and 1 / lambda
  const double dt2 = (double)dt * (double)dt;
  const float cD = tet_mat ? (float)(1.0 / dt2) : (float)(1.0 / ((double)lame_mu * dt2));
  const float cH = tet_mat ? (float)(1.0 / dt2) : (float)(1.0 / ((double)lame_lambda * dt2));
  cudaStream_t st = S(stream);
  // the ticket must start at zero; a clear, not an allocation
  XPBD_CUDA(cudaMemsetAsync(scratch + kNoAllocTicket, 0, sizeof(unsigned long long), st));
  const int grid = blocks_for(d.T);
  if (precise_hydro) k_residual_noalloc<true><<<grid, kBlock, 0, st>>>(d, cD, cH, scratch, out);
  else k_residual_noalloc<false><<<grid, kBlock, 0, st>>>(d, cD, cH, scratch, out);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

}  // extern "C"


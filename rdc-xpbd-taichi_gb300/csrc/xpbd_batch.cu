// Batched RDC-XPBD substep: many independent bodies of uneven size stepped by
// one launch per phase.
//
// Layout: every body's tets are padded to a multiple of 256 and its vertices
// to a multiple of 256, then all bodies are concatenated.  A 256-tet patch
// (the tile unit of the single-body kernels) therefore belongs to exactly one
// body (patch_body), and so does every 256-vertex block (vblock_body).  Each
// body carries its own Lame parameters, FP64 Chebyshev state (rho_hat,
// prev_r_hat, omega) and residual accumulators; the residual sweep's per-body
// ticket lets the last patch CTA of a body apply that body's rho_hat / omega
// recurrence (neohookean_solver.py:495-504, :537-546), so bodies never wait
// for each other and no grid-wide barrier is needed.
#include <cstdlib>
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "xpbd_device.cuh"

namespace xpbd {
namespace batch {

constexpr int kP = 256;

struct BodyState {
  double acc[3];
  unsigned int ticket;
  int has_prev;
  double rho_hat;
  double prev_r_hat;
  double omega;
  double r0;    // r_hat of the substep's first iteration (stop mode)
  int stop_at;  // iterations the body runs this substep (stop mode lowers it)
  int pad;
};

struct Flags {
  int nonfinite;
  int bad_mesh;
};

// Iteration control: it[k & 1] = k while iteration k runs (written by the
// previous iteration's update); n_active = bodies still iterating (stop mode).
// Stop mode: iteration k's tet sweeps cover the patches listed in
// act_patch[k & 1][0 .. n_act_patches[k & 1]), the patches of the bodies
// still iterating in body order, and its update covers the vertex blocks in
// act_vblock[k & 1].  kb_begin lists everything for iteration 0; kb_list,
// which runs beside the update of iteration k, lists iteration k + 1's into
// the other parity, so the sweeps are spread over the work that remains.
struct Ctl {
  int it[2];
  int n_active;
  int pad;
  int n_act_patches[2];
  int n_act_vblocks[2];
};

// Substeps of one frame whose per-body iteration counts are kept.
constexpr int kMaxCountedSubsteps = 256;

struct BDev {
  int V, T, n_patches, n_bodies, n_sdf, n_pverts;
  float4* x;
  float4* v;
  float4* p[2];
  float4* dx;
  const float4* dm_a;
  const float4* dm_b;
  const float* dm_c;
  float2* lam;
  const uint32_t* lid;
  const int* voff;
  const int* pverts;
  const int* patch_body;
  const int* patch_ntets;
  const int* vblock_body;
  const float* inv_mu;
  const float* inv_la;
  const float* tinv_mu;  // per-tet 1 / mu (nullptr: the body's)
  const float* tinv_la;  // per-tet 1 / lambda
  int paired;            // tets laid out by xpbd_pair_tets
  const int* body_patches;
  const int* body_tets;
  const int* perm;
  const xpbd_sdf* sdfs;
  BodyState* bs;
  Flags* flags;
  double* hist;  // [n_bodies][max_records][4]
  int max_records;
  Ctl* ctl;
  int* act_patch[2];      // [n_patches] patches of the iteration's sweeps, by parity (Ctl)
  int* act_vblock[2];     // [V / 256] vertex blocks of the iteration's update, by parity
  int* act_off;           // [n_bodies][2] a listed body's first patch / vertex-block position (-1: not listed)
  const int* body_first;  // [n_bodies] first patch of every body
  const int* body_vfirst; // [n_bodies] first 256-vertex block of every body
  const int* body_vblocks; // [n_bodies] vertex blocks of every body
  int* iters;    // [n_bodies][kMaxCountedSubsteps] iterations run per substep
  // stop mode: parity of the launched iteration (its index & 1), whose index
  // the kernels read from ctl->it[stop_par]; -1 = fixed iteration count
  int stop_par;
  float2* lam_tape;  // taping: the projection also stores the multipliers entering it here (nullptr: none)
};

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

__device__ __forceinline__ float3 post_position(const float4 p, const float4 D) {
  float3 r = make_float3(p.x, p.y, p.z);
  if (D.w > 0.f) {
    r.x += D.x / D.w;
    r.y += D.y / D.w;
    r.z += D.z / D.w;
  }
  return r;
}

// Stop mode, beside the update of iteration k (parity par): the patches and
// vertex blocks of the bodies that run iteration k + 1 (their stop_at lies
// beyond it), into the lists of parity par ^ 1; one CTA.  A block scan over
// the bodies in order gives each listed body its first positions; then every
// warp writes the patch and vertex-block ids of some of the bodies.
__global__ void __launch_bounds__(1024) kb_list(BDev d, int par) {
  __shared__ int s_wp[32], s_wv[32];
  __shared__ int s_bp, s_bv;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int next = *reinterpret_cast<const volatile int*>(&d.ctl->it[par]) + 1;
  const int q = par ^ 1;
  if (tid == 0) s_bp = s_bv = 0;
  __syncthreads();
  for (int b0 = 0; b0 < d.n_bodies; b0 += blockDim.x) {
    const int b = b0 + tid;
    const bool act = b < d.n_bodies && next < d.bs[b].stop_at;
    const int np = act ? __ldg(d.body_patches + b) : 0, nv = act ? __ldg(d.body_vblocks + b) : 0;
    int cp = np, cv = nv;  // inclusive warp scans
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int tp = __shfl_up_sync(0xffffffffu, cp, o), tv = __shfl_up_sync(0xffffffffu, cv, o);
      if (lane >= o) {
        cp += tp;
        cv += tv;
      }
    }
    if (lane == 31) {
      s_wp[warp] = cp;
      s_wv[warp] = cv;
    }
    __syncthreads();
    int op = s_bp, ov = s_bv;
    for (int w = 0; w < warp; ++w) {
      op += s_wp[w];
      ov += s_wv[w];
    }
    if (b < d.n_bodies) {
      d.act_off[2 * b] = act ? op + cp - np : -1;
      d.act_off[2 * b + 1] = ov + cv - nv;
    }
    __syncthreads();
    if (tid == 0)
      for (int w = 0; w < nw; ++w) {
        s_bp += s_wp[w];
        s_bv += s_wv[w];
      }
    __syncthreads();
  }
  if (tid == 0) {
    d.ctl->n_act_patches[q] = s_bp;
    d.ctl->n_act_vblocks[q] = s_bv;
  }
  for (int b = warp; b < d.n_bodies; b += nw) {
    const int op = d.act_off[2 * b];
    if (op < 0) continue;
    const int ov = d.act_off[2 * b + 1];
    const int fp = __ldg(d.body_first + b), np = __ldg(d.body_patches + b);
    const int fv = __ldg(d.body_vfirst + b), nv = __ldg(d.body_vblocks + b);
    for (int i = lane; i < np; i += 32) d.act_patch[q][op + i] = fp + i;
    for (int i = lane; i < nv; i += 32) d.act_vblock[q][ov + i] = fv + i;
  }
}

// Begin of a substep for every body: per-body reset of prev_r_hat / omega
// (neohookean_solver.py:461, :466) and predict + sequential SDF projection.
__global__ void __launch_bounds__(256) kb_begin(BDev d, float dt, float gx, float gy, float gz, int K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0) {
    for (int b = threadIdx.x; b < d.n_bodies; b += blockDim.x) {
      d.bs[b].has_prev = 0;
      d.bs[b].omega = 1.0;
      d.bs[b].r0 = 0.0;
      d.bs[b].stop_at = K;
    }
    if (threadIdx.x == 0) {
      d.ctl->it[0] = 0;
      d.ctl->n_active = d.n_bodies;
      d.ctl->n_act_patches[0] = d.n_patches;
      d.ctl->n_act_vblocks[0] = d.V >> 8;
    }
  }
  if (d.stop_par >= 0) {  // stop mode: iteration 0 lists every patch and vertex block
    for (int q = i; q < d.n_patches; q += gridDim.x * blockDim.x) d.act_patch[0][q] = q;
    if (i < (d.V >> 8)) d.act_vblock[0][i] = i;
  }
  if (i >= d.V) return;
  const float4 xi = d.x[i];
  float4 vi = d.v[i];
  const float w = xi.w;
  if (w > 0.f) {
    vi.x += gx * dt;
    vi.y += gy * dt;
    vi.z += gz * dt;
    d.v[i] = vi;
  }
  float3 p = make_float3(xi.x + vi.x * dt, xi.y + vi.y * dt, xi.z + vi.z * dt);
  if (w > 0.f) sdf_project_all(d.sdfs, d.n_sdf, p, make_float3(vi.x, vi.y, vi.z));
  d.p[0][i] = make_float4(p.x, p.y, p.z, w);
}

// advance (xpbd_base.py:148-160).  dyn (stop mode): body b ran stop_at
// iterations, so its positions are in p[stop_at & 1] with Chebyshev (p[0]
// without); `sub` >= 0 records every body's count for that substep.
__global__ void __launch_bounds__(256) kb_end(BDev d, int cur, float dt, float damping, int dyn, int cheb, int sub) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (blockIdx.x == 0 && sub >= 0 && sub < kMaxCountedSubsteps)
    for (int b = threadIdx.x; b < d.n_bodies; b += blockDim.x)
      d.iters[(size_t)b * kMaxCountedSubsteps + sub] = d.bs[b].stop_at;
  if (i >= d.V) return;
  if (dyn) cur = cheb ? (d.bs[__ldg(d.vblock_body + (i >> 8))].stop_at & 1) : 0;
  const float4 xi = d.x[i];
  if (xi.w <= 0.f) {
    d.p[cur][i] = xi;
    return;
  }
  const float4 pi = d.p[cur][i];
  const float e = expf(-dt * damping);
  const float4 vi = d.v[i];
  d.v[i] = make_float4((pi.x - xi.x) / dt * e, (pi.y - xi.y) / dt * e, (pi.z - xi.z) / dt * e, vi.w);
  d.x[i] = make_float4(pi.x, pi.y, pi.z, xi.w);
}

// Projection, one CTA of kP / kTPT threads per patch (the single-body tile
// kernel with per-body compliance 1 / (mu_b dt^2), 1 / (lambda_b dt^2), or
// with kTetMat per-tet 1 / (mu_t dt^2), 1 / (lambda_t dt^2)); each thread
// projects kTPT consecutive tets (project_chain).
template <bool kBlockMode, bool kFirst, bool kPrecise, int kTPT, bool kTetMat>
__global__ void __launch_bounds__(kP / kTPT, project_min_blocks(kTPT)) kb_project(BDev d, int cur, float inv_dt2, float relax_h, float relax_d) {
  constexpr int kThreads = kP / kTPT;
  __shared__ float4 sp[256];
  __shared__ int sg[256];
  int p = blockIdx.x;
  if (d.stop_par >= 0) {  // stop mode: CTA q takes listed patch q
    if (p >= __ldg(&d.ctl->n_act_patches[d.stop_par])) return;
    p = __ldg(d.act_patch[d.stop_par] + p);
  }
  const int b = __ldg(d.patch_body + p);
  const int vb = __ldg(d.voff + p);
  const int nv = __ldg(d.voff + p + 1) - vb;
  const int nt = __ldg(d.patch_ntets + p);
  const int l0 = kTPT * threadIdx.x;
  const int t0 = p * kP + l0;
  float4 A[kTPT], B[kTPT];
  float C[kTPT];
  uint32_t lid[kTPT];
  float2 L[kTPT];
  float mD[kTPT], mH[kTPT];
  if (kTPT == 2) {  // one load per record array (the patch's slots are padded to kP)
    ldg_pair(d.dm_a + t0, A[0], A[1]);
    ldg_pair(d.dm_b + t0, B[0], B[1]);
    const float2 c = __ldg(reinterpret_cast<const float2*>(d.dm_c + t0));
    const uint2 li = __ldg(reinterpret_cast<const uint2*>(d.lid + t0));
    C[0] = c.x;
    C[1] = c.y;
    lid[0] = li.x;
    lid[1] = li.y;
    L[0] = L[1] = make_float2(0.f, 0.f);
    if (!kFirst) {
      const float4 l2 = *reinterpret_cast<const float4*>(d.lam + t0);
      L[0] = make_float2(l2.x, l2.y);
      L[1] = make_float2(l2.z, l2.w);
    }
    mD[0] = mD[1] = mH[0] = mH[1] = 0.f;
    if (kTetMat) {
      const float2 u = __ldg(reinterpret_cast<const float2*>(d.tinv_mu + t0));
      const float2 v = __ldg(reinterpret_cast<const float2*>(d.tinv_la + t0));
      mD[0] = u.x;
      mD[1] = u.y;
      mH[0] = v.x;
      mH[1] = v.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kTPT; ++k) {
      A[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      B[k] = A[k];
      C[k] = 0.f;
      lid[k] = 0u;
      L[k] = make_float2(0.f, 0.f);
      mD[k] = mH[k] = 0.f;
      if (l0 + k < nt) {
        A[k] = __ldg(d.dm_a + t0 + k);
        B[k] = __ldg(d.dm_b + t0 + k);
        C[k] = __ldg(d.dm_c + t0 + k);
        lid[k] = __ldg(d.lid + t0 + k);
        if (!kFirst) L[k] = d.lam[t0 + k];
        if (kTetMat) {
          mD[k] = __ldg(d.tinv_mu + t0 + k);
          mH[k] = __ldg(d.tinv_la + t0 + k);
        }
      }
    }
  }
  const float4* P = d.p[cur];
  for (int j = threadIdx.x; j < nv; j += kThreads) {
    const int g = __ldg(d.pverts + vb + j);
    sg[j] = g;
    sp[j] = ldg4(P + g);
  }
  __syncthreads();
  const int n = nt - l0 < kTPT ? nt - l0 : kTPT;
  if (n <= 0) return;
  if (kTetMat) {
    project_chain<kBlockMode, kPrecise, kTPT, true>(A, B, C, lid, L, d.lam + t0, n, sp, sg, d.dx, inv_dt2, inv_dt2,
                                                    relax_h, relax_d, d.paired != 0, mD, mH,
                                                    d.lam_tape ? d.lam_tape + t0 : nullptr);
  } else {
    const float cD = __ldg(d.inv_mu + b) * inv_dt2, cH = __ldg(d.inv_la + b) * inv_dt2;
    project_chain<kBlockMode, kPrecise, kTPT>(A, B, C, lid, L, d.lam + t0, n, sp, sg, d.dx, cD, cH, relax_h,
                                              relax_d, d.paired != 0, nullptr, nullptr,
                                              d.lam_tape ? d.lam_tape + t0 : nullptr);
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

struct BSweep {
  int cur;
  float inv_dt2;
  int par;       // the iteration's index & 1 (its index is ctl->it[par])
  int warmup;
  int rec_base;  // history row of the substep's iteration 0 (-1: none)
  int res;       // Chebyshev recurrence
  int stop;      // stop mode
  double rho_min, rho_max, rho_beta;
  double target, floor;
};

// Add a CTA's partial sums over `npatch` patches of body b to the body's FP64
// accumulators; the CTA that completes the body's patch count applies the
// rho_hat / omega recurrence (neohookean_solver.py:495-504, :537-546) and
// writes the body's history row.  All threads of the CTA call it.
template <bool kRes, bool kMon, int kWarps>
__device__ __forceinline__ void flush_body(const BDev& d, const BSweep& a, int it, int b, int npatch, float sr,
                                           float sh, float sd, double (*red)[kWarps]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double r0 = warp_sum((double)sr), r1 = warp_sum((double)sh), r2 = warp_sum((double)sd);
  __syncthreads();  // red[] of the previous flush has been consumed
  if (lane == 0) {
    red[0][warp] = r0;
    red[1][warp] = r1;
    red[2][warp] = r2;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double b0 = 0.0, b1 = 0.0, b2 = 0.0;
  for (int k = 0; k < kWarps; ++k) {
    b0 += red[0][k];
    b1 += red[1][k];
    b2 += red[2][k];
  }
  BodyState* bs = d.bs + b;
  if (kRes) atomicAdd(&bs->acc[0], b0);
  if (kMon) {
    atomicAdd(&bs->acc[1], b1);
    atomicAdd(&bs->acc[2], b2);
  }
  __threadfence();
  const unsigned int tk = atomicAdd(&bs->ticket, (unsigned)npatch);
  if (tk + (unsigned)npatch != (unsigned)__ldg(d.body_patches + b)) return;
  __threadfence();
  volatile BodyState* st = bs;
  const double S = st->acc[0], Hs = st->acc[1], Ds = st->acc[2];
  st->acc[0] = 0.0;
  st->acc[1] = 0.0;
  st->acc[2] = 0.0;
  st->ticket = 0u;
  const int ntb = __ldg(d.body_tets + b);
  const double n = (double)ntb;
  double r_hat = 0.0, omega = 1.0;
  if (kRes) {
    r_hat = ntb > 0 ? S / n : 0.0;
    if (!isfinite(S)) d.flags->nonfinite = 1;
  }
  if (kRes && a.res) {
    if (st->has_prev && st->prev_r_hat > 1e-12) {
      double rho_inst = r_hat / (st->prev_r_hat + 1e-12);
      rho_inst = fmax(a.rho_min, fmin(a.rho_max, rho_inst));
      st->rho_hat = (1.0 - a.rho_beta) * st->rho_hat + a.rho_beta * rho_inst;
    }
    st->prev_r_hat = r_hat;
    st->has_prev = 1;
    const double rho2 = st->rho_hat * st->rho_hat;
    if (it < a.warmup) omega = 1.0;
    else if (it == a.warmup) omega = 2.0 / (2.0 - rho2);
    else omega = 4.0 / (4.0 - rho2 * st->omega);
    st->omega = omega;
  }
  // stop mode: the body's last iteration is this one once r_hat meets the
  // target (or the floor); it still finishes (update) in this iteration
  if (kRes && a.stop) {
    if (it == 0) st->r0 = r_hat;
    if ((r_hat <= a.target * st->r0 || r_hat <= a.floor) && it + 1 < st->stop_at) {
      st->stop_at = it + 1;
      atomicSub(&d.ctl->n_active, 1);
    }
  }
  if (a.rec_base >= 0) {
    double* h = d.hist + 4 * ((size_t)b * d.max_records + a.rec_base + it);
    h[0] = r_hat;
    h[1] = omega;
    h[2] = kMon && ntb > 0 ? Hs / n : 0.0;
    h[3] = kMon && ntb > 0 ? Ds / n : 0.0;
  }
}

// Residual (neohookean_solver.py:298-329) and monitoring sums (:256-296).
// Each CTA walks a contiguous run of `chunk` patches (patches are ordered by
// body) and flushes its partial sums whenever the body changes.  In stop mode
// the run is taken from the sweep's body list (Ctl), split evenly over the
// grid, so the CTAs share the patches of the bodies still iterating.
// Two tets per thread are compiled for 9 resident CTAs per SM (56 registers;
// the per-tet-material forms spill a few bytes): on 256 uneven bodies the
// sweep takes 3.7% less time than at the 8 CTAs its 64 registers allowed.
template <bool kRes, bool kMon, bool kPrecise, int kTPT, bool kTetMat>
__global__ void __launch_bounds__(kP / kTPT, kTPT == 2 ? 9 : 1) kb_residual(BDev d, BSweep a, int chunk) {
  constexpr int kThreads = kP / kTPT;
  __shared__ float4 sp[256];
  __shared__ double red[3][kThreads / 32];
  int n_items = d.n_patches;
  if (a.stop) {
    n_items = __ldg(&d.ctl->n_act_patches[a.par]);
    chunk = (n_items + gridDim.x - 1) / gridDim.x;
  }
  const int c0 = blockIdx.x * chunk;
  const int c1 = c0 + chunk < n_items ? c0 + chunk : n_items;
  const float4* P = d.p[a.cur];
  const int l0 = kTPT * threadIdx.x;
  const int it = *reinterpret_cast<const volatile int*>(&d.ctl->it[a.par]);
  float sr = 0.f, sh = 0.f, sd = 0.f;
  int run = 0;
  // stop mode: sweep position q is listed patch act_patch[q]
  const int* list = d.act_patch[a.par];
  int p = a.stop && c0 < c1 ? __ldg(list + c0) : c0;
  for (int q = c0; q < c1; ++q) {
    const int pn = q + 1 < c1 ? (a.stop ? __ldg(list + q + 1) : q + 1) : -1;
    const int b = __ldg(d.patch_body + p);
    const int vb = __ldg(d.voff + p);
    const int nv = __ldg(d.voff + p + 1) - vb;
    const int nt = __ldg(d.patch_ntets + p);
    const int t0 = p * kP + l0;
    float4 A[kTPT], B[kTPT];
    float C[kTPT];
    uint32_t lid[kTPT];
    float2 L[kTPT];
    float mD[kTPT], mH[kTPT];
    if (kTPT == 2) {  // one load per record array (the patch's slots are padded to kP)
      ldg_pair(d.dm_a + t0, A[0], A[1]);
      ldg_pair(d.dm_b + t0, B[0], B[1]);
      const float2 c = __ldg(reinterpret_cast<const float2*>(d.dm_c + t0));
      const uint2 li = __ldg(reinterpret_cast<const uint2*>(d.lid + t0));
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
      if (kTetMat && kRes) {
        const float2 u = __ldg(reinterpret_cast<const float2*>(d.tinv_mu + t0));
        const float2 v = __ldg(reinterpret_cast<const float2*>(d.tinv_la + t0));
        mD[0] = u.x;
        mD[1] = u.y;
        mH[0] = v.x;
        mH[1] = v.y;
      }
    } else {
#pragma unroll
      for (int k = 0; k < kTPT; ++k) {
        if (l0 + k < nt) {
          A[k] = __ldg(d.dm_a + t0 + k);
          B[k] = __ldg(d.dm_b + t0 + k);
          C[k] = __ldg(d.dm_c + t0 + k);
          lid[k] = __ldg(d.lid + t0 + k);
          L[k] = kRes ? d.lam[t0 + k] : make_float2(0.f, 0.f);
          if (kTetMat && kRes) {
            mD[k] = __ldg(d.tinv_mu + t0 + k);
            mH[k] = __ldg(d.tinv_la + t0 + k);
          }
        }
      }
    }
    __syncthreads();  // the previous patch's readers are done with sp
    for (int j = threadIdx.x; j < nv; j += kThreads) {
      const int g = __ldg(d.pverts + vb + j);
      const float3 x = post_position(ldg4(P + g), ldg4(d.dx + g));
      sp[j] = make_float4(x.x, x.y, x.z, 0.f);
    }
    __syncthreads();
    const float aDs = kRes && !kTetMat ? __ldg(d.inv_mu + b) * a.inv_dt2 : 0.f;
    const float aHs = kRes && !kTetMat ? __ldg(d.inv_la + b) * a.inv_dt2 : 0.f;
#pragma unroll
    for (int k = 0; k < kTPT; ++k) {
      if (l0 + k >= nt) break;
      Tet tt;
      tt.dm[0] = A[k].x; tt.dm[1] = A[k].y; tt.dm[2] = A[k].z;
      tt.dm[3] = A[k].w; tt.dm[4] = B[k].x; tt.dm[5] = B[k].y;
      tt.dm[6] = B[k].z; tt.dm[7] = B[k].w; tt.dm[8] = C[k];
      tt.p[0] = sp[lid[k] & 0xffu];
      tt.p[1] = sp[(lid[k] >> 8) & 0xffu];
      tt.p[2] = sp[(lid[k] >> 16) & 0xffu];
      tt.p[3] = sp[lid[k] >> 24];
      float F[9];
      deformation_gradient(tt, F);
      float C_D, C_H;
      invariants<kPrecise>(F, C_D, C_H);
      if (kRes) {
        const float six_det = 6.f * det9(tt.dm);
        const float cDk = kTetMat ? a.inv_dt2 * mD[k] : aDs, cHk = kTetMat ? a.inv_dt2 * mH[k] : aHs;
        const float rD = C_D + six_det * cDk * L[k].x, rH = C_H + six_det * cHk * L[k].y;
        sr += sqrtf(rD * rD + rH * rH);
      }
      if (kMon) {
        sh += fabsf(C_H);
        sd += fabsf(C_D);
      }
    }
    ++run;
    if (pn < 0 || __ldg(d.patch_body + pn) != b) {
      flush_body<kRes, kMon, kThreads / 32>(d, a, it, b, run, sr, sh, sd, red);
      sr = sh = sd = 0.f;
      run = 0;
    }
    p = pn;
  }
}

// post_solve + Chebyshev mix with the omega of the vertex block's body.
// Each thread takes kBUpdateBlocks vertices, one in each of consecutive
// 256-vertex blocks, so that all of its loads are in flight together.
constexpr int kBUpdateBlocks = 2;

// Iteration control of one update launch: CTA 0 advances the iteration
// index and (stop mode, under a frame graph) sets the loop condition.
struct BUpd {
  int par;       // the iteration's index & 1
  int K;         // iterations per substep (stop mode: the cap)
  int stop;
  int use_cond;
  cudaGraphConditionalHandle cond;
  float4* post_out;  // taping through omega: the post-Jacobi positions (nullptr: none)
  float4* xs_out;    // taping: the positions entering the next iteration (nullptr: none)
};

template <bool kCheb, bool kFirstIt>
__global__ void __launch_bounds__(256) kb_update(BDev d, int cur, float gamma, BUpd u) {
  const int vb0 = blockIdx.x * kBUpdateBlocks;
  if (blockIdx.x == 0) {
    const int it = *reinterpret_cast<const volatile int*>(&d.ctl->it[u.par]);
    if (threadIdx.x == 0) {
      d.ctl->it[u.par ^ 1] = it + 1;
      if (u.use_cond) {
        const bool more = it + 1 < u.K && *reinterpret_cast<const volatile int*>(&d.ctl->n_active) > 0;
        cudaGraphSetConditional(u.cond, more ? 1u : 0u);
      }
    }
  }
  // every load is issued before the first store: as far as the compiler
  // knows the buffers may alias, so a load after a store would wait for it
  float4 pc[kBUpdateBlocks], D[kBUpdateBlocks], yp[kBUpdateBlocks];
  float om[kBUpdateBlocks];
  int vi[kBUpdateBlocks];  // the thread's vertex in each of its blocks, -1: none
  // stop mode: the CTA's blocks are entries of the iteration's vertex-block list
  const int nlist = u.stop ? __ldg(&d.ctl->n_act_vblocks[u.par]) : 0;
#pragma unroll
  for (int k = 0; k < kBUpdateBlocks; ++k) {
    int vb = vb0 + k;
    if (u.stop) vb = vb < nlist ? __ldg(d.act_vblock[u.par] + vb) : -1;
    const int i = vb * 256 + threadIdx.x;
    vi[k] = vb >= 0 && i < d.V ? i : -1;
    om[k] = 1.f;
    if (vi[k] >= 0) {
      pc[k] = d.p[cur][i];
      D[k] = d.dx[i];
      yp[k] = pc[k];
      if (kCheb) {
        if (!kFirstIt) yp[k] = d.p[cur ^ 1][i];
        om[k] = (float)d.bs[__ldg(d.vblock_body + vb)].omega;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < kBUpdateBlocks; ++k) {
    const int i = vi[k];
    if (i < 0) continue;
    d.dx[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 xp = post_position(pc[k], D[k]);
    if (u.post_out) u.post_out[i] = make_float4(xp.x, xp.y, xp.z, pc[k].w);
    float4 xo;
    if (kCheb) {
      const float nx = gamma * (xp.x - pc[k].x) + pc[k].x;
      const float ny = gamma * (xp.y - pc[k].y) + pc[k].y;
      const float nz = gamma * (xp.z - pc[k].z) + pc[k].z;
      xo = make_float4(yp[k].x + om[k] * (nx - yp[k].x), yp[k].y + om[k] * (ny - yp[k].y),
                       yp[k].z + om[k] * (nz - yp[k].z), pc[k].w);
      d.p[cur ^ 1][i] = xo;
    } else {
      xo = make_float4(xp.x, xp.y, xp.z, pc[k].w);
      d.p[cur][i] = xo;
    }
    if (u.xs_out) u.xs_out[i] = xo;
  }
}

__global__ void kb_export(BDev d, const float4* f, float* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
  const int j = d.perm[i];
  if (j < 0) return;  // padding vertex
  const float4 o = f[i];
  dst[3 * (size_t)j] = o.x;
  dst[3 * (size_t)j + 1] = o.y;
  dst[3 * (size_t)j + 2] = o.z;
}

__global__ void kb_import(BDev d, float4* f, const float* __restrict__ src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
  const int j = d.perm[i];
  if (j < 0) return;
  float4 o = f[i];
  o.x = src[3 * (size_t)j];
  o.y = src[3 * (size_t)j + 1];
  o.z = src[3 * (size_t)j + 2];
  f[i] = o;
}

// One-time validation of every index the kernels follow.
__global__ void kb_validate(BDev d, int n_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < d.n_patches) {
    const int a = d.voff[t], e = d.voff[t + 1], b = d.patch_body[t], nt = d.patch_ntets[t];
    if (a < 0 || e < a || e > d.n_pverts || e - a > 256 || b < 0 || b >= d.n_bodies || nt < 0 || nt > kP)
      d.flags->bad_mesh = 1;
    // a body's patches are consecutive, from body_first[b] on
    else if (t < d.body_first[b] || t >= d.body_first[b] + d.body_patches[b])
      d.flags->bad_mesh = 1;
    for (int q = 0; q < nt && !d.flags->bad_mesh; ++q) {
      const uint32_t l = d.lid[t * kP + q];
      if ((int)(l & 0xffu) >= e - a || (int)((l >> 8) & 0xffu) >= e - a || (int)((l >> 16) & 0xffu) >= e - a ||
          (int)(l >> 24) >= e - a)
        d.flags->bad_mesh = 1;
    }
    for (int k = a; k < e && !d.flags->bad_mesh; ++k)
      if ((unsigned)d.pverts[k] >= (unsigned)d.V) d.flags->bad_mesh = 1;
  }
  if (t < d.V / 256) {
    const int b = d.vblock_body[t];
    if (b < 0 || b >= d.n_bodies) d.flags->bad_mesh = 1;
  }
  if (d.perm && t < d.V) {
    if (d.perm[t] >= n_out || d.perm[t] < -1) d.flags->bad_mesh = 1;
  }
}

// Per-body rho_hat to / from a device array (adjoint checkpoints).
__global__ void kb_rho_copy(BDev d, double* dst, const double* src) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= d.n_bodies) return;
  if (dst) dst[b] = d.bs[b].rho_hat;
  if (src) d.bs[b].rho_hat = src[b];
}

// Accessors of the batched layout for the vertex adjoint kernels
// (xpbd_adjoint.cuh); the tet adjoint is the tile kernel kba_project below.
__device__ __forceinline__ int adj_verts(const BDev& d) { return d.V; }
__device__ __forceinline__ int adj_tets(const BDev& d) { return d.T; }
__device__ __forceinline__ float adj_omega(const BDev& d, int i, int k) {
  const int b = __ldg(d.vblock_body + (i >> 8));
  return (float)d.hist[4 * ((size_t)b * d.max_records + k) + 1];
}
__device__ __forceinline__ int adj_nbodies(const BDev& d) { return d.n_bodies; }
__device__ __forceinline__ int adj_vbody(const BDev& d, int i) { return __ldg(d.vblock_body + (i >> 8)); }
__device__ __forceinline__ double adj_hist(const BDev& d, int b, int k, int c) {
  return d.hist[4 * ((size_t)b * d.max_records + k) + c];
}
__device__ __forceinline__ double adj_body_tets(const BDev& d, int b) { return (double)__ldg(d.body_tets + b); }
}  // namespace batch
}  // namespace xpbd

#include "xpbd_adjoint.cuh"

namespace xpbd {
namespace batch {

// Scatters a tet's four corner vectors g into acc (global vertex ids through
// the patch map sg) with red.global.add.v4.  Thread 2u holds tet 2u of the
// patch and thread 2u + 1 tet 2u + 1; when the two share a face in the
// xpbd_pair_tets layout (corners 0, 1, 2 of the odd tet are corners 1, 0, 2
// of the even one, recognised from the packed patch-local ids) the even
// thread adds the three shared corners and the odd one flushes only its
// corner 3: 5 reductions per pair instead of 8.  With acc2, each vector also
// goes there divided by its vertex's cnt.  Every thread of the warp calls it
// (padding threads with live = false).
__device__ __forceinline__ void scatter_corners(bool paired, bool live, uint32_t lid, float3 (&g)[4],
                                                const int* sg, float4* acc, float4* acc2 = nullptr,
                                                const float* cnt = nullptr) {
  bool merge = false;
  const bool odd = threadIdx.x & 1u;
  if (paired) {
    const unsigned full = 0xffffffffu;
    const uint32_t lid_p = __shfl_xor_sync(full, lid, 1);
    const bool live_p = __shfl_xor_sync(full, (int)live, 1) != 0;
    float3 h[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      h[q].x = __shfl_xor_sync(full, g[q].x, 1);
      h[q].y = __shfl_xor_sync(full, g[q].y, 1);
      h[q].z = __shfl_xor_sync(full, g[q].z, 1);
    }
    const uint32_t le = odd ? lid_p : lid, lo = odd ? lid : lid_p;
    merge = live && live_p && (lo & 0xffffffu) == (__byte_perm(le, 0u, 0x3201u) & 0xffffffu);
    if (merge && !odd) {
      g[0].x += h[1].x; g[0].y += h[1].y; g[0].z += h[1].z;
      g[1].x += h[0].x; g[1].y += h[0].y; g[1].z += h[0].z;
      g[2].x += h[2].x; g[2].y += h[2].y; g[2].z += h[2].z;
    }
  }
  if (!live) return;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (!(merge && odd) || q == 3) {
      const int v = sg[(lid >> (8 * q)) & 0xffu];
      red_add_v4(acc + v, g[q].x, g[q].y, g[q].z, 0.f);
      if (acc2) {
        const float cn = cnt[v];
        const float ic = cn > 0.f ? 1.f / cn : 0.f;
        red_add_v4(acc2 + v, g[q].x * ic, g[q].y * ic, g[q].z * ic, 0.f);
      }
    }
}

// Reverse of the batched block projection of iteration k, one CTA per 256-tet
// patch: the patch's positions entering the iteration (from the tape) and its
// vertices' accumulator adjoints are staged in shared memory once, then each
// thread reverses one tet (tet_adjoint) and scatters its corner adjoints into
// abuf[dst] (scatter_corners).  With the omega chain each tet adds the
// residual's multiplier and material parts (rtet).  c = 1 / dt^2; the tet's compliances are
// c / V0 times its (or its body's) 1 / mu and 1 / lambda.  Compiled for 3
// resident CTAs per SM (80 registers; the tet adjoint alone wants 96, which
// allows only 2 CTAs and leaves the staging latency exposed).
template <bool kPrecise>
__global__ void __launch_bounds__(kP, 3) kba_project(BDev d, Tape tp, Adj a, int k, float c, int dst) {
  __shared__ float4 sp[256];
  __shared__ float4 sb[256];
  __shared__ int sg[256];
  const int p = blockIdx.x;
  const int vb = __ldg(d.voff + p);
  const int nv = __ldg(d.voff + p + 1) - vb;
  const int nt = __ldg(d.patch_ntets + p);
  const bool live = (int)threadIdx.x < nt;
  const int t = p * kP + threadIdx.x;
  // the tet's own records first: their latency overlaps the tile staging
  uint32_t lid = 0u;
  float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;
  float C = 0.f, m_mu = 0.f, m_la = 0.f;
  float2 L = make_float2(0.f, 0.f), lb_next = L;
  if (live) {
    lid = __ldg(d.lid + t);
    A = __ldg(d.dm_a + t);
    B = __ldg(d.dm_b + t);
    C = __ldg(d.dm_c + t);
    if (d.tinv_mu) {
      m_mu = __ldg(d.tinv_mu + t);
      m_la = __ldg(d.tinv_la + t);
    } else {
      const int body = __ldg(d.patch_body + p);
      m_mu = __ldg(d.inv_mu + body);
      m_la = __ldg(d.inv_la + body);
    }
    L = tp.lams[(size_t)k * d.T + t];
    lb_next = a.lambar[t];  // written three kernels back
  }
  pdl_wait();  // the accumulator adjoints and rtet of the kernels before it
  pdl_trigger();
  if (a.rtet && live) {  // rtet[t] = (lambda_{k+1} adjoint, material adjoints)
    const float2 r = reinterpret_cast<const float2*>(a.rtet + t)[0];
    lb_next.x += r.x;
    lb_next.y += r.y;
  }
  const float4* X = tp.xs + (size_t)k * d.V;
  for (int j = threadIdx.x; j < nv; j += kP) {
    const int g = __ldg(d.pverts + vb + j);
    sg[j] = g;
    sp[j] = __ldg(X + g);
    sb[j] = a.dxbar[g];
  }
  __syncthreads();
  float3 gout[4] = {};
  if (live) {
    Tet tt;
    tt.dm[0] = A.x; tt.dm[1] = A.y; tt.dm[2] = A.z;
    tt.dm[3] = A.w; tt.dm[4] = B.x; tt.dm[5] = B.y;
    tt.dm[6] = B.z; tt.dm[7] = B.w; tt.dm[8] = C;
    int l[4];
    float3 dpb[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      l[q] = (int)((lid >> (8 * q)) & 0xffu);
      tt.p[q] = sp[l[q]];
      dpb[q] = f3(sb[l[q]]);
    }
    const float inv_v0 = 6.f * det9(tt.dm);
    const float s0 = c * inv_v0;  // d aD / d(1/mu) = d aH / d(1/lambda)
    const float aD = s0 * m_mu, aH = s0 * m_la;
    float2 lb;
    float aDb, aHb;
    tet_adjoint<kPrecise>(tt, L, aD, aH, lb_next, dpb, gout, lb, aDb, aHb);
    a.lambar[t] = lb;
    float2 rm = make_float2(0.f, 0.f);
    if (a.rtet) rm = reinterpret_cast<const float2*>(a.rtet + t)[1];
    a.g_mu[t] += (double)(aDb * s0 + rm.x);
    a.g_la[t] += (double)(aHb * s0 + rm.y);
  }
  scatter_corners(d.paired != 0, live, lid, gout, sg, adj_buf(a, dst));
}

// r_hat_k's adjoint into the tets of iteration k, one CTA per patch (the
// batched layout of ka_residual_adj): every CTA steps its body's omega chain
// (the body's first patch stores it), the patch's post-Jacobi positions are
// staged in shared memory, and each thread takes one tet.  The position part
// goes to abuf[dst] (x~_k's adjoint: post = x~_k + dx / cnt) and, divided by
// cnt, to the accumulator's adjoint dxbar (scatter_corners); the multiplier
// and material parts go to rtet (zero where r_hat_k's adjoint is), read by
// kba_project of iteration k.
template <bool kPrecise>
__global__ void __launch_bounds__(kP) kba_residual_adj(BDev d, Tape tp, Adj a, int k, float c, int dst) {
  pdl_wait();  // omega_k's adjoint summed by ka_cheb before it
  pdl_trigger();
  __shared__ float4 sp[256];
  __shared__ int sg[256];
  __shared__ float s_rb;
  const int p = blockIdx.x;
  const int body = __ldg(d.patch_body + p);
  if (threadIdx.x == 0)
    s_rb = (float)(chain_step(a, body, k, p == __ldg(d.body_first + body)) / adj_body_tets(d, body));
  const int vb = __ldg(d.voff + p);
  const int nv = __ldg(d.voff + p + 1) - vb;
  const int nt = __ldg(d.patch_ntets + p);
  const bool live = (int)threadIdx.x < nt;
  const int t = p * kP + threadIdx.x;
  __syncthreads();
  const float rb_n = s_rb;
  if (rb_n == 0.f) {
    if (live) a.rtet[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  uint32_t lid = 0u;
  float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A;
  float C = 0.f, m_mu = 0.f, m_la = 0.f;
  float2 L1 = make_float2(0.f, 0.f);
  if (live) {
    lid = __ldg(d.lid + t);
    A = __ldg(d.dm_a + t);
    B = __ldg(d.dm_b + t);
    C = __ldg(d.dm_c + t);
    if (d.tinv_mu) {
      m_mu = __ldg(d.tinv_mu + t);
      m_la = __ldg(d.tinv_la + t);
    } else {
      m_mu = __ldg(d.inv_mu + body);
      m_la = __ldg(d.inv_la + body);
    }
    L1 = tp.lams[(size_t)(k + 1) * d.T + t];
  }
  const float4* X = tp.posts + (size_t)k * d.V;
  for (int j = threadIdx.x; j < nv; j += kP) {
    const int g = __ldg(d.pverts + vb + j);
    sg[j] = g;
    sp[j] = __ldg(X + g);
  }
  __syncthreads();
  float3 g[4] = {};
  if (live) {
    Tet tt;
    tt.dm[0] = A.x; tt.dm[1] = A.y; tt.dm[2] = A.z;
    tt.dm[3] = A.w; tt.dm[4] = B.x; tt.dm[5] = B.y;
    tt.dm[6] = B.z; tt.dm[7] = B.w; tt.dm[8] = C;
#pragma unroll
    for (int q = 0; q < 4; ++q) tt.p[q] = sp[(lid >> (8 * q)) & 0xffu];
    const float s0 = c * 6.f * det9(tt.dm);  // d aD / d(1/mu) = d aH / d(1/lambda)
    float2 lb;
    float aDb, aHb;
    residual_adjoint<kPrecise>(tt, L1, s0 * m_mu, s0 * m_la, rb_n, g, lb, aDb, aHb);
    a.rtet[t] = make_float4(lb.x, lb.y, aDb * s0, aHb * s0);
  }
  scatter_corners(d.paired != 0, live, lid, g, sg, adj_buf(a, dst), a.dxbar, a.cnt);
}

}  // namespace batch
}  // namespace xpbd

using namespace xpbd;
using namespace xpbd::batch;

namespace {

thread_local std::string g_err;

int bfail(int st, const std::string& m) {
  g_err = m;
  return st;
}

// On failure the runtime's per-thread last error is cleared as well.
#define B_CUDA(call)                                                                \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      cudaGetLastError();                                                           \
      return bfail(XPBD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    }                                                                               \
  } while (0)

struct Batch {
  int res_ctas = 1;   // CTAs of the residual sweep (resident CTAs of the GPU)
  int res_ctas2 = 1;  // the same for the two-tets-per-thread residual
  xpbd_params prm{};
  BDev d{};
  int cur = 0;
  int n_out = 0;
  bool capturing = false;
  cudaStream_t cap = nullptr;
  cudaStream_t cap_body = nullptr;  // captures the body of a stop-mode loop node
  cudaStream_t aux = nullptr;       // stop mode: kb_list beside the update
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaStream_t aux_body = nullptr;  // the same inside the body of a loop node
  float4* tape_post = nullptr;      // taping through omega: where the update writes post-Jacobi positions
  float4* tape_xs = nullptr;        // taping: where the update writes the next iteration's positions
  cudaEvent_t ev_fork_body = nullptr, ev_join_body = nullptr;
  cudaGraphExec_t exec = nullptr;
  double key_frame_dt = -1, key_dt = -1;
  int key_sub = -1;
  bool profiling = false;
  bool pdl = true;  // programmatic dependent launch of the reverse iterations (off with XPBD_NO_PDL=1)
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[XPBD_K_COUNT];
  double prof_ms[XPBD_K_COUNT] = {0, 0, 0, 0, 0, 0};
  long long prof_n[XPBD_K_COUNT] = {0, 0, 0, 0, 0, 0};
};

inline cudaStream_t BS(void* s) { return reinterpret_cast<cudaStream_t>(s); }
inline int nblk(int n) { return (n + 255) / 256; }

struct BProf {
  Batch* s;
  int cls;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  cudaEvent_t take() {
    if (!s->pool.empty()) {
      cudaEvent_t e = s->pool.back();
      s->pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    return cudaEventCreate(&e) == cudaSuccess ? e : nullptr;
  }
  BProf(Batch* s_, int c, cudaStream_t st_) : s(s_), cls(c), st(st_) {
    if (s->profiling && (a = take())) cudaEventRecord(a, st);
  }
  ~BProf() {
    if (!a) return;
    cudaEvent_t b = take();
    if (!b) return;
    cudaEventRecord(b, st);
    s->pending[cls].push_back({a, b});
  }
};

// tets per thread of the batched tile kernels: 1, or 2 (params 2 and 4)
inline int batch_tpt(const xpbd_params& p) { return p.tets_per_thread >= 2 ? 2 : 1; }

template <bool kBlock, bool kFirst, int kTPT, bool kTetMat>
void project_btm(Batch* s, float inv_dt2, cudaStream_t st) {
  const xpbd_params& p = s->prm;
  const float rh = p.hydrostatic_relaxation, rd = p.deviatoric_relaxation;
  if (p.precise_hydro)
    kb_project<kBlock, kFirst, true, kTPT, kTetMat><<<s->d.n_patches, kP / kTPT, 0, st>>>(s->d, s->cur, inv_dt2, rh,
                                                                                          rd);
  else
    kb_project<kBlock, kFirst, false, kTPT, kTetMat><<<s->d.n_patches, kP / kTPT, 0, st>>>(s->d, s->cur, inv_dt2,
                                                                                           rh, rd);
}

template <bool kBlock, bool kFirst, int kTPT>
void project_bt(Batch* s, float inv_dt2, cudaStream_t st) {
  if (s->d.tinv_mu) project_btm<kBlock, kFirst, kTPT, true>(s, inv_dt2, st);
  else project_btm<kBlock, kFirst, kTPT, false>(s, inv_dt2, st);
}

template <bool kBlock, bool kFirst>
void project_b(Batch* s, float inv_dt2, cudaStream_t st) {
  if (batch_tpt(s->prm) == 2) project_bt<kBlock, kFirst, 2>(s, inv_dt2, st);
  else project_bt<kBlock, kFirst, 1>(s, inv_dt2, st);
}

template <bool kRes, bool kMon, bool kTetMat>
void residual_bm(Batch* s, const BSweep& a, cudaStream_t st) {
  const bool two = batch_tpt(s->prm) == 2;
  const int ctas = two ? s->res_ctas2 : s->res_ctas;
  const int chunk = (s->d.n_patches + ctas - 1) / ctas;
  const int grid = (s->d.n_patches + chunk - 1) / chunk;
  const bool pr = s->prm.precise_hydro != 0;
  if (two) {
    if (pr) kb_residual<kRes, kMon, true, 2, kTetMat><<<grid, kP / 2, 0, st>>>(s->d, a, chunk);
    else kb_residual<kRes, kMon, false, 2, kTetMat><<<grid, kP / 2, 0, st>>>(s->d, a, chunk);
  } else {
    if (pr) kb_residual<kRes, kMon, true, 1, kTetMat><<<grid, kP, 0, st>>>(s->d, a, chunk);
    else kb_residual<kRes, kMon, false, 1, kTetMat><<<grid, kP, 0, st>>>(s->d, a, chunk);
  }
}

template <bool kRes, bool kMon>
void residual_b(Batch* s, const BSweep& a, cudaStream_t st) {
  if (s->d.tinv_mu && kRes) residual_bm<kRes, kMon, true>(s, a, st);
  else residual_bm<kRes, kMon, false>(s, a, st);
}

inline bool stop_mode_b(const xpbd_params& p) { return p.target_rel_residual > 0.0 || p.residual_floor > 0.0; }

// Second stream and events on which stop mode runs kb_list beside the update.
// A stream that joins a capture belongs to it until that capture ends, so the
// body of a loop node (captured while the frame's capture is open) has its own.
struct Fork {
  cudaStream_t aux;
  cudaEvent_t fork, join;
};

// One Jacobi iteration of every body.  `first`: iteration 0 (lambda reset);
// `par`: the iteration's index & 1 (the index itself is on the device);
// `cond`: the loop condition of a stop-mode frame graph (nullptr: none).
int iteration_b(Batch* s, bool first, int par, float dt, int rec_base, cudaStream_t st,
                const cudaGraphConditionalHandle* cond, const Fork& fk) {
  const xpbd_params& p = s->prm;
  const bool stop = stop_mode_b(p);
  const float inv_dt2 = (float)(1.0 / ((double)dt * (double)dt));
  s->d.stop_par = stop ? par : -1;
  {
    BProf pr(s, XPBD_K_PROJECT, st);
    const bool blk = p.block_mode != 0;
    if (first) blk ? project_b<true, true>(s, inv_dt2, st) : project_b<false, true>(s, inv_dt2, st);
    else blk ? project_b<true, false>(s, inv_dt2, st) : project_b<false, false>(s, inv_dt2, st);
  }
  const bool cheb = p.cheb_enable != 0, mon = p.monitor != 0;
  if (cheb || mon || stop) {
    BSweep a;
    a.cur = s->cur;
    a.inv_dt2 = inv_dt2;
    a.par = par;
    a.warmup = p.cheb_warmup;
    a.rec_base = rec_base;
    a.res = cheb;
    a.stop = stop;
    a.rho_min = p.rho_min;
    a.rho_max = p.rho_max;
    a.rho_beta = p.rho_beta;
    a.target = p.target_rel_residual;
    a.floor = p.residual_floor;
    BProf pr(s, XPBD_K_RESIDUAL, st);
    if ((cheb || stop) && mon) residual_b<true, true>(s, a, st);
    else if (cheb || stop) residual_b<true, false>(s, a, st);
    else residual_b<false, true>(s, a, st);
  }
  if (stop) {
    // the next iteration's lists, beside the update (both follow the residual)
    B_CUDA(cudaEventRecord(fk.fork, st));
    B_CUDA(cudaStreamWaitEvent(fk.aux, fk.fork, 0));
    kb_list<<<1, 1024, 0, fk.aux>>>(s->d, par);
    B_CUDA(cudaEventRecord(fk.join, fk.aux));
  }
  BProf pr(s, XPBD_K_UPDATE, st);
  const int g = (nblk(s->d.V) + kBUpdateBlocks - 1) / kBUpdateBlocks;
  BUpd u{};
  u.par = par;
  u.K = p.constraints_iter;
  u.stop = stop;
  u.use_cond = cond != nullptr;
  if (cond) u.cond = *cond;
  u.post_out = s->tape_post;
  u.xs_out = s->tape_xs;
  if (cheb) {
    if (first) kb_update<true, true><<<g, 256, 0, st>>>(s->d, s->cur, p.cheb_gamma, u);
    else kb_update<true, false><<<g, 256, 0, st>>>(s->d, s->cur, p.cheb_gamma, u);
    s->cur ^= 1;
  } else {
    kb_update<false, false><<<g, 256, 0, st>>>(s->d, s->cur, p.cheb_gamma, u);
  }
  s->d.stop_par = -1;
  if (stop) B_CUDA(cudaStreamWaitEvent(st, fk.join, 0));
  return XPBD_OK;
}

// Stop mode under capture: iterations 0 and 1 as plain nodes, then a WHILE
// conditional node over iterations of parity 0 and 1, looping while any body
// iterates (the condition comes from every update from iteration 1 on).
int capture_stop_loop_b(Batch* s, float dt, int rec_base, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaGraph_t g = nullptr;
  B_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  if (cs != cudaStreamCaptureStatusActive || !g) return bfail(XPBD_ERR_CUDA, "stop-mode loop outside a capture");
  cudaGraphConditionalHandle h = 0;
  B_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
  const Fork fk{s->aux, s->ev_fork, s->ev_join}, fkb{s->aux_body, s->ev_fork_body, s->ev_join_body};
  int r = iteration_b(s, true, 0, dt, rec_base, st, nullptr, fk);
  if (!r) r = iteration_b(s, false, 1, dt, rec_base, st, &h, fk);
  if (r) return r;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nd = 0;
  B_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &nd));
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  B_CUDA(cudaGraphAddNode(&node, g, deps, edges, nd, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  B_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  B_CUDA(cudaStreamBeginCaptureToGraph(s->cap_body, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  r = iteration_b(s, false, 0, dt, rec_base, s->cap_body, &h, fkb);
  if (!r) r = iteration_b(s, false, 1, dt, rec_base, s->cap_body, &h, fkb);
  cudaGraph_t out = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s->cap_body, &out);
  if (r) return r;
  B_CUDA(e);
  return XPBD_OK;
}

int substep_b(Batch* s, float dt, int rec_base, cudaStream_t st) {
  const int K = s->prm.constraints_iter;
  if (rec_base >= 0 && rec_base + K > s->d.max_records) return bfail(XPBD_ERR_HISTORY_FULL, "history full");
  const bool stop = stop_mode_b(s->prm);
  s->cur = 0;
  {
    BProf pr(s, XPBD_K_BEGIN, st);
    s->d.stop_par = stop ? 0 : -1;  // stop mode: kb_begin lists every patch
    kb_begin<<<nblk(s->d.V), 256, 0, st>>>(s->d, dt, s->prm.gravity[0], s->prm.gravity[1], s->prm.gravity[2], K);
    s->d.stop_par = -1;
  }
  if (stop && s->capturing && K > 2) {
    int r = capture_stop_loop_b(s, dt, rec_base, st);
    if (r) return r;
  } else {
    const Fork fk{s->aux, s->ev_fork, s->ev_join};
    for (int it = 0; it < K; ++it) {
      const int r = iteration_b(s, it == 0, it & 1, dt, rec_base, st, nullptr, fk);
      if (r) return r;
    }
  }
  const int sub = rec_base >= 0 && K > 0 ? rec_base / K : -1;
  BProf pr(s, XPBD_K_END, st);
  kb_end<<<nblk(s->d.V), 256, 0, st>>>(s->d, s->cur, dt, s->prm.damping, stop ? 1 : 0, s->prm.cheb_enable ? 1 : 0,
                                      sub);
  return XPBD_OK;
}

int frame_b(Batch* s, double frame_dt, double dt, int substeps, cudaStream_t st) {
  double left = frame_dt;
  int rec = 0;
  while (left > 0.0) {
    const double dt0 = dt < left ? dt : left;
    left -= dt0;
    const float sub = (float)(dt0 / substeps);
    for (int k = 0; k < substeps; ++k) {
      const int base = rec + s->prm.constraints_iter <= s->d.max_records ? rec : -1;
      int r = substep_b(s, sub, base, st);
      if (r) return r;
      rec += s->prm.constraints_iter;
    }
  }
  return XPBD_OK;
}

void drop_b(Batch* s) {
  if (s->exec) cudaGraphExecDestroy(s->exec);
  s->exec = nullptr;
  s->key_frame_dt = s->key_dt = -1;
  s->key_sub = -1;
}

}  // namespace

extern "C" {

const char* xpbd_batch_last_error(void) { return g_err.c_str(); }

int xpbd_batch_create(const xpbd_params* params, const xpbd_batch* body, const xpbd_sdf* sdfs, int32_t n_sdf,
                      int32_t max_records, void** out_handle) {
  g_err.clear();
  if (!out_handle || !body || !params) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL argument");
  *out_handle = nullptr;
  if (n_sdf <= 0 || !sdfs) return bfail(XPBD_ERR_NO_SDF, "At least one SDF object must be provided.");
  for (int k = 0; k < n_sdf; ++k)
    if (sdfs[k].kind < XPBD_SDF_PLANE || sdfs[k].kind > XPBD_SDF_CUBE)
      return bfail(XPBD_ERR_INVALID_ARGUMENT, "unknown SDF kind");
  if (body->n_bodies <= 0 || body->n_verts <= 0 || body->n_tets <= 0 || body->n_patches <= 0)
    return bfail(XPBD_ERR_BAD_MESH, "empty batch");
  if (body->n_verts % 256 || body->n_tets != body->n_patches * kP)
    return bfail(XPBD_ERR_BAD_MESH, "n_verts must be a multiple of 256 and n_tets = 256 n_patches");
  if (!body->x || !body->v || !body->p0 || !body->p1 || !body->dx || !body->dm_a || !body->dm_b || !body->dm_c ||
      !body->lam || !body->tet_lid || !body->patch_voff || !body->patch_verts || !body->patch_body ||
      !body->patch_ntets || !body->vblock_body || !body->body_inv_mu || !body->body_inv_lambda ||
      !body->body_n_patches || !body->body_n_tets || !body->vert_perm)
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL batch buffer");
  if ((body->tet_inv_mu == nullptr) != (body->tet_inv_lambda == nullptr))
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "per-tet materials need both tet_inv_mu and tet_inv_lambda");
  if (max_records < 0) return bfail(XPBD_ERR_INVALID_ARGUMENT, "max_records < 0");
  if (!(params->target_rel_residual >= 0.0) || !(params->residual_floor >= 0.0))
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "target_rel_residual and residual_floor must be >= 0");
  Batch* s = new (std::nothrow) Batch();
  if (s) {
    const char* no_pdl = std::getenv("XPBD_NO_PDL");
    s->pdl = !(no_pdl && no_pdl[0] == '1');
  }
  if (!s) return bfail(XPBD_ERR_INVALID_ARGUMENT, "out of host memory");
  s->prm = *params;
  s->d.stop_par = -1;
  s->n_out = body->n_out_verts;
  BDev& d = s->d;
  d.V = body->n_verts;
  d.T = body->n_tets;
  d.n_patches = body->n_patches;
  d.n_bodies = body->n_bodies;
  d.n_sdf = n_sdf;
  d.n_pverts = body->n_patch_verts;
  d.x = reinterpret_cast<float4*>(body->x);
  d.v = reinterpret_cast<float4*>(body->v);
  d.p[0] = reinterpret_cast<float4*>(body->p0);
  d.p[1] = reinterpret_cast<float4*>(body->p1);
  d.dx = reinterpret_cast<float4*>(body->dx);
  d.dm_a = reinterpret_cast<const float4*>(body->dm_a);
  d.dm_b = reinterpret_cast<const float4*>(body->dm_b);
  d.dm_c = body->dm_c;
  d.lam = reinterpret_cast<float2*>(body->lam);
  d.lid = body->tet_lid;
  d.voff = body->patch_voff;
  d.pverts = body->patch_verts;
  d.patch_body = body->patch_body;
  d.patch_ntets = body->patch_ntets;
  d.vblock_body = body->vblock_body;
  d.inv_mu = body->body_inv_mu;
  d.inv_la = body->body_inv_lambda;
  d.tinv_mu = body->tet_inv_mu;
  d.tinv_la = body->tet_inv_mu ? body->tet_inv_lambda : nullptr;
  d.paired = body->tet_pairs != 0;
  d.body_patches = body->body_n_patches;
  d.body_tets = body->body_n_tets;
  d.perm = body->vert_perm;
  d.max_records = max_records > 0 ? max_records : 1;
  auto cleanup = [&](int st) {
    if (d.sdfs) cudaFree(const_cast<xpbd_sdf*>(d.sdfs));
    if (d.bs) cudaFree(d.bs);
    if (d.flags) cudaFree(d.flags);
    if (d.hist) cudaFree(d.hist);
    if (d.ctl) cudaFree(d.ctl);
    if (d.act_patch[0]) cudaFree(d.act_patch[0]);
    if (d.act_vblock[0]) cudaFree(d.act_vblock[0]);
    if (d.act_off) cudaFree(d.act_off);
    if (d.body_vfirst) cudaFree(const_cast<int*>(d.body_vfirst));
    if (d.body_vblocks) cudaFree(const_cast<int*>(d.body_vblocks));
    if (s->aux) cudaStreamDestroy(s->aux);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_join) cudaEventDestroy(s->ev_join);
    if (s->aux_body) cudaStreamDestroy(s->aux_body);
    if (s->ev_fork_body) cudaEventDestroy(s->ev_fork_body);
    if (s->ev_join_body) cudaEventDestroy(s->ev_join_body);
    if (d.body_first) cudaFree(const_cast<int*>(d.body_first));
    if (d.iters) cudaFree(d.iters);
    if (s->cap) cudaStreamDestroy(s->cap);
    if (s->cap_body) cudaStreamDestroy(s->cap_body);
    delete s;
    return st;
  };
  xpbd_sdf* ds = nullptr;
  cudaError_t e = cudaMalloc(&ds, sizeof(xpbd_sdf) * n_sdf);
  d.sdfs = ds;
  if (e == cudaSuccess) e = cudaMemcpy(ds, sdfs, sizeof(xpbd_sdf) * n_sdf, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&d.bs, sizeof(BodyState) * d.n_bodies);
  if (e == cudaSuccess) e = cudaMalloc(&d.flags, sizeof(Flags));
  if (e == cudaSuccess) e = cudaMalloc(&d.hist, sizeof(double) * 4 * (size_t)d.max_records * d.n_bodies);
  if (e == cudaSuccess) e = cudaMalloc(&d.ctl, sizeof(Ctl));
  const size_t nvb = (size_t)d.V / 256;
  if (e == cudaSuccess) e = cudaMalloc(&d.act_patch[0], sizeof(int) * 2 * (size_t)d.n_patches);
  if (e == cudaSuccess) e = cudaMalloc(&d.act_vblock[0], sizeof(int) * 2 * nvb);
  if (e == cudaSuccess) e = cudaMalloc(&d.act_off, sizeof(int) * 2 * (size_t)d.n_bodies);
  int *bvfirst = nullptr, *bvblocks = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&bvfirst, sizeof(int) * (size_t)d.n_bodies);
  d.body_vfirst = bvfirst;
  if (e == cudaSuccess) e = cudaMalloc(&bvblocks, sizeof(int) * (size_t)d.n_bodies);
  d.body_vblocks = bvblocks;
  if (e == cudaSuccess) {
    d.act_patch[1] = d.act_patch[0] + d.n_patches;
    d.act_vblock[1] = d.act_vblock[0] + nvb;
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->aux_body, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork_body, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join_body, cudaEventDisableTiming);
  int* bfirst = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&bfirst, sizeof(int) * (size_t)d.n_bodies);
  d.body_first = bfirst;
  if (e == cudaSuccess) e = cudaMalloc(&d.iters, sizeof(int) * (size_t)kMaxCountedSubsteps * d.n_bodies);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cap_body, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cleanup(bfail(XPBD_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e)));
  std::vector<BodyState> hb(d.n_bodies);
  for (auto& b : hb) {
    std::memset(&b, 0, sizeof(b));
    b.rho_hat = 0.999;  // neohookean_solver.py:65
    b.omega = 1.0;
  }
  Flags hf{0, 0};
  e = cudaMemcpy(d.bs, hb.data(), sizeof(BodyState) * d.n_bodies, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d.flags, &hf, sizeof(hf), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d.hist, 0, sizeof(double) * 4 * (size_t)d.max_records * d.n_bodies);
  if (e == cudaSuccess) e = cudaMemset(d.ctl, 0, sizeof(Ctl));
  {
    // first patch of every body: the exclusive prefix of the patch counts
    std::vector<int> np(d.n_bodies), first(d.n_bodies);
    if (e == cudaSuccess)
      e = cudaMemcpy(np.data(), body->body_n_patches, sizeof(int) * (size_t)d.n_bodies, cudaMemcpyDeviceToHost);
    long long acc = 0;
    for (int b = 0; b < d.n_bodies && e == cudaSuccess; ++b) {
      first[b] = (int)acc;
      acc += np[b] > 0 ? np[b] : 0;
    }
    if (e == cudaSuccess && acc != d.n_patches)
      return cleanup(bfail(XPBD_ERR_BAD_MESH, "body_n_patches do not add up to n_patches"));
    if (e == cudaSuccess) e = cudaMemcpy(bfirst, first.data(), sizeof(int) * (size_t)d.n_bodies, cudaMemcpyHostToDevice);
    // every body's vertex blocks: a contiguous run of vblock_body
    std::vector<int> vbody((size_t)d.V / 256), vf(d.n_bodies, -1), vn(d.n_bodies, 0);
    if (e == cudaSuccess && !vbody.empty())
      e = cudaMemcpy(vbody.data(), body->vblock_body, sizeof(int) * vbody.size(), cudaMemcpyDeviceToHost);
    bool contiguous = true;
    for (size_t k = 0; k < vbody.size() && e == cudaSuccess; ++k) {
      const int b = vbody[k];
      if (b < 0 || b >= d.n_bodies) {
        contiguous = false;
        break;
      }
      if (vn[b] == 0) vf[b] = (int)k;
      else if (vf[b] + vn[b] != (int)k) contiguous = false;
      ++vn[b];
    }
    if (e == cudaSuccess && !contiguous)
      return cleanup(bfail(XPBD_ERR_BAD_MESH, "a body's vertex blocks must be consecutive"));
    if (e == cudaSuccess) e = cudaMemcpy(bvfirst, vf.data(), sizeof(int) * (size_t)d.n_bodies, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(bvblocks, vn.data(), sizeof(int) * (size_t)d.n_bodies, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemset(d.iters, 0, sizeof(int) * (size_t)kMaxCountedSubsteps * d.n_bodies);
  if (e != cudaSuccess) return cleanup(bfail(XPBD_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e)));
  {
    int dev = 0, sms = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kb_residual<true, false, true, 1, false>, kP, 0) != cudaSuccess ||
        bps < 1)
      bps = 2;
    s->res_ctas = sms * bps > 0 ? sms * bps : 1;
    bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kb_residual<true, false, true, 2, false>, kP / 2, 0) !=
            cudaSuccess ||
        bps < 1)
      bps = 4;
    s->res_ctas2 = sms * bps > 0 ? sms * bps : 1;
  }
  const int nval = d.V > d.n_patches ? d.V : d.n_patches;
  kb_validate<<<nblk(nval), 256>>>(d, s->n_out);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&hf, d.flags, sizeof(hf), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cleanup(bfail(XPBD_ERR_CUDA, std::string("validate: ") + cudaGetErrorString(e)));
  if (hf.bad_mesh) return cleanup(bfail(XPBD_ERR_BAD_MESH, "batch index out of range"));
  *out_handle = s;
  return XPBD_OK;
}

int xpbd_batch_destroy(void* h) {
  Batch* s = static_cast<Batch*>(h);
  if (!s) return XPBD_OK;
  drop_b(s);
  for (auto& v : s->pending)
    for (auto& pr : v) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  for (cudaEvent_t e : s->pool) cudaEventDestroy(e);
  cudaFree(const_cast<xpbd_sdf*>(s->d.sdfs));
  cudaFree(s->d.bs);
  cudaFree(s->d.flags);
  cudaFree(s->d.hist);
  cudaFree(s->d.ctl);
  cudaFree(s->d.act_patch[0]);
  cudaFree(s->d.act_vblock[0]);
  cudaFree(s->d.act_off);
  cudaFree(const_cast<int*>(s->d.body_vfirst));
  cudaFree(const_cast<int*>(s->d.body_vblocks));
  if (s->aux) cudaStreamDestroy(s->aux);
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->ev_join) cudaEventDestroy(s->ev_join);
  if (s->aux_body) cudaStreamDestroy(s->aux_body);
  if (s->ev_fork_body) cudaEventDestroy(s->ev_fork_body);
  if (s->ev_join_body) cudaEventDestroy(s->ev_join_body);
  cudaFree(const_cast<int*>(s->d.body_first));
  cudaFree(s->d.iters);
  if (s->cap) cudaStreamDestroy(s->cap);
  if (s->cap_body) cudaStreamDestroy(s->cap_body);
  delete s;
  return XPBD_OK;
}

int xpbd_batch_substep(void* h, float dt, int32_t record_base, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  int r = substep_b(s, dt, record_base, BS(stream));
  if (r) return r;
  B_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_batch_solve(void* h, double frame_dt, double dt, int32_t substeps, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  if (substeps <= 0 || !(dt > 0.0) || !(frame_dt >= 0.0) || frame_dt / dt > 1e6)
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "need substeps > 0, dt > 0, frame_dt >= 0");
  if (!s->prm.use_graph || s->profiling) {
    int r = frame_b(s, frame_dt, dt, substeps, BS(stream));
    if (r) return r;
    B_CUDA(cudaGetLastError());
    return XPBD_OK;
  }
  if (!(s->exec && s->key_frame_dt == frame_dt && s->key_dt == dt && s->key_sub == substeps)) {
    drop_b(s);
    B_CUDA(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
    s->capturing = true;
    int r = frame_b(s, frame_dt, dt, substeps, s->cap);
    s->capturing = false;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s->cap, &g);
    if (r) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    if (e != cudaSuccess) return bfail(XPBD_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      s->exec = nullptr;
      return bfail(XPBD_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    }
    s->key_frame_dt = frame_dt;
    s->key_dt = dt;
    s->key_sub = substeps;
  }
  B_CUDA(cudaGraphLaunch(s->exec, BS(stream)));
  return XPBD_OK;
}

int xpbd_batch_read_history(void* h, double* out, int32_t n, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !out || n < 0 || n > s->d.max_records) return bfail(XPBD_ERR_INVALID_ARGUMENT, "bad history read");
  B_CUDA(cudaStreamSynchronize(BS(stream)));
  for (int b = 0; b < s->d.n_bodies; ++b)
    B_CUDA(cudaMemcpy(out + 4 * (size_t)b * n, s->d.hist + 4 * (size_t)b * s->d.max_records,
                      sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost));
  return XPBD_OK;
}

int xpbd_batch_read_iterations(void* h, int32_t* host_out, int32_t n, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !host_out || n < 0 || n > kMaxCountedSubsteps)
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "bad iteration-count read (n must be 0.." +
                                                std::to_string(kMaxCountedSubsteps) + ")");
  B_CUDA(cudaStreamSynchronize(BS(stream)));
  for (int b = 0; b < s->d.n_bodies && n > 0; ++b)
    B_CUDA(cudaMemcpy(host_out + (size_t)b * n, s->d.iters + (size_t)b * kMaxCountedSubsteps, sizeof(int) * (size_t)n,
                      cudaMemcpyDeviceToHost));
  return XPBD_OK;
}

int xpbd_batch_get_rho_hat(void* h, double* out, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !out) return bfail(XPBD_ERR_INVALID_ARGUMENT, "bad argument");
  B_CUDA(cudaStreamSynchronize(BS(stream)));
  std::vector<BodyState> hb(s->d.n_bodies);
  B_CUDA(cudaMemcpy(hb.data(), s->d.bs, sizeof(BodyState) * s->d.n_bodies, cudaMemcpyDeviceToHost));
  for (int b = 0; b < s->d.n_bodies; ++b) out[b] = hb[b].rho_hat;
  return XPBD_OK;
}

int xpbd_batch_check_status(void* h, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  Flags f{0, 0};
  B_CUDA(cudaStreamSynchronize(BS(stream)));
  B_CUDA(cudaMemcpy(&f, s->d.flags, sizeof(f), cudaMemcpyDeviceToHost));
  return f.nonfinite ? bfail(XPBD_ERR_NONFINITE, "non-finite residual") : XPBD_OK;
}

int xpbd_batch_export_vec3(void* h, int32_t field, float* dst, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !dst) return bfail(XPBD_ERR_INVALID_ARGUMENT, "bad argument");
  if (field == XPBD_FIELD_PRED_X && stop_mode_b(s->prm))
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "in stop mode the predicted positions sit in a per-body buffer");
  const float4* f = field == XPBD_FIELD_X ? s->d.x : field == XPBD_FIELD_V ? s->d.v
                    : field == XPBD_FIELD_PRED_X ? s->d.p[s->cur] : nullptr;
  if (!f) return bfail(XPBD_ERR_INVALID_ARGUMENT, "unknown field");
  kb_export<<<nblk(s->d.V), 256, 0, BS(stream)>>>(s->d, f, dst);
  B_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_batch_import_vec3(void* h, int32_t field, const float* src, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !src) return bfail(XPBD_ERR_INVALID_ARGUMENT, "bad argument");
  if (field == XPBD_FIELD_PRED_X && stop_mode_b(s->prm))
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "in stop mode the predicted positions sit in a per-body buffer");
  float4* f = field == XPBD_FIELD_X ? s->d.x : field == XPBD_FIELD_V ? s->d.v
              : field == XPBD_FIELD_PRED_X ? s->d.p[s->cur] : nullptr;
  if (!f) return bfail(XPBD_ERR_INVALID_ARGUMENT, "unknown field");
  kb_import<<<nblk(s->d.V), 256, 0, BS(stream)>>>(s->d, f, src);
  B_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_batch_set_profiling(void* h, int32_t enable) {
  Batch* s = static_cast<Batch*>(h);
  if (!s) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  s->profiling = enable != 0;
  return XPBD_OK;
}

int xpbd_batch_read_profile(void* h, double* ms, int64_t* launches, int32_t n, int32_t reset, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || n < 0 || n > XPBD_K_COUNT) return bfail(XPBD_ERR_INVALID_ARGUMENT, "bad profile read");
  B_CUDA(cudaStreamSynchronize(BS(stream)));
  for (int k = 0; k < XPBD_K_COUNT; ++k) {
    for (auto& pr : s->pending[k]) {
      float t = 0.f;
      B_CUDA(cudaEventElapsedTime(&t, pr.first, pr.second));
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


int xpbd_batch_set_params(void* h, const xpbd_params* params) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !params) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or params");
  if (params->constraints_iter < 0 || params->cheb_warmup < 0)
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "constraints_iter and cheb_warmup must be >= 0");
  if (!(params->target_rel_residual >= 0.0) || !(params->residual_floor >= 0.0))
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "target_rel_residual and residual_floor must be >= 0");
  if (std::memcmp(&s->prm, params, sizeof(xpbd_params)) != 0) drop_b(s);
  s->prm = *params;
  return XPBD_OK;
}

int xpbd_batch_save_rho_hat(void* h, double* dst_device, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !dst_device) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or destination");
  kb_rho_copy<<<nblk(s->d.n_bodies), 256, 0, BS(stream)>>>(s->d, dst_device, nullptr);
  B_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_batch_load_rho_hat(void* h, const double* src_device, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !src_device) return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or source");
  kb_rho_copy<<<nblk(s->d.n_bodies), 256, 0, BS(stream)>>>(s->d, nullptr, src_device);
  B_CUDA(cudaGetLastError());
  return XPBD_OK;
}

static int check_batch_diff(Batch* s) {
  if (!s->prm.block_mode) return bfail(XPBD_ERR_INVALID_ARGUMENT, "the adjoint supports block mode only");
  if (stop_mode_b(s->prm)) return bfail(XPBD_ERR_INVALID_ARGUMENT, "the adjoint needs a fixed iteration count");
  if (s->prm.constraints_iter > s->d.max_records)
    return bfail(XPBD_ERR_HISTORY_FULL, "history shorter than constraints_iter");
  return XPBD_OK;
}

int xpbd_batch_substep_tape(void* h, float dt, const xpbd_tape* tape, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !tape || !tape->xs || !tape->lams || !tape->xpre || !tape->v1)
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or tape buffer");
  int r = check_batch_diff(s);
  if (r) return r;
  cudaStream_t st = BS(stream);
  const int K = s->prm.constraints_iter, V = s->d.V, T = s->d.T;
  Tape tp{reinterpret_cast<float4*>(tape->xs), reinterpret_cast<float2*>(tape->lams),
          reinterpret_cast<float4*>(tape->xpre), reinterpret_cast<float4*>(tape->v1),
          reinterpret_cast<float4*>(tape->posts), tape->rho_in};
  if (tp.posts && !tp.rho_in) return bfail(XPBD_ERR_INVALID_ARGUMENT, "a tape with posts needs rho_in");
  const float* g = s->prm.gravity;
  if (tp.posts) kb_rho_copy<<<nblk(s->d.n_bodies), 256, 0, st>>>(s->d, tp.rho_in, nullptr);
  k_tape_begin<BDev><<<nblk(V), 256, 0, st>>>(s->d, tp, dt, g[0], g[1], g[2]);
  s->cur = 0;
  kb_begin<<<nblk(V), 256, 0, st>>>(s->d, dt, g[0], g[1], g[2], K);
  // iteration 0 enters with the predicted positions and zero multipliers; after
  // it the projection records the multipliers entering each iteration and the
  // update the positions entering the next (xs[K]: those after the last)
  B_CUDA(cudaMemcpyAsync(tp.xs, s->d.p[s->cur], sizeof(float4) * V, cudaMemcpyDeviceToDevice, st));
  B_CUDA(cudaMemsetAsync(tp.lams, 0, sizeof(float2) * T, st));
  for (int it = 0; it < K; ++it) {
    s->d.lam_tape = it > 0 ? tp.lams + (size_t)it * T : nullptr;
    s->tape_post = tp.posts ? tp.posts + (size_t)it * V : nullptr;
    s->tape_xs = tp.xs + (size_t)(it + 1) * V;
    const int r = iteration_b(s, it == 0, it & 1, dt, 0, st, nullptr, Fork{s->aux, s->ev_fork, s->ev_join});
    s->d.lam_tape = nullptr;
    s->tape_post = nullptr;
    s->tape_xs = nullptr;
    if (r) return r;
  }
  if (tp.posts)  // the multipliers after the last iteration (the residual's lambda_K)
    B_CUDA(cudaMemcpyAsync(tp.lams + (size_t)K * T, s->d.lam, sizeof(float2) * T, cudaMemcpyDeviceToDevice, st));
  if (tape->hist)  // rows 0..K-1 of every body
    B_CUDA(cudaMemcpy2DAsync(tape->hist, sizeof(double) * 4 * (size_t)K, s->d.hist,
                             sizeof(double) * 4 * (size_t)s->d.max_records, sizeof(double) * 4 * (size_t)K,
                             (size_t)s->d.n_bodies, cudaMemcpyDeviceToDevice, st));
  kb_end<<<nblk(V), 256, 0, st>>>(s->d, s->cur, dt, s->prm.damping, 0, 0, -1);
  B_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_batch_substep_adjoint(void* h, float dt, const xpbd_tape* tape, const xpbd_adjoint* adj, void* stream) {
  Batch* s = static_cast<Batch*>(h);
  if (!s || !tape || !adj || !adj->gx || !adj->gv || !adj->g_inv_mu || !adj->g_inv_lambda || !adj->work0 ||
      !adj->work1 || !adj->ybar || !adj->dxbar || !adj->lambar || !adj->cnt)
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle, tape or adjoint buffer");
  int r = check_batch_diff(s);
  if (r) return r;
  cudaStream_t st = BS(stream);
  const int K = s->prm.constraints_iter, V = s->d.V, T = s->d.T;
  Tape tp{reinterpret_cast<float4*>(tape->xs), reinterpret_cast<float2*>(tape->lams),
          reinterpret_cast<float4*>(tape->xpre), reinterpret_cast<float4*>(tape->v1),
          reinterpret_cast<float4*>(tape->posts), tape->rho_in};
  // through omega: the tape holds the post-Jacobi positions and the adjoint a chain state
  const bool through_omega = tp.posts && tp.rho_in && adj->omega_state && s->prm.cheb_enable;
  BDev dv = s->d;  // the history rows of the substep: the tape's copy, else the batch's rows 0..K-1
  if (tape->hist) {
    dv.hist = tape->hist;
    dv.max_records = K;
  }
  Adj a;
  a.om = through_omega ? adj->omega_state : nullptr;
  a.om_n = om_stride(K);
  a.rtet = through_omega ? reinterpret_cast<float4*>(adj->work_res_tet) : nullptr;
  if (through_omega && !a.rtet)
    return bfail(XPBD_ERR_INVALID_ARGUMENT, "the omega chain of a batch needs work_res_tet");
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
  B_CUDA(cudaMemsetAsync(a.lambar, 0, sizeof(float2) * T, st));
  const float e_over_dt = expf(-dt * s->prm.damping) / dt;
  const ChainPrm cp{K, s->prm.cheb_warmup, s->prm.rho_min, s->prm.rho_max, s->prm.rho_beta};
  if (a.om) ka_chain<BDev><<<(s->d.n_bodies + 7) / 8, 256, 0, st>>>(dv, tp, a, cp);
  ka_end<BDev><<<nblk(V), 256, 0, st>>>(dv, a, e_over_dt);
  const float c = (float)(1.0 / ((double)dt * (double)dt));
  int src = 0;
  // the reverse iterations' kernels may each start while the one before
  // drains (programmatic dependent launch; they wait before reading its output)
  const bool o = s->pdl && !s->profiling;
  const int np = s->d.n_patches;
  for (int k = K - 1; k >= 0; --k) {
    if (s->prm.cheb_enable) launch_k(ka_cheb<BDev, true>, nblk(V), 256, 0, st, o, dv, tp, a, k, s->prm.cheb_gamma, src);
    else launch_k(ka_cheb<BDev, false>, nblk(V), 256, 0, st, o, dv, tp, a, k, s->prm.cheb_gamma, src);
    if (through_omega) {
      if (s->prm.precise_hydro) launch_k(kba_residual_adj<true>, np, kP, 0, st, o, dv, tp, a, k, c, src ^ 1);
      else launch_k(kba_residual_adj<false>, np, kP, 0, st, o, dv, tp, a, k, c, src ^ 1);
    }
    if (s->prm.precise_hydro) launch_k(kba_project<true>, np, kP, 0, st, o, dv, tp, a, k, c, src ^ 1);
    else launch_k(kba_project<false>, np, kP, 0, st, o, dv, tp, a, k, c, src ^ 1);
    src ^= 1;
  }
  ka_begin<BDev><<<nblk(V), 256, 0, st>>>(dv, tp, a, src, dt);
  B_CUDA(cudaGetLastError());
  return XPBD_OK;
}

}  // extern "C"

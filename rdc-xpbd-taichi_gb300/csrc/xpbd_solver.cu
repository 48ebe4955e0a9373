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
//                  FP64 reduction, last block updates rho_hat/omega  :298-329, :492-546
//     update  (V): post_solve + Chebyshev mix, dx reset          :115-142, :548-549
//   end     (V): velocity update                                xpbd_base.py:148-160
// The predicted positions ping-pong between p0/p1: the Chebyshev mix writes
// x_{k+1} over y_{k-1} in place, so no buffer copies are needed
// (neohookean_solver.py:121-142 copies three buffers instead).

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "xpbd_device.cuh"

namespace xpbd {

constexpr int kBlock = 256;

// FP64 solver state that lives on the device (neohookean_solver.py:59-69).
struct DevState {
  double acc[3];        // residual sum, |C_H| sum, |C_D| sum of the running sweep
  unsigned int ticket;  // blocks finished in the running sweep
  int has_prev;         // prev_r_hat is not None
  double rho_hat;       // persists across substeps and frames
  double prev_r_hat;
  double omega;         // omega of the latest iteration of this substep
  int nonfinite;        // sticky: a residual sum was NaN/Inf
  int bad_mesh;         // set by the index validation kernel
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
  const float2* dm_c;
  float2* lam;
  const int* v2t_off;
  const int* v2t_slot;
  float4* corner;
  const int* perm;  // solver vertex i <- caller vertex perm[i] (nullptr = identity)
  const xpbd_sdf* sdfs;
  int n_sdf;
  DevState* st;
  double* hist;
};

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

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
    d.st->has_prev = 0;
    d.st->omega = 1.0;
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

// advance (xpbd_base.py:148-160) from p[cur].
__global__ void __launch_bounds__(kBlock) k_end(Dev d, int cur, float dt, float damping) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
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
  if (i >= d.V) return;
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
template <bool kCheb, bool kFirstIt, bool kResetDx>
__global__ void __launch_bounds__(kBlock) k_update(Dev d, int cur, float gamma) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
  const float4 pc = d.p[cur][i];
  const float4 D = d.dx[i];
  if (kResetDx) d.dx[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  float3 xp = make_float3(pc.x, pc.y, pc.z);
  if (D.w > 0.f) {
    xp.x += D.x / D.w;
    xp.y += D.y / D.w;
    xp.z += D.z / D.w;
  }
  if (kCheb) {
    const float om = (float)d.st->omega;
    const float4 yp = kFirstIt ? pc : d.p[cur ^ 1][i];
    const float nx = gamma * (xp.x - pc.x) + pc.x;
    const float ny = gamma * (xp.y - pc.y) + pc.y;
    const float nz = gamma * (xp.z - pc.z) + pc.z;
    d.p[cur ^ 1][i] = make_float4(yp.x + om * (nx - yp.x), yp.y + om * (ny - yp.y), yp.z + om * (nz - yp.z), pc.w);
  } else {
    d.p[cur][i] = make_float4(xp.x, xp.y, xp.z, pc.w);
  }
}

// ---------------------------------------------------------------------------
// tet kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ void load_tet(const Dev& d, int t, int4& id, Tet& tt) {
  id = __ldg(d.tets + t);
  const float4 a = __ldg(d.dm_a + t);
  const float4 b = __ldg(d.dm_b + t);
  const float2 c = __ldg(d.dm_c + t);
  tt.dm[0] = a.x; tt.dm[1] = a.y; tt.dm[2] = a.z;
  tt.dm[3] = a.w; tt.dm[4] = b.x; tt.dm[5] = b.y;
  tt.dm[6] = b.z; tt.dm[7] = b.w; tt.dm[8] = c.x;
  tt.V0 = c.y;
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
template <bool kBlockMode, bool kFirst, bool kPrecise, bool kGather>
__global__ void __launch_bounds__(kBlock) k_project(Dev d, int cur, float dt, float mu, float la, float relax_h,
                                                   float relax_d) {
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
  const float w[4] = {tt.p[0].w, tt.p[1].w, tt.p[2].w, tt.p[3].w};
  const int vid[4] = {id.x, id.y, id.z, id.w};

  float F[9];
  deformation_gradient(tt, F);
  float C_D, C_H;
  invariants<kPrecise>(F, C_D, C_H);
  float gF[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) gF[k] = F[k] * 2.f;
  float3 gD[4];
  corner_gradients(gF, tt.dm, gD);
  float H[9];
  cofactor(F, H);
  float3 gH[4];
  corner_gradients(H, tt.dm, gH);

  const float alpha_D = 1.f / (mu * tt.V0);
  const float alpha_H = 1.f / (la * tt.V0);
  const float dt2 = dt * dt;

  if (kBlockMode) {
    float A11 = w[0] * dot3(gD[0], gD[0]) + w[1] * dot3(gD[1], gD[1]) + w[2] * dot3(gD[2], gD[2]) +
                w[3] * dot3(gD[3], gD[3]);
    float A22 = w[0] * dot3(gH[0], gH[0]) + w[1] * dot3(gH[1], gH[1]) + w[2] * dot3(gH[2], gH[2]) +
                w[3] * dot3(gH[3], gH[3]);
    const float A12 = w[0] * dot3(gD[0], gH[0]) + w[1] * dot3(gD[1], gH[1]) + w[2] * dot3(gD[2], gH[2]) +
                      w[3] * dot3(gD[3], gH[3]);
    const float aD = alpha_D / dt2;
    const float aH = alpha_H / dt2;
    A11 += aD;
    A22 += aH;
    const float b1 = -(C_D + aD * L.x);
    const float b2 = -(C_H + aH * L.y);
    float dD, dH;
    if (!solve2x2_pivot_lu(A11, A12, A12, A22, b1, b2, dD, dH)) {
      // :425-432 ill-conditioned fallback: diagonal scalar updates
      dD = fabsf(A11) > kEps ? b1 / A11 : 0.f;
      dH = fabsf(A22) > kEps ? b2 / A22 : 0.f;
    }
    d.lam[t] = make_float2(L.x + dD, L.y + dH);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float3 dp = make_float3(w[c] * (gD[c].x * dD + gH[c].x * dH), w[c] * (gD[c].y * dD + gH[c].y * dH),
                                    w[c] * (gD[c].z * dD + gH[c].z * dH));
      emit<kGather>(d, t, c, vid[c], dp, 1.f);
    }
  } else {
    // hydrostatic then deviatoric, each gated by w_sum > EPS (:237, :177)
    float wsH = w[0] * dot3(gH[0], gH[0]);
    wsH += w[1] * dot3(gH[1], gH[1]);
    wsH += w[2] * dot3(gH[2], gH[2]);
    wsH += w[3] * dot3(gH[3], gH[3]);
    float wsD = w[0] * dot3(gD[0], gD[0]);
    wsD += w[1] * dot3(gD[1], gD[1]);
    wsD += w[2] * dot3(gD[2], gD[2]);
    wsD += w[3] * dot3(gD[3], gD[3]);
    float dlH = 0.f, dlD = 0.f, cH = 0.f, cD = 0.f;
    if (wsH > kEps) {
      const float at = alpha_H / dt2;
      dlH = -(C_H + at * L.y) / (wsH + at);
      dlH *= relax_h;
      cH = 1.f;
    }
    if (wsD > kEps) {
      const float at = alpha_D / dt2;
      dlD = -(C_D + at * L.x) / (wsD + at);
      dlD *= relax_d;
      cD = 1.f;
    }
    d.lam[t] = make_float2(L.x + dlD, L.y + dlH);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float sH = dlH * w[c], sD = dlD * w[c];
      const float3 dp = make_float3(sH * gH[c].x + sD * gD[c].x, sH * gH[c].y + sD * gD[c].y,
                                    sH * gH[c].z + sD * gD[c].z);
      emit<kGather>(d, t, c, vid[c], dp, cH + cD);
    }
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
  float dt, mu, la;
  int it, warmup, rec;
  double rho_min, rho_max, rho_beta;
};

// compute_xpbd_residual (neohookean_solver.py:298-329) and the monitoring
// errors (:256-296) at the post-Jacobi positions p[cur] + dx/count, i.e.
// before the Chebyshev mix (:490-494).  Per-thread FP32 partials over a
// grid-stride range, FP64 warp/block/grid reduction.  The last block to
// finish applies the rho_hat / omega recurrence (:495-504, :537-546) in FP64
// and writes history row `rec` = {r_hat, omega, hydro, dev}.
template <bool kRes, bool kMon, bool kPrecise>
__global__ void __launch_bounds__(kBlock) k_residual(Dev d, SweepArgs a) {
  float sr = 0.f, sh = 0.f, sd = 0.f;
  const float4* P = d.p[a.cur];
  const float dt2 = a.dt * a.dt;
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
    float F[9];
    deformation_gradient(tt, F);
    float C_D, C_H;
    invariants<kPrecise>(F, C_D, C_H);
    if (kRes) {
      const float2 L = d.lam[t];
      const float aD = (1.f / (a.mu * tt.V0)) / dt2;
      const float aH = (1.f / (a.la * tt.V0)) / dt2;
      const float rD = C_D + aD * L.x;
      const float rH = C_H + aH * L.y;
      sr += sqrtf(rD * rD + rH * rH);
    }
    if (kMon) {
      sh += fabsf(C_H);
      sd += fabsf(C_D);
    }
  }
  __shared__ double red[3][kBlock / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double r0 = warp_sum((double)sr), r1 = warp_sum((double)sh), r2 = warp_sum((double)sd);
  if (lane == 0) {
    red[0][warp] = r0;
    red[1][warp] = r1;
    red[2][warp] = r2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b0 = 0.0, b1 = 0.0, b2 = 0.0;
    for (int k = 0; k < kBlock / 32; ++k) {
      b0 += red[0][k];
      b1 += red[1][k];
      b2 += red[2][k];
    }
    if (kRes) atomicAdd(&d.st->acc[0], b0);
    if (kMon) {
      atomicAdd(&d.st->acc[1], b1);
      atomicAdd(&d.st->acc[2], b2);
    }
    __threadfence();
    const unsigned int tk = atomicAdd(&d.st->ticket, 1u);
    last = (tk == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  volatile DevState* st = d.st;
  const double S = st->acc[0], Hs = st->acc[1], Ds = st->acc[2];
  st->acc[0] = 0.0;
  st->acc[1] = 0.0;
  st->acc[2] = 0.0;
  st->ticket = 0u;
  const double n = (double)d.T;
  double r_hat = 0.0, omega = 1.0;
  if (kRes) {
    r_hat = d.T > 0 ? S / n : 0.0;
    if (!isfinite(S)) st->nonfinite = 1;
    if (st->has_prev && st->prev_r_hat > 1e-12) {
      double rho_inst = r_hat / (st->prev_r_hat + 1e-12);
      rho_inst = fmax(a.rho_min, fmin(a.rho_max, rho_inst));
      st->rho_hat = (1.0 - a.rho_beta) * st->rho_hat + a.rho_beta * rho_inst;
    }
    st->prev_r_hat = r_hat;
    st->has_prev = 1;
    const double rho = st->rho_hat;
    const double rho2 = rho * rho;
    if (a.it < a.warmup) omega = 1.0;
    else if (a.it == a.warmup) omega = 2.0 / (2.0 - rho2);
    else omega = 4.0 / (4.0 - rho2 * st->omega);
    st->omega = omega;
  }
  if (a.rec >= 0) {
    double* h = d.hist + 4 * (size_t)a.rec;
    h[0] = r_hat;
    h[1] = omega;
    h[2] = kMon && d.T > 0 ? Hs / n : 0.0;
    h[3] = kMon && d.T > 0 ? Ds / n : 0.0;
  }
}

// Field transfer in caller vertex order (mesh.verts.<f>.from_numpy / to_numpy).
__global__ void __launch_bounds__(kBlock) k_import(Dev d, float4* f, const float* __restrict__ src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.V) return;
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

}  // namespace xpbd

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

#define XPBD_CUDA(call)                                                                             \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fail(XPBD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct GraphKey {
  double frame_dt = -1.0, dt = -1.0;
  int substeps = -1;
};

struct Solver {
  // profiling (xpbd_set_profiling): event pairs per kernel class
  bool profiling = false;
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[XPBD_K_COUNT];
  double prof_ms[XPBD_K_COUNT] = {0, 0, 0, 0, 0, 0};
  long long prof_n[XPBD_K_COUNT] = {0, 0, 0, 0, 0, 0};
  xpbd_params prm{};
  Dev d{};
  int device = 0;
  int sm_count = 0;
  int max_records = 0;
  int cur = 0;  // buffer holding the current predicted positions
  cudaStream_t cap = nullptr;
  cudaGraphExec_t exec = nullptr;
  GraphKey key;
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
      if (a) cudaEventRecord(a, st);
    }
  }
  ~Prof() {
    if (!a) return;
    cudaEvent_t b = take_event(s);
    if (!b) return;
    cudaEventRecord(b, st);
    s->pending[cls].push_back({a, b});
  }
};

inline int blocks_for(int n) { return (n + kBlock - 1) / kBlock; }

int check_params(const xpbd_params* p) {
  if (!p) return fail(XPBD_ERR_INVALID_ARGUMENT, "params is NULL");
  if (p->constraints_iter < 0) return fail(XPBD_ERR_INVALID_ARGUMENT, "constraints_iter < 0");
  if (p->scatter != XPBD_SCATTER_ATOMIC && p->scatter != XPBD_SCATTER_GATHER)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown scatter variant");
  if (!(p->lame_mu != 0.f) || !(p->lame_lambda != 0.f))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "Lame parameters must be non-zero");
  return XPBD_OK;
}

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
void launch_project_t(Solver* s, float dt, cudaStream_t st) {
  const int g = blocks_for(s->d.T);
  const xpbd_params& p = s->prm;
  if (p.scatter == XPBD_SCATTER_GATHER)
    k_project<kBlockMode, kFirst, kPrecise, true><<<g, kBlock, 0, st>>>(
        s->d, s->cur, dt, p.lame_mu, p.lame_lambda, p.hydrostatic_relaxation, p.deviatoric_relaxation);
  else
    k_project<kBlockMode, kFirst, kPrecise, false><<<g, kBlock, 0, st>>>(
        s->d, s->cur, dt, p.lame_mu, p.lame_lambda, p.hydrostatic_relaxation, p.deviatoric_relaxation);
}

void launch_project(Solver* s, bool first, float dt, cudaStream_t st) {
  Prof prof(s, XPBD_K_PROJECT, st);
  const bool blk = s->prm.block_mode != 0, pr = s->prm.precise_hydro != 0;
  if (blk) {
    if (first) pr ? launch_project_t<true, true, true>(s, dt, st) : launch_project_t<true, true, false>(s, dt, st);
    else pr ? launch_project_t<true, false, true>(s, dt, st) : launch_project_t<true, false, false>(s, dt, st);
  } else {
    if (first) pr ? launch_project_t<false, true, true>(s, dt, st) : launch_project_t<false, true, false>(s, dt, st);
    else pr ? launch_project_t<false, false, true>(s, dt, st) : launch_project_t<false, false, false>(s, dt, st);
  }
}

template <bool kRes, bool kMon>
void launch_residual_t(Solver* s, const SweepArgs& a, int grid, cudaStream_t st) {
  if (s->prm.precise_hydro) k_residual<kRes, kMon, true><<<grid, kBlock, 0, st>>>(s->d, a);
  else k_residual<kRes, kMon, false><<<grid, kBlock, 0, st>>>(s->d, a);
}

// One Jacobi iteration (neohookean_solver.py:474-556).
void launch_iteration(Solver* s, int it, float dt, int rec, cudaStream_t st) {
  const xpbd_params& p = s->prm;
  launch_project(s, it == 0, dt, st);
  if (p.scatter == XPBD_SCATTER_GATHER) {
    Prof prof(s, XPBD_K_GATHER, st);
    k_gather<<<blocks_for(s->d.V), kBlock, 0, st>>>(s->d);
  }
  const bool cheb = p.cheb_enable != 0, mon = p.monitor != 0;
  if (cheb || mon) {
    SweepArgs a;
    a.cur = s->cur;
    a.dt = dt;
    a.mu = p.lame_mu;
    a.la = p.lame_lambda;
    a.it = it;
    a.warmup = p.cheb_warmup;
    a.rec = rec;
    a.rho_min = p.rho_min;
    a.rho_max = p.rho_max;
    a.rho_beta = p.rho_beta;
    int grid = blocks_for(s->d.T);
    const int cap = s->sm_count * 4;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    Prof prof(s, XPBD_K_RESIDUAL, st);
    if (cheb && mon) launch_residual_t<true, true>(s, a, grid, st);
    else if (cheb) launch_residual_t<true, false>(s, a, grid, st);
    else launch_residual_t<false, true>(s, a, grid, st);
  }
  const int g = blocks_for(s->d.V);
  const bool reset = p.scatter != XPBD_SCATTER_GATHER;
  Prof prof(s, XPBD_K_UPDATE, st);
  if (cheb) {
    if (it == 0) {
      if (reset) k_update<true, true, true><<<g, kBlock, 0, st>>>(s->d, s->cur, p.cheb_gamma);
      else k_update<true, true, false><<<g, kBlock, 0, st>>>(s->d, s->cur, p.cheb_gamma);
    } else {
      if (reset) k_update<true, false, true><<<g, kBlock, 0, st>>>(s->d, s->cur, p.cheb_gamma);
      else k_update<true, false, false><<<g, kBlock, 0, st>>>(s->d, s->cur, p.cheb_gamma);
    }
    s->cur ^= 1;
  } else {
    if (reset) k_update<false, false, true><<<g, kBlock, 0, st>>>(s->d, s->cur, p.cheb_gamma);
    else k_update<false, false, false><<<g, kBlock, 0, st>>>(s->d, s->cur, p.cheb_gamma);
  }
}

int do_solve_step(Solver* s, float dt, int record_base, cudaStream_t st) {
  const int K = s->prm.constraints_iter;
  if (record_base >= 0 && record_base + K > s->max_records)
    return fail(XPBD_ERR_HISTORY_FULL, "history holds " + std::to_string(s->max_records) + " records");
  launch_begin(s, false, true, dt, st);
  for (int it = 0; it < K; ++it) launch_iteration(s, it, dt, record_base >= 0 ? record_base + it : -1, st);
  return XPBD_OK;
}

int do_substep(Solver* s, float dt, int record_base, cudaStream_t st) {
  const int K = s->prm.constraints_iter;
  if (record_base >= 0 && record_base + K > s->max_records)
    return fail(XPBD_ERR_HISTORY_FULL, "history holds " + std::to_string(s->max_records) + " records");
  s->cur = 0;
  launch_begin(s, true, true, dt, st);
  for (int it = 0; it < K; ++it) launch_iteration(s, it, dt, record_base >= 0 ? record_base + it : -1, st);
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

void drop_graph(Solver* s) {
  if (s->exec) cudaGraphExecDestroy(s->exec);
  s->exec = nullptr;
  s->key = GraphKey();
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
      !body->dm_c || !body->lam)
    return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL body buffer");
  if (params->scatter == XPBD_SCATTER_GATHER && (!body->v2t_offsets || !body->v2t_slots || !body->corner_dx))
    return fail(XPBD_ERR_INVALID_ARGUMENT, "gather variant needs v2t_offsets, v2t_slots and corner_dx");
  if (max_records < 0) return fail(XPBD_ERR_INVALID_ARGUMENT, "max_records < 0");

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
  d.dm_c = reinterpret_cast<const float2*>(body->dm_c);
  d.lam = reinterpret_cast<float2*>(body->lam);
  d.v2t_off = body->v2t_offsets;
  d.v2t_slot = body->v2t_slots;
  d.corner = reinterpret_cast<float4*>(body->corner_dx);
  d.perm = body->vert_perm;
  d.n_sdf = n_sdf;
  s->max_records = max_records;

  auto cleanup = [&](int status) {
    if (d.sdfs) cudaFree(const_cast<xpbd_sdf*>(d.sdfs));
    if (d.st) cudaFree(d.st);
    if (d.hist) cudaFree(d.hist);
    if (s->cap) cudaStreamDestroy(s->cap);
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
  if (e != cudaSuccess) return cleanup(fail(XPBD_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e)));
  DevState h{};
  h.rho_hat = 0.999;  // neohookean_solver.py:65
  h.omega = 1.0;
  e = cudaMemcpy(d.st, &h, sizeof(h), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d.hist, 0, sizeof(double) * 4 * (size_t)(max_records > 0 ? max_records : 1));
  if (e != cudaSuccess) return cleanup(fail(XPBD_ERR_CUDA, std::string("setup: ") + cudaGetErrorString(e)));
  // validate the mesh indices once, before any kernel gathers through them
  const int nval = (d.T > d.V + 1 ? d.T : d.V + 1);
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
  if (std::memcmp(&s->prm, params, sizeof(xpbd_params)) != 0) drop_graph(s);
  s->prm = *params;
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
  if (!s->prm.use_graph || s->profiling) {
    int r = enqueue_frame(s, frame_dt, dt, substeps, S(stream));
    if (r != XPBD_OK) return r;
    XPBD_CUDA(cudaGetLastError());
    return XPBD_OK;
  }
  if (!(s->exec && s->key.frame_dt == frame_dt && s->key.dt == dt && s->key.substeps == substeps)) {
    drop_graph(s);
    XPBD_CUDA(cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal));
    int r = enqueue_frame(s, frame_dt, dt, substeps, s->cap);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s->cap, &g);
    if (r != XPBD_OK) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    if (e != cudaSuccess) return fail(XPBD_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      s->exec = nullptr;
      return fail(XPBD_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
    }
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

int xpbd_read_profile(void* handle, double* ms, int64_t* launches, int32_t n, int32_t reset, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || n < 0 || n > XPBD_K_COUNT) return fail(XPBD_ERR_INVALID_ARGUMENT, "bad profile read");
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
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

static float4* field_ptr(Solver* s, int32_t field) {
  switch (field) {
    case XPBD_FIELD_X: return s->d.x;
    case XPBD_FIELD_V: return s->d.v;
    case XPBD_FIELD_PRED_X: return s->d.p[s->cur];
    default: return nullptr;
  }
}

int xpbd_import_vec3(void* handle, int32_t field, const float* src, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !src) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or source");
  float4* f = field_ptr(s, field);
  if (!f) return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown field");
  k_import<<<blocks_for(s->d.V), kBlock, 0, S(stream)>>>(s->d, f, src);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_export_vec3(void* handle, int32_t field, float* dst, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s || !dst) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle or destination");
  float4* f = field_ptr(s, field);
  if (!f) return fail(XPBD_ERR_INVALID_ARGUMENT, "unknown field");
  k_export<<<blocks_for(s->d.V), kBlock, 0, S(stream)>>>(s->d, f, dst);
  XPBD_CUDA(cudaGetLastError());
  return XPBD_OK;
}

int xpbd_check_status(void* handle, void* stream) {
  Solver* s = static_cast<Solver*>(handle);
  if (!s) return fail(XPBD_ERR_INVALID_ARGUMENT, "NULL handle");
  int flag = 0;
  XPBD_CUDA(cudaMemcpyAsync(&flag, &s->d.st->nonfinite, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
  XPBD_CUDA(cudaStreamSynchronize(S(stream)));
  return flag ? fail(XPBD_ERR_NONFINITE, "non-finite residual") : XPBD_OK;
}

}  // extern "C"

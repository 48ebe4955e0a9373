// Device-side math of the RDC-XPBD substep: tet kinematics, the Neo-Hookean
// constraint pair, the 2x2 pivoted LU and the SDF obstacles.  FP32 throughout
// (the reference's arithmetic type); callers reduce in FP64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/xpbd_gb300.h"

namespace xpbd {

// xpbd_gpu/constants.py:3
constexpr float kEps = 1e-12f;

struct Tet {
  float4 p[4];    // gathered predicted positions, w = inv_m
  float dm[9];    // inv_Dm row-major
  float V0;
};

// F = Ds * inv_Dm with Ds = [p1-p0, p2-p0, p3-p0] as columns
// (neohookean_solver.py:371-373).  F[r*3+c].
__device__ __forceinline__ void deformation_gradient(const Tet& t, float F[9]) {
  const float e[3][3] = {
      {t.p[1].x - t.p[0].x, t.p[2].x - t.p[0].x, t.p[3].x - t.p[0].x},
      {t.p[1].y - t.p[0].y, t.p[2].y - t.p[0].y, t.p[3].y - t.p[0].y},
      {t.p[1].z - t.p[0].z, t.p[2].z - t.p[0].z, t.p[3].z - t.p[0].z}};
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      F[r * 3 + c] = e[r][0] * t.dm[0 * 3 + c] + e[r][1] * t.dm[1 * 3 + c] + e[r][2] * t.dm[2 * 3 + c];
}

// C_D = tr(F^T F) - 3 and C_H = det F - 1 (neohookean_solver.py:376-380).
// kPrecise evaluates both through G = F - I:
//   tr(F^T F) - 3 = 2 tr G + |G|^2,
//   det(I + G) - 1 = tr G + (sum of principal 2x2 minors of G) + det G,
// which avoids the cancellation against 3 and 1 when F is near a rotation-free
// isochoric state (nu -> 0.5).
template <bool kPrecise>
__device__ __forceinline__ void invariants(const float F[9], float& C_D, float& C_H) {
  if (kPrecise) {
    const float g00 = F[0] - 1.f, g11 = F[4] - 1.f, g22 = F[8] - 1.f;
    const float g01 = F[1], g02 = F[2], g10 = F[3], g12 = F[5], g20 = F[6], g21 = F[7];
    const float tr = g00 + g11 + g22;
    const float gg = g00 * g00 + g01 * g01 + g02 * g02 + g10 * g10 + g11 * g11 + g12 * g12 +
                     g20 * g20 + g21 * g21 + g22 * g22;
    C_D = 2.f * tr + gg;
    const float m2 = (g00 * g11 - g01 * g10) + (g00 * g22 - g02 * g20) + (g11 * g22 - g12 * g21);
    const float detG = g00 * (g11 * g22 - g21 * g12) - g10 * (g01 * g22 - g21 * g02) +
                       g20 * (g01 * g12 - g11 * g02);
    C_H = tr + (m2 + detG);
  } else {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 9; ++i) s += F[i] * F[i];
    C_D = s - 3.f;
    // cofactor expansion along the first column
    const float det = F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
                      F[6] * (F[1] * F[5] - F[4] * F[2]);
    C_H = det - 1.f;
  }
}

// Corner gradients g_{c+1}[r] = sum_k gradF[r][k] * inv_Dm[c][k]
// (grad123 = gradF * inv_Dm^T, neohookean_solver.py:382-404); g0 = -(g1+g2+g3).
__device__ __forceinline__ void corner_gradients(const float gF[9], const float dm[9], float3 g[4]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    g[c + 1].x = gF[0] * dm[c * 3 + 0] + gF[1] * dm[c * 3 + 1] + gF[2] * dm[c * 3 + 2];
    g[c + 1].y = gF[3] * dm[c * 3 + 0] + gF[4] * dm[c * 3 + 1] + gF[5] * dm[c * 3 + 2];
    g[c + 1].z = gF[6] * dm[c * 3 + 0] + gF[7] * dm[c * 3 + 1] + gF[8] * dm[c * 3 + 2];
  }
  g[0].x = -(g[1].x + g[2].x + g[3].x);
  g[0].y = -(g[1].y + g[2].y + g[3].y);
  g[0].z = -(g[1].z + g[2].z + g[3].z);
}

// dC_H/dF = [F1 x F2, F2 x F0, F0 x F1] as columns (neohookean_solver.py:391-398).
__device__ __forceinline__ void cofactor(const float F[9], float H[9]) {
  // column j of F: (F[j], F[3+j], F[6+j])
  const float3 c0 = make_float3(F[0], F[3], F[6]);
  const float3 c1 = make_float3(F[1], F[4], F[7]);
  const float3 c2 = make_float3(F[2], F[5], F[8]);
  const float3 x0 = make_float3(c1.y * c2.z - c1.z * c2.y, c1.z * c2.x - c1.x * c2.z, c1.x * c2.y - c1.y * c2.x);
  const float3 x1 = make_float3(c2.y * c0.z - c2.z * c0.y, c2.z * c0.x - c2.x * c0.z, c2.x * c0.y - c2.y * c0.x);
  const float3 x2 = make_float3(c0.y * c1.z - c0.z * c1.y, c0.z * c1.x - c0.x * c1.z, c0.x * c1.y - c0.y * c1.x);
  H[0] = x0.x; H[1] = x1.x; H[2] = x2.x;
  H[3] = x0.y; H[4] = x1.y; H[5] = x2.y;
  H[6] = x0.z; H[7] = x1.z; H[8] = x2.z;
}

__device__ __forceinline__ float dot3(const float3 a, const float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// solve2x2_pivot_lu (neohookean_solver.py:331-356); returns ok.  The
// elimination A11 - m A01 rounds the product before the subtraction (no fused
// multiply-add): for a stiff material the geometric part of the block is
// nearly singular (grad C_D ~ 2 grad C_H near F = I), and the fused form loses
// the small remainder that the compliance leaves -- on the reference's cow at
// E 5e8 it took the FP32 result 1e-3 of the diagonal from FP64 within five
// iterations, against 1e-6 with the product rounded.
__device__ __forceinline__ bool solve2x2_pivot_lu(float A00, float A01, float A10, float A11, float b0, float b1,
                                                  float& x0, float& x1) {
  if (fabsf(A00) < fabsf(A10)) {
    float t = A00; A00 = A10; A10 = t;
    t = A01; A01 = A11; A11 = t;
    t = b0; b0 = b1; b1 = t;
  }
  x0 = 0.f;
  x1 = 0.f;
  if (fabsf(A00) < kEps) return false;
  const float m = A10 / A00;
  const float A11_ = A11 - __fmul_rn(m, A01);
  const float b1_ = b1 - m * b0;
  if (fabsf(A11_) < kEps) return false;
  x1 = b1_ / A11_;
  x0 = (b0 - A01 * x1) / A00;
  return true;
}

// One tet of solve_neohookean_block (neohookean_solver.py:358-451) when
// kBlockMode, else of the split pair solve_hydrostatic + solve_deviatoric
// (:196-254, :144-194), both reading the same predicted positions.  Updates L
// = (lambda_D, lambda_H) and returns the four corner displacements and the
// constraint count added to each corner.
// aD, aH: the time-scaled compliances alpha / dt^2 of the tet (:413-416).
template <bool kBlockMode, bool kPrecise>
__device__ __forceinline__ void project_tet(const Tet& tt, float aD, float aH, float relax_h, float relax_d, float2& L,
                                            float3 dp[4], float& cnt) {
  const float w[4] = {tt.p[0].w, tt.p[1].w, tt.p[2].w, tt.p[3].w};
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

  if (kBlockMode) {
    float A11 = w[0] * dot3(gD[0], gD[0]) + w[1] * dot3(gD[1], gD[1]) + w[2] * dot3(gD[2], gD[2]) +
                w[3] * dot3(gD[3], gD[3]);
    float A22 = w[0] * dot3(gH[0], gH[0]) + w[1] * dot3(gH[1], gH[1]) + w[2] * dot3(gH[2], gH[2]) +
                w[3] * dot3(gH[3], gH[3]);
    const float A12 = w[0] * dot3(gD[0], gH[0]) + w[1] * dot3(gD[1], gH[1]) + w[2] * dot3(gD[2], gH[2]) +
                      w[3] * dot3(gD[3], gH[3]);
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
    L.x += dD;
    L.y += dH;
#pragma unroll
    for (int c = 0; c < 4; ++c)
      dp[c] = make_float3(w[c] * (gD[c].x * dD + gH[c].x * dH), w[c] * (gD[c].y * dD + gH[c].y * dH),
                          w[c] * (gD[c].z * dD + gH[c].z * dH));
    cnt = 1.f;  // :448-451 count every corner
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
      const float at = aH;
      dlH = -(C_H + at * L.y) / (wsH + at);
      dlH *= relax_h;
      cH = 1.f;
    }
    if (wsD > kEps) {
      const float at = aD;
      dlD = -(C_D + at * L.x) / (wsD + at);
      dlD *= relax_d;
      cD = 1.f;
    }
    L.x += dlD;
    L.y += dlH;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float sH = dlH * w[c], sD = dlD * w[c];
      dp[c] = make_float3(sH * gH[c].x + sD * gD[c].x, sH * gH[c].y + sD * gD[c].y, sH * gH[c].z + sD * gD[c].z);
    }
    cnt = cH + cD;
  }
}

// ---------------------------------------------------------------------------
// SDFs (sdf.py)
// ---------------------------------------------------------------------------

__device__ __forceinline__ float sdf_dist(const xpbd_sdf& s, const float3 p) {
  if (s.kind == XPBD_SDF_PLANE) {  // sdf.py:68-70
    return (p.x - s.a[0]) * s.b[0] + (p.y - s.a[1]) * s.b[1] + (p.z - s.a[2]) * s.b[2];
  }
  if (s.kind == XPBD_SDF_SPHERE) {  // sdf.py:86-88
    const float dx = p.x - s.a[0], dy = p.y - s.a[1], dz = p.z - s.a[2];
    return sqrtf(dx * dx + dy * dy + dz * dz) - s.b[0];
  }
  // XPBD_SDF_CUBE, sdf.py:107-110
  const float dx = fabsf(p.x - s.a[0]) - s.b[0];
  const float dy = fabsf(p.y - s.a[1]) - s.b[1];
  const float dz = fabsf(p.z - s.a[2]) - s.b[2];
  const float mx = fmaxf(dx, 0.f), my = fmaxf(dy, 0.f), mz = fmaxf(dz, 0.f);
  return sqrtf(mx * mx + my * my + mz * mz) + fminf(fmaxf(dx, fmaxf(dy, dz)), 0.f);
}

__device__ __forceinline__ float3 sdf_normal(const xpbd_sdf& s, const float3 p) {
  if (s.kind == XPBD_SDF_PLANE) return make_float3(s.b[0], s.b[1], s.b[2]);  // sdf.py:72-74
  const float dx = p.x - s.a[0], dy = p.y - s.a[1], dz = p.z - s.a[2];
  if (s.kind == XPBD_SDF_SPHERE) {  // sdf.py:90-92: v * 1 / (|v| + eps)
    const float inv = 1.f / (sqrtf(dx * dx + dy * dy + dz * dz) + kEps);
    return make_float3(dx * inv, dy * inv, dz * inv);
  }
  // sdf.py:112-124: sign of the dominant axis of (p - c)
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int axis = 0;
  float amax = ax;
  if (ay > ax) { axis = 1; amax = ay; }
  if (az > amax) axis = 2;
  float3 n = make_float3(0.f, 0.f, 0.f);
  if (axis == 0) n.x = dx > 0.f ? 1.f : -1.f;
  else if (axis == 1) n.y = dy > 0.f ? 1.f : -1.f;
  else n.z = dz > 0.f ? 1.f : -1.f;
  return n;
}

// _solve_sdf_collision_one + SdfModel.check (xpbd_base.py:162-174, sdf.py:14-27)
// for one live vertex; SDFs are applied sequentially in list order.
__device__ __forceinline__ void sdf_project_all(const xpbd_sdf* __restrict__ sdfs, int n_sdf, float3& p,
                                                const float3 vel) {
  for (int s = 0; s < n_sdf; ++s) {
    const xpbd_sdf sd = sdfs[s];
    const float phi = sdf_dist(sd, p);
    if (phi < 0.f) {
      const float3 n = sdf_normal(sd, p);
      const float dotnv = n.x * (sd.vel[0] - vel.x) + n.y * (sd.vel[1] - vel.y) + n.z * (sd.vel[2] - vel.z);
      if (dotnv > 0.f || sd.fixed) {
        const float pen = -sdf_dist(sd, p);
        if (pen > 0.f) {
          p.x += n.x * pen;
          p.y += n.y * pen;
          p.z += n.z * pen;
        }
      }
    }
  }
}

// Programmatic dependent launch (sm_90+).  A kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may start while its
// predecessor in the stream drains.  pdl_wait() returns once the predecessor
// has completed and its writes are visible (without the attribute it returns
// at once); pdl_trigger() lets the successor launch.  Every kernel of such a
// chain waits before it triggers, so when a kernel starts, every kernel
// before its immediate predecessor has completed: what those wrote may be
// read before pdl_wait().
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launch `k` on `st`; with `overlap` it may start while its predecessor in the
// stream drains (programmatic dependent launch: the kernel calls pdl_wait()
// before it reads what the predecessor writes).
template <typename... KArgs, typename... Args>
inline void launch_k(void (*k)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, bool overlap, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = overlap ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// Vector reduction into global memory: red.global.add.v4.f32 (sm_90+).
__device__ __forceinline__ void red_add_v4(float4* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

// L2 eviction priority for read-only tet records.  With `keep` the records
// are loaded evict_last, so a mesh whose records fit in L2 keeps them there
// from one sweep to the next instead of losing them to the position and
// accumulator traffic; otherwise evict_normal (a plain load).
__device__ __forceinline__ uint64_t l2_policy(bool keep) {
  uint64_t pol;
  if (keep)
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  else
    asm("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

__device__ __forceinline__ float4 ldg_hint(const float4* p, uint64_t pol) {
  float4 r;
  asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
      : "l"(p), "l"(pol));
  return r;
}

__device__ __forceinline__ float ldg_hint(const float* p, uint64_t pol) {
  float r;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(r) : "l"(p), "l"(pol));
  return r;
}

__device__ __forceinline__ uint32_t ldg_hint(const uint32_t* p, uint64_t pol) {
  uint32_t r;
  asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  return r;
}

__device__ __forceinline__ int ldg_hint(const int* p, uint64_t pol) {
  int r;
  asm("ld.global.nc.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(r) : "l"(p), "l"(pol));
  return r;
}

// The records of two consecutive tets (t even: float4 pairs 32-byte aligned,
// scalar pairs 8-byte aligned) in one load per array.  With two tets per
// thread, loading t and t + 1 separately makes each warp instruction touch
// every other 16 bytes of a 1 KiB span, so a warp reads each sector through
// L1 twice; the 256-bit load (sm_100+) reads it once.
__device__ __forceinline__ void ldg_pair(const float4* p, uint64_t pol, float4& a, float4& b) {
  asm("ld.global.nc.L2::cache_hint.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8], %9;"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p), "l"(pol));
}

__device__ __forceinline__ void ldg_pair(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

__device__ __forceinline__ float2 ldg_pair(const float* p, uint64_t pol) {
  float2 r;
  asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(r.x), "=f"(r.y) : "l"(p), "l"(pol));
  return r;
}

__device__ __forceinline__ uint2 ldg_pair(const uint32_t* p, uint64_t pol) {
  uint2 r;
  asm("ld.global.nc.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(r.x), "=r"(r.y) : "l"(p), "l"(pol));
  return r;
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies (TMA, cp.async.bulk) tracked by an mbarrier.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Bounded wait for phase `parity` of an mbarrier: true when it completed,
// false after `max_polls` polls (the caller records the timeout).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int max_polls) {
  const uint32_t a = smem_addr(bar);
  for (int i = 0; i < max_polls; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Ampere-style asynchronous 16-byte copies global -> shared (L2 only), grouped.
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// det of a row-major 3x3 (cofactor expansion along the first column); for
// inv_Dm it is 1 / det(Dm) = 1 / (6 V0) with the sign of the rest volume.
__device__ __forceinline__ float det9(const float m[9]) {
  return m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) + m[6] * (m[1] * m[5] - m[4] * m[2]);
}

// Resident CTAs per SM the tile projections are compiled for, by tets per
// thread: with 2, 9 CTAs of 128 threads cap a thread at 56 registers.  The
// chain needs 72 without spills, but the few spilled bytes (16-24 per
// thread) cost less than the latency that two more CTAs hide: on a 64^3-cell
// Kuhn cube (1.57 M tets) the projection measured 37.5 us at 7 CTAs, 36.5 at
// 8 and 35.7 at 9; 10 CTAs
// (48 registers) spill 60-84 bytes.  Otherwise no minimum.
__host__ __device__ constexpr int project_min_blocks(int tpt) { return tpt == 2 ? 9 : 1; }

__device__ __forceinline__ void add4(float4& a, const float4 b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  a.w += b.w;
}

// Tile projection of kTPT consecutive tets of one thread (records
// A, B, C, lid; multipliers L, stored to lam_out[k] as each tet is done), n of
// them valid.  Vertex
// positions come from the patch tile sp (global ids sg).  Consecutive tets of
// a patch usually share a face, so the previous tet's four corner sums stay in
// registers: a corner of the next tet that matches one is added there, and a
// held corner the next tet does not touch is flushed with red.global.add.v4.
// A chain of kTPT tets sharing s corners per step issues 4 + (kTPT - 1)(4 - s)
// reductions instead of 4 kTPT.  A face pair laid out by xpbd_pair_tets (the
// second tet's corners 0, 1, 2 are the first's 1, 0, 2, recognised from the
// packed patch-local ids) merges its three shared corners without comparisons.  cD, cH: time-scaled inverse Lame parameters;
// the tet's compliances are 6 det(inv_Dm) cD and 6 det(inv_Dm) cH (1 / V0).
// kTetMat: per-tet materials, the compliances are further multiplied by the
// tet's 1 / mu and 1 / lambda (mD[k], mH[k]).  lam_in (taping): the
// multipliers entering the iteration are also stored there.
template <bool kBlockMode, bool kPrecise, int kTPT, bool kTetMat = false>
__device__ __forceinline__ void project_chain(const float4 (&A)[kTPT], const float4 (&B)[kTPT], const float (&C)[kTPT],
                                              const uint32_t (&lid)[kTPT], float2 (&L)[kTPT], float2* lam_out,
                                              int n, const float4* sp, const int* sg, float4* dx, float cD,
                                              float cH, float relax_h, float relax_d, bool paired,
                                              const float* mD = nullptr, const float* mH = nullptr,
                                              float2* lam_in = nullptr) {
  float4 acc[4];
  int hid[4] = {-1, -1, -1, -1};
#pragma unroll
  for (int k = 0; k < kTPT; ++k) {
    if (k >= n) break;
    Tet tt;
    tt.dm[0] = A[k].x; tt.dm[1] = A[k].y; tt.dm[2] = A[k].z;
    tt.dm[3] = A[k].w; tt.dm[4] = B[k].x; tt.dm[5] = B[k].y;
    tt.dm[6] = B[k].z; tt.dm[7] = B[k].w; tt.dm[8] = C[k];
    int id[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      id[c] = (int)((lid[k] >> (8 * c)) & 0xffu);
      tt.p[c] = sp[id[c]];
    }
    const float six_det = 6.f * det9(tt.dm);
    float3 dp[4];
    float cnt;
    if (lam_in) lam_in[k] = L[k];
    if (kTetMat)
      project_tet<kBlockMode, kPrecise>(tt, six_det * (cD * mD[k]), six_det * (cH * mH[k]), relax_h, relax_d, L[k],
                                        dp, cnt);
    else
      project_tet<kBlockMode, kPrecise>(tt, six_det * cD, six_det * cH, relax_h, relax_d, L[k], dp, cnt);
    lam_out[k] = L[k];
    float4 nacc[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) nacc[c] = make_float4(dp[c].x, dp[c].y, dp[c].z, cnt);
    if (paired && (k & 1)) {
      // Two-tet unit of xpbd_pair_tets (paired is uniform over the grid).  A
      // face pair has aligned corners: corners 0, 1, 2 of this tet are corners
      // 1, 0, 2 of the held one, and corner 3 is flushed.  Any other unit
      // flushes all four held corners unmerged.
      if ((lid[k] & 0xffffffu) == (__byte_perm(lid[k - 1], 0u, 0x3201u) & 0xffffffu)) {
        add4(nacc[0], acc[1]);
        add4(nacc[1], acc[0]);
        add4(nacc[2], acc[2]);
        red_add_v4(dx + sg[hid[3]], acc[3].x, acc[3].y, acc[3].z, acc[3].w);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) red_add_v4(dx + sg[hid[q]], acc[q].x, acc[q].y, acc[q].z, acc[q].w);
      }
    } else {
      // Held corners: merge into the matching new corner, or flush.  A tet's
      // corners are distinct vertices, so a held corner matches at most one.
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        bool used = false;
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (hid[q] == id[c]) {
            add4(nacc[c], acc[q]);
            used = true;
          }
        if (hid[q] >= 0 && !used) red_add_v4(dx + sg[hid[q]], acc[q].x, acc[q].y, acc[q].z, acc[q].w);
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      acc[c] = nacc[c];
      hid[c] = id[c];
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (hid[q] >= 0) red_add_v4(dx + sg[hid[q]], acc[q].x, acc[q].y, acc[q].z, acc[q].w);
}

}  // namespace xpbd

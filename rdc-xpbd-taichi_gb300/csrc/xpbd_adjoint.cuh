// Adjoint (reverse-mode) kernels of one block Neo-Hookean substep.
//
// The forward substep is recomputed from a per-substep checkpoint with its
// intermediate states recorded on a tape (predicted positions before every
// Jacobi iteration, the multipliers entering it, the predicted positions
// before the SDF list and the velocities after gravity); the kernels below
// then run the substep backwards:
//   ka_end      advance            (xpbd_base.py:148-160)
//   per iteration k = K-1 .. 0:
//     ka_cheb   Chebyshev mix + post_solve (neohookean_solver.py:115-142, :548)
//     ka_project block projection: Jacobian-transpose of F -> (C, grad C) ->
//                2x2 compliance solve -> dx (:358-451), with the material
//                adjoints accumulated per tet in FP64
//   ka_begin    SDF list in reverse order + predict (xpbd_base.py:139-178)
// Conventions: the contact sets and the pivot branch are piecewise constant;
// the derivative of the 2x2 solve is that of A^-1 b.  Omega is a
// stop-gradient unless the tape holds the post-Jacobi positions (Tape::posts)
// and the adjoint an omega state (Adj::om): then
//     ka_chain         replays the substep's rho_hat curve into a table of
//                      per-iteration chain coefficients (FP64, one warp per
//                      body; neohookean_solver.py:495-504, :537-546)
//     ka_cheb          also sums omega_k's adjoint over the vertices
// and, between ka_cheb and the tet adjoint of each iteration,
//     ka_residual_adj  steps the omega_k -> rho_hat_k -> r_hat_k chain (every
//                      CTA for its body; one CTA per body stores the state)
//                      and takes r_hat_k's adjoint to the post-Jacobi
//                      positions, the multipliers after the iteration and the
//                      compliances (:298-329).
//
// The kernels are templates over the solver's device view D (the single-body
// and the batched layouts).  Each layout provides, next to its own type so
// that argument-dependent lookup finds them:
//   int   adj_verts(const D&), adj_tets(const D&)   vertex and tet slots
//   bool  adj_load_tet(const D&, int t, int vid[4], Tet&, float& inv_v0,
//                      float& m_mu, float& m_la)   false for a padding slot;
//         m_mu, m_la multiply the compliance factors (the tet's 1/mu and
//         1/lambda with per-tet materials, else 1); only ka_project needs it
//         (a layout with its own tet kernel calls tet_adjoint directly)
//   float adj_omega(const D&, int i, int k)          omega of vertex i's body
//                                                    at iteration k
// and the members x, v, sdfs, n_sdf.  The omega chain also needs
//   int    adj_nbodies(const D&)                    bodies (Chebyshev states)
//   int    adj_vbody(const D&, int i)               body of vertex i
//   double adj_hist(const D&, int b, int k, int c)  history row k of body b
//   double adj_body_tets(const D&, int b)           real tets of body b
#pragma once

namespace xpbd {

struct Tape {
  float4* xs;    // [(K+1)][V] predicted positions entering iteration k (w = inv_m)
  float2* lams;  // [K][T] multipliers entering iteration k ([K+1] with posts: and after the last)
  float4* xpre;  // [V] predicted positions before the SDF list
  float4* v1;    // [V] velocities after gravity
  float4* posts;  // [K][V] post-Jacobi positions of iteration k; nullptr: omega is a stop-gradient
  double* rho_in; // [bodies] rho_hat entering the substep (with posts)
};

// Omega chain state per body (Adj::om), om_stride(K) = 8 + 6 K doubles.  Pairs
// indexed by the iteration's parity (iteration k reads [k & 1] and writes
// [(k & 1) ^ 1]): the adjoint of omega_k summed over the vertices (ka_cheb),
// the adjoints of omega_k and r_hat_k passed down from iteration k + 1, and
// the adjoint of rho_hat (it persists across substeps: zero the state before
// a backward pass).  Then per iteration k a row of coefficients (kTab + 6 k):
//   1 / omega_k, d omega_k / d rho_hat_k, d omega_k / d omega_{k-1},
//   the rho_hat update weight beta (0 where rho_hat was not updated),
//   d ratio_k / d r_hat_k and d ratio_k / d r_hat_{k-1} (0 where clamped).
enum { kOmSum = 0, kOmCarry = 2, kRCarry = 4, kRhoBar = 6, kTab = 8, kTabRow = 6 };
__host__ __device__ __forceinline__ int om_stride(int K) { return kTab + kTabRow * K; }

struct Adj {
  float4* gx;        // [V] in: dL/dx at the end of the substep, out: at its start
  float4* gv;        // [V] in / out, likewise for v
  double* g_mu;      // [T] accumulated dL/d(1/mu)
  double* g_la;      // [T] accumulated dL/d(1/lambda)
  float4* abuf[2];   // [V] adjoint of the predicted positions (ping-pong)
  float4* ybar;      // [V] adjoint of the Chebyshev y_prev
  float4* dxbar;     // [V] adjoint of the Jacobi accumulator
  float2* lambar;    // [T] adjoint of the multipliers
  const float* cnt;  // [V] constraints per vertex (valence in block mode)
  double* om;        // [bodies][om_stride(K)] omega chain state; nullptr: omega is a stop-gradient
  int om_n;          // om_stride(K)
  // Batched layout with the omega chain: [T] the residual adjoint's multiplier
  // and material parts (lambda_{k+1}, 1/mu, 1/lambda) of every tet, read by the
  // tet adjoint.  nullptr in the single-body layout, whose residual adjoint
  // adds them in place.
  float4* rtet;
};

__device__ __forceinline__ float3 f3(const float4 a) { return make_float3(a.x, a.y, a.z); }
// abuf[k] for a run-time k without indexing the kernel-parameter array (which
// would copy the whole Adj parameter block to local memory)
__device__ __forceinline__ float4* adj_buf(const Adj& a, int k) { return k ? a.abuf[1] : a.abuf[0]; }

__device__ __forceinline__ float3 cross3(const float3 a, const float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Velocities after gravity and predicted positions before the SDF list.
template <class D>
__global__ void __launch_bounds__(256) k_tape_begin(D d, Tape tp, float dt, float gx, float gy, float gz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= adj_verts(d)) return;
  const float4 xi = d.x[i];
  float4 vi = d.v[i];
  if (xi.w > 0.f) {
    vi.x += gx * dt;
    vi.y += gy * dt;
    vi.z += gz * dt;
  }
  tp.v1[i] = vi;
  tp.xpre[i] = make_float4(xi.x + vi.x * dt, xi.y + vi.y * dt, xi.z + vi.z * dt, xi.w);
}

struct ChainPrm {
  int K, warmup;
  double rho_min, rho_max, beta;
};

// Start of the omega chain of a substep (one warp per body): carries the
// adjoint of rho_hat over from the later substep, clears the other state and
// tabulates the coefficients of every iteration.  Lane j takes iteration j
// (32 at a time): the ratio r_hat_j / r_hat_{j-1}, its clamp and the rho_hat
// update are independent per iteration except for rho_hat_j = a_j rho_hat_{j-1}
// + b_j, which is an inclusive scan of affine maps across the lanes.
template <class D>
__global__ void __launch_bounds__(256) ka_chain(D d, Tape tp, Adj a, ChainPrm c) {
  const int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= adj_nbodies(d)) return;  // warp-uniform
  const unsigned full = 0xffffffffu;
  double* o = a.om + (size_t)a.om_n * b;
  if (lane == 0) {
    // the adjoint of rho_hat entering the later substep (written by its
    // iteration 0 into slot 1) is that of rho_hat leaving this one
    o[kRhoBar + ((c.K - 1) & 1)] = o[kRhoBar + 1];
    o[kOmSum] = o[kOmSum + 1] = o[kOmCarry] = o[kOmCarry + 1] = o[kRCarry] = o[kRCarry + 1] = 0.0;
  }
  double rho_prev = tp.rho_in[b];
  for (int j0 = 0; j0 < c.K; j0 += 32) {
    const int j = j0 + lane;
    const bool in = j < c.K;
    double r = 0.0, prev = 0.0, om = 1.0, om_prev = 1.0;
    if (in) {
      r = adj_hist(d, b, j, 0);
      om = adj_hist(d, b, j, 1);
      if (j > 0) {
        prev = adj_hist(d, b, j - 1, 0);
        om_prev = adj_hist(d, b, j - 1, 1);
      }
    }
    const bool upd = in && j > 0 && prev > 1e-12;
    double ri = 0.0, c1 = 0.0, c2 = 0.0;
    if (upd) {
      const double dd = prev + 1e-12;
      const double ratio = r / dd;
      ri = fmax(c.rho_min, fmin(c.rho_max, ratio));
      if (ri == ratio) {
        c1 = 1.0 / dd;
        c2 = -ratio / dd;
      }
    }
    double ma = upd ? 1.0 - c.beta : 1.0, mb = upd ? c.beta * ri : 0.0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const double pa = __shfl_up_sync(full, ma, off), pb = __shfl_up_sync(full, mb, off);
      if (lane >= off) {
        mb = ma * pb + mb;
        ma = ma * pa;
      }
    }
    const double rho = ma * rho_prev + mb;
    rho_prev = __shfl_sync(full, rho, 31);
    double A = 0.0, B = 0.0;
    if (j == c.warmup) {
      const double den = 2.0 - rho * rho;
      A = 4.0 * rho / (den * den);
    } else if (j > c.warmup) {
      const double den = 4.0 - rho * rho * om_prev;
      A = 8.0 * rho * om_prev / (den * den);
      B = 4.0 * rho * rho / (den * den);
    }
    if (in) {
      double* t = o + kTab + kTabRow * j;
      t[0] = 1.0 / om;
      t[1] = A;
      t[2] = B;
      t[3] = upd ? c.beta : 0.0;
      t[4] = c1;
      t[5] = c2;
    }
  }
}

// Reverse of advance: live vertices x' = x~_K, v' = (x~_K - x) e / dt; pinned
// vertices keep x and v.
template <class D>
__global__ void __launch_bounds__(256) ka_end(D d, Adj a, float e_over_dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= adj_verts(d)) return;
  const float4 gx = a.gx[i], gv = a.gv[i];
  if (d.x[i].w > 0.f) {
    a.abuf[0][i] = make_float4(gx.x + gv.x * e_over_dt, gx.y + gv.y * e_over_dt, gx.z + gv.z * e_over_dt, 0.f);
    a.gx[i] = make_float4(-gv.x * e_over_dt, -gv.y * e_over_dt, -gv.z * e_over_dt, 0.f);
    a.gv[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  } else {
    a.abuf[0][i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  a.ybar[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Reverse of the Chebyshev mix and post_solve of iteration k:
//   post = x~_k + dx / cnt,  xn = gamma (post - x~_k) + x~_k,
//   x~_{k+1} = y_prev + omega (xn - y_prev),  y_prev(k+1) = x~_k,
// with y_prev(0) = x~_0.  Reads abuf[src] (adjoint of x~_{k+1}), writes
// abuf[src^1] (direct part of the adjoint of x~_k), ybar and dxbar.
template <class D, bool kCheb>
__global__ void __launch_bounds__(256) ka_cheb(D d, Tape tp, Adj a, int k, float gamma, int src) {
  pdl_wait();  // x~_{k+1}'s adjoint from the tet adjoint before it
  pdl_trigger();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float4 xb = i < adj_verts(d) ? adj_buf(a, src)[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  if (kCheb && a.om) {
    // omega_k's adjoint: sum over the vertices of x~bar_{k+1} . (xn - y_prev),
    // with xn - y_prev = (x~_{k+1} - y_prev) / omega_k (divided in chain_step).  A
    // CTA covers 256 vertices of one body.
    // FP32 within a warp, FP64 across warps and CTAs
    float part = 0.f;
    if (i < adj_verts(d)) {
      const size_t V = (size_t)adj_verts(d);
      const float4 x1 = tp.xs[(size_t)(k + 1) * V + i], y = tp.xs[(size_t)(k > 0 ? k - 1 : 0) * V + i];
      part = xb.x * (x1.x - y.x) + xb.y * (x1.y - y.y) + xb.z * (x1.z - y.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    __shared__ float s_part[8];
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
      double sum = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) sum += (double)s_part[w];
      const int i0 = blockIdx.x * blockDim.x;
      if (i0 < adj_verts(d)) atomicAdd(a.om + (size_t)a.om_n * adj_vbody(d, i0) + kOmSum + (k & 1), sum);
    }
  }
  if (i >= adj_verts(d)) return;
  float3 post, cur, yn;
  if (kCheb) {
    const float om = adj_omega(d, i, k);
    const float4 yb = a.ybar[i];
    post = make_float3(om * gamma * xb.x, om * gamma * xb.y, om * gamma * xb.z);
    const float c = om * (1.f - gamma);
    cur = make_float3(c * xb.x + post.x + yb.x, c * xb.y + post.y + yb.y, c * xb.z + post.z + yb.z);
    yn = make_float3((1.f - om) * xb.x, (1.f - om) * xb.y, (1.f - om) * xb.z);
    if (k == 0) {
      cur.x += yn.x;
      cur.y += yn.y;
      cur.z += yn.z;
    }
  } else {
    post = f3(xb);
    cur = post;
    yn = make_float3(0.f, 0.f, 0.f);
  }
  adj_buf(a, src ^ 1)[i] = make_float4(cur.x, cur.y, cur.z, 0.f);
  a.ybar[i] = make_float4(yn.x, yn.y, yn.z, 0.f);
  const float c = a.cnt[i];
  const float ic = c > 0.f ? 1.f / c : 0.f;
  a.dxbar[i] = make_float4(post.x * ic, post.y * ic, post.z * ic, 0.f);
}

// Reverse of the block projection of one tet.  In: the tet's positions
// entering the iteration (tt.p, w = inv_m) and inv_Dm, its multipliers L
// entering it, compliances aD, aH, the adjoint of its multipliers after the
// iteration (lb_next) and the adjoints of its corners' Jacobi accumulators
// (dpb).  Out: the adjoints of the four corner positions (gout), of the
// multipliers entering the iteration (lb_out) and of aD, aH (aDb, aHb).
template <bool kPrecise>
__device__ __forceinline__ void tet_adjoint(const Tet& tt, const float2 L, const float aD, const float aH,
                                            const float2 lb_next, const float3 (&dpb)[4], float3 (&gout)[4],
                                            float2& lb_out, float& aDb, float& aHb) {
  const float w[4] = {tt.p[0].w, tt.p[1].w, tt.p[2].w, tt.p[3].w};
  // ---- forward recompute ----
  float F[9];
  deformation_gradient(tt, F);
  float C_D, C_H;
  invariants<kPrecise>(F, C_D, C_H);
  float gF[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) gF[q] = 2.f * F[q];
  float3 gD[4], gH[4];
  corner_gradients(gF, tt.dm, gD);
  float H[9];
  cofactor(F, H);
  corner_gradients(H, tt.dm, gH);
  float A11 = aD, A22 = aH, A12 = 0.f;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    A11 += w[c] * dot3(gD[c], gD[c]);
    A22 += w[c] * dot3(gH[c], gH[c]);
    A12 += w[c] * dot3(gD[c], gH[c]);
  }
  const float b1 = -(C_D + aD * L.x), b2 = -(C_H + aH * L.y);
  // products rounded before the difference, as in the forward's elimination
  const float det = __fmul_rn(A11, A22) - __fmul_rn(A12, A12);
  const float idet = 1.f / det;
  const float dD = (A22 * b1 - A12 * b2) * idet;
  const float dH = (A11 * b2 - A12 * b1) * idet;
  // ---- reverse ----
  float dDb = lb_next.x, dHb = lb_next.y;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    dDb += w[c] * dot3(gD[c], dpb[c]);
    dHb += w[c] * dot3(gH[c], dpb[c]);
  }
  const float bb1 = (A22 * dDb - A12 * dHb) * idet;
  const float bb2 = (A11 * dHb - A12 * dDb) * idet;
  const float A11b = -bb1 * dD, A22b = -bb2 * dH, A12b = -(bb1 * dH + bb2 * dD);
  const float CDb = -bb1, CHb = -bb2;
  aDb = -L.x * bb1 + A11b;
  aHb = -L.y * bb2 + A22b;
  lb_out = make_float2(lb_next.x - aD * bb1, lb_next.y - aH * bb2);
  // adjoints of the corner gradients
  float3 gDb[4], gHb[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float wd = w[c] * dD, wh = w[c] * dH, a1 = 2.f * w[c] * A11b, a2 = 2.f * w[c] * A22b, a3 = w[c] * A12b;
    gDb[c] = make_float3(wd * dpb[c].x + a1 * gD[c].x + a3 * gH[c].x, wd * dpb[c].y + a1 * gD[c].y + a3 * gH[c].y,
                         wd * dpb[c].z + a1 * gD[c].z + a3 * gH[c].z);
    gHb[c] = make_float3(wh * dpb[c].x + a2 * gH[c].x + a3 * gD[c].x, wh * dpb[c].y + a2 * gH[c].y + a3 * gD[c].y,
                         wh * dpb[c].z + a2 * gH[c].z + a3 * gD[c].z);
  }
  // g_{c+1}[r] = sum_q G[r][q] dm[c][q], g_0 = -sum  =>  G_bar[r][q] = sum_c (gb_{c+1} - gb_0)[r] dm[c][q]
  float ed[3][3], eh[3][3];  // [c][r]
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    ed[c][0] = gDb[c + 1].x - gDb[0].x;
    ed[c][1] = gDb[c + 1].y - gDb[0].y;
    ed[c][2] = gDb[c + 1].z - gDb[0].z;
    eh[c][0] = gHb[c + 1].x - gHb[0].x;
    eh[c][1] = gHb[c + 1].y - gHb[0].y;
    eh[c][2] = gHb[c + 1].z - gHb[0].z;
  }
  float GDb[9], Hb[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      float sd = 0.f, sh = 0.f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sd += ed[c][r] * tt.dm[c * 3 + q];
        sh += eh[c][r] * tt.dm[c * 3 + q];
      }
      GDb[r * 3 + q] = sd;
      Hb[r * 3 + q] = sh;
    }
  // F_bar = 2 GD_bar + 2 C_D_bar F + C_H_bar cof(F) + (d cof)^T H_bar
  float Fb[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) Fb[q] = 2.f * GDb[q] + 2.f * CDb * F[q] + CHb * H[q];
  {
    const float3 F0 = make_float3(F[0], F[3], F[6]), F1 = make_float3(F[1], F[4], F[7]), F2 = make_float3(F[2], F[5], F[8]);
    const float3 H0b = make_float3(Hb[0], Hb[3], Hb[6]), H1b = make_float3(Hb[1], Hb[4], Hb[7]),
                 H2b = make_float3(Hb[2], Hb[5], Hb[8]);
    const float3 c0 = cross3(H1b, F2), c0b = cross3(F1, H2b);
    const float3 c1 = cross3(F2, H0b), c1b = cross3(H2b, F0);
    const float3 c2 = cross3(H0b, F1), c2b = cross3(F0, H1b);
    Fb[0] += c0.x + c0b.x; Fb[3] += c0.y + c0b.y; Fb[6] += c0.z + c0b.z;
    Fb[1] += c1.x + c1b.x; Fb[4] += c1.y + c1b.y; Fb[7] += c1.z + c1b.z;
    Fb[2] += c2.x + c2b.x; Fb[5] += c2.y + c2b.y; Fb[8] += c2.z + c2b.z;
  }
  // F = E Dm (E[r][c] = e_c[r])  =>  E_bar[r][c] = sum_q F_bar[r][q] dm[c][q]
#pragma unroll
  for (int c = 0; c < 3; ++c)
    gout[c + 1] = make_float3(Fb[0] * tt.dm[c * 3] + Fb[1] * tt.dm[c * 3 + 1] + Fb[2] * tt.dm[c * 3 + 2],
                              Fb[3] * tt.dm[c * 3] + Fb[4] * tt.dm[c * 3 + 1] + Fb[5] * tt.dm[c * 3 + 2],
                              Fb[6] * tt.dm[c * 3] + Fb[7] * tt.dm[c * 3 + 1] + Fb[8] * tt.dm[c * 3 + 2]);
  gout[0] = make_float3(-(gout[1].x + gout[2].x + gout[3].x), -(gout[1].y + gout[2].y + gout[3].y),
                        -(gout[1].z + gout[2].z + gout[3].z));
}

// Reverse of the block projection of iteration k, one thread per tet; scatters
// the position adjoints into abuf[dst] and updates the multiplier adjoint.
template <class D, bool kPrecise>
__global__ void __launch_bounds__(128) ka_project(D d, Tape tp, Adj a, int k, float cD, float cH, int dst) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= adj_tets(d)) return;
  int vid[4];
  Tet tt;
  float inv_v0, m_mu, m_la;
  if (!adj_load_tet(d, t, vid, tt, inv_v0, m_mu, m_la)) return;
  const float4* X = tp.xs + (size_t)k * adj_verts(d);
#pragma unroll
  for (int c = 0; c < 4; ++c) tt.p[c] = __ldg(X + vid[c]);
  const float2 L = tp.lams[(size_t)k * adj_tets(d) + t];
  const float sD = cD * inv_v0, sH = cH * inv_v0;  // d aD / d(1/mu), d aH / d(1/lambda)
  const float aD = sD * m_mu, aH = sH * m_la;
  float3 dpb[4], gout[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) dpb[c] = f3(a.dxbar[vid[c]]);
  float2 lb;
  float aDb, aHb;
  tet_adjoint<kPrecise>(tt, L, aD, aH, a.lambar[t], dpb, gout, lb, aDb, aHb);
  a.lambar[t] = lb;
  float4* G = adj_buf(a, dst);
#pragma unroll
  for (int c = 0; c < 4; ++c) red_add_v4(G + vid[c], gout[c].x, gout[c].y, gout[c].z, 0.f);
  // materials: aD = (1/mu) sD, aH = (1/lambda) sH
  a.g_mu[t] += (double)(aDb * sD);
  a.g_la[t] += (double)(aHb * sH);
}

// One step of the omega chain backwards, iteration k of body b: from omega_k's
// adjoint to rho_hat_k's and r_hat_k's (returned).  Every CTA that needs r_hat_k's
// adjoint calls it with the same inputs; the one with `store` keeps the state
// for iteration k - 1.
__device__ __forceinline__ double chain_step(const Adj& a, int b, int k, bool store) {
  double* o = a.om + (size_t)a.om_n * b;
  const double* t = o + kTab + kTabRow * k;
  const int q = k & 1;
  const double wb = o[kOmSum + q] * t[0] + o[kOmCarry + q];
  double rho_bar = o[kRhoBar + q] + t[1] * wb;
  const double ri_bar = t[3] * rho_bar;
  rho_bar -= ri_bar;
  const double rb = o[kRCarry + q] + t[4] * ri_bar;
  if (store) {
    o[kOmCarry + (q ^ 1)] = t[2] * wb;
    o[kRCarry + (q ^ 1)] = t[5] * ri_bar;
    o[kRhoBar + (q ^ 1)] = rho_bar;
    o[kOmSum + (q ^ 1)] = 0.0;  // ka_cheb of iteration k - 1 sums into it
  }
  return rb;
}

// The residual's part of one tet: r_hat = (1/n) sum_t sqrt(rD^2 + rH^2),
// rD = C_D + aD lambda_D, rH = C_H + aH lambda_H at the post-Jacobi positions
// (tt.p) with the multipliers after the iteration (L1).  From r_hat's adjoint
// rb_n = rb / n: the corner position adjoints (g) and those of L1 and of aD, aH.
template <bool kPrecise>
__device__ __forceinline__ void residual_adjoint(const Tet& tt, const float2 L1, const float aD, const float aH,
                                                 const float rb_n, float3 (&g)[4], float2& lb, float& aDb,
                                                 float& aHb) {
  float F[9];
  deformation_gradient(tt, F);
  float C_D, C_H;
  invariants<kPrecise>(F, C_D, C_H);
  const float rD = C_D + aD * L1.x, rH = C_H + aH * L1.y;
  const float sq = sqrtf(rD * rD + rH * rH);
  const float rDb = sq > 0.f ? rb_n * rD / sq : 0.f, rHb = sq > 0.f ? rb_n * rH / sq : 0.f;
  float H[9], Fb[9];
  cofactor(F, H);
#pragma unroll
  for (int q = 0; q < 9; ++q) Fb[q] = 2.f * rDb * F[q] + rHb * H[q];
  corner_gradients(Fb, tt.dm, g);
  lb = make_float2(rDb * aD, rHb * aH);
  aDb = rDb * L1.x;
  aHb = rHb * L1.y;
}

// r_hat_k's adjoint into the tets of iteration k (single-body layout, one
// thread per tet): scatters the position adjoints into the Jacobi
// accumulator's (dxbar, post = x~ + dx / cnt) and into abuf[dst] (x~_k's),
// adds to the multipliers' adjoint (still that of lambda_{k+1}) and to the
// material adjoints.
template <class D, bool kPrecise>
__global__ void __launch_bounds__(128) ka_residual_adj(D d, Tape tp, Adj a, int k, float cD, float cH, int dst) {
  __shared__ float s_rb;
  if (threadIdx.x == 0) s_rb = (float)(chain_step(a, 0, k, blockIdx.x == 0) / adj_body_tets(d, 0));
  __syncthreads();
  const float rb_n = s_rb;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= adj_tets(d) || rb_n == 0.f) return;
  int vid[4];
  Tet tt;
  float inv_v0, m_mu, m_la;
  if (!adj_load_tet(d, t, vid, tt, inv_v0, m_mu, m_la)) return;
  const float4* X = tp.posts + (size_t)k * adj_verts(d);
#pragma unroll
  for (int c = 0; c < 4; ++c) tt.p[c] = __ldg(X + vid[c]);
  const float2 L1 = tp.lams[(size_t)(k + 1) * adj_tets(d) + t];
  const float sD = cD * inv_v0, sH = cH * inv_v0;
  float3 g[4];
  float2 lb;
  float aDb, aHb;
  residual_adjoint<kPrecise>(tt, L1, sD * m_mu, sH * m_la, rb_n, g, lb, aDb, aHb);
  float4* G = adj_buf(a, dst);
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float cn = a.cnt[vid[c]];
    const float ic = cn > 0.f ? 1.f / cn : 0.f;
    red_add_v4(G + vid[c], g[c].x, g[c].y, g[c].z, 0.f);
    red_add_v4(a.dxbar + vid[c], g[c].x * ic, g[c].y * ic, g[c].z * ic, 0.f);
  }
  const float2 l0 = a.lambar[t];
  a.lambar[t] = make_float2(l0.x + lb.x, l0.y + lb.y);
  a.g_mu[t] += (double)(aDb * sD);
  a.g_la[t] += (double)(aHb * sH);
}

// q_bar = J^T q_bar for the SDF projection q' = q + n(q) (-phi(q)) at q.
__device__ __forceinline__ float3 sdf_adjoint(const xpbd_sdf& s, const float3 q, float3 gb) {
  if (s.kind == XPBD_SDF_PLANE) {
    const float dn = gb.x * s.b[0] + gb.y * s.b[1] + gb.z * s.b[2];
    return make_float3(gb.x - s.b[0] * dn, gb.y - s.b[1] * dn, gb.z - s.b[2] * dn);
  }
  const float dx = q.x - s.a[0], dy = q.y - s.a[1], dz = q.z - s.a[2];
  if (s.kind == XPBD_SDF_SPHERE) {  // J = (r + eps) / (|d| + eps) (I - |d| / (|d| + eps) u u^T)
    const float sl = sqrtf(dx * dx + dy * dy + dz * dz);
    const float iu = 1.f / sl;
    const float ux = dx * iu, uy = dy * iu, uz = dz * iu;
    const float kk = (s.b[0] + kEps) / (sl + kEps), cc = sl / (sl + kEps);
    const float ug = ux * gb.x + uy * gb.y + uz * gb.z;
    return make_float3(kk * (gb.x - cc * ux * ug), kk * (gb.y - cc * uy * ug), kk * (gb.z - cc * uz * ug));
  }
  // cube: J = I - n grad(phi)^T; n on the dominant axis of (q - c), grad(phi)
  // on the largest (|q - c| - half size), both signed like (q - c)
  const float ad[3] = {fabsf(dx), fabsf(dy), fabsf(dz)};
  const float dv[3] = {dx, dy, dz};
  int na = 0;
  float amax = ad[0];
  if (ad[1] > ad[0]) { na = 1; amax = ad[1]; }
  if (ad[2] > amax) na = 2;
  const float e[3] = {ad[0] - s.b[0], ad[1] - s.b[1], ad[2] - s.b[2]};
  int ga = 0;
  if (e[1] > e[ga]) ga = 1;
  if (e[2] > e[ga]) ga = 2;
  const float sn = dv[na] > 0.f ? 1.f : -1.f, sg = dv[ga] > 0.f ? 1.f : -1.f;
  float g[3] = {gb.x, gb.y, gb.z};
  g[ga] -= sg * sn * g[na];
  return make_float3(g[0], g[1], g[2]);
}

// Reverse of the SDF list (in reverse order) and of predict; adds into gx, gv.
template <class D>
__global__ void __launch_bounds__(256) ka_begin(D d, Tape tp, Adj a, int src, float dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= adj_verts(d)) return;
  float3 gb = f3(adj_buf(a, src)[i]);
  const float4 pre = tp.xpre[i];
  if (pre.w > 0.f) {
    const float3 vel = f3(tp.v1[i]);
    for (int s = d.n_sdf - 1; s >= 0; --s) {
      // positions entering SDF s: replay the list up to s
      float3 q = f3(pre);
      for (int r = 0; r < s; ++r) {
        const xpbd_sdf sd = d.sdfs[r];
        const float phi = sdf_dist(sd, q);
        if (phi < 0.f) {
          const float3 n = sdf_normal(sd, q);
          const float dotnv = n.x * (sd.vel[0] - vel.x) + n.y * (sd.vel[1] - vel.y) + n.z * (sd.vel[2] - vel.z);
          if (dotnv > 0.f || sd.fixed) {
            q.x -= n.x * phi;
            q.y -= n.y * phi;
            q.z -= n.z * phi;
          }
        }
      }
      const xpbd_sdf sd = d.sdfs[s];
      const float phi = sdf_dist(sd, q);
      if (phi < 0.f) {
        const float3 n = sdf_normal(sd, q);
        const float dotnv = n.x * (sd.vel[0] - vel.x) + n.y * (sd.vel[1] - vel.y) + n.z * (sd.vel[2] - vel.z);
        if (dotnv > 0.f || sd.fixed) gb = sdf_adjoint(sd, q, gb);
      }
    }
  }
  float4 gx = a.gx[i], gv = a.gv[i];
  gx.x += gb.x; gx.y += gb.y; gx.z += gb.z;
  gv.x += gb.x * dt; gv.y += gb.y * dt; gv.z += gb.z * dt;
  a.gx[i] = gx;
  a.gv[i] = gv;
}

}  // namespace xpbd

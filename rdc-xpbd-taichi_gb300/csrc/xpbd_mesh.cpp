// Host mesh preprocessing for the GB300 solver.
//
// The reference obtains its mesh from meshtaichi_patcher (xpbd_base.py:42),
// whose patch partition + reorder serves Taichi's mesh_local staging.  Here the
// mesh is reordered along a Z-order (Morton) curve so that the tet sweep's
// vertex gathers and the Jacobi scatter hit nearby cache lines, and a
// vertex -> (tet, corner) CSR is built for the deterministic gather variant.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "../../include/xpbd_gb300.h"

namespace {

// Spread the low 21 bits of v so that bit i lands at bit 3i.
inline uint64_t spread3(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

struct Box {
  double lo[3], scale[3];
};

inline uint64_t morton(const Box& b, double x, double y, double z) {
  const double q[3] = {(x - b.lo[0]) * b.scale[0], (y - b.lo[1]) * b.scale[1], (z - b.lo[2]) * b.scale[2]};
  uint64_t c[3];
  for (int k = 0; k < 3; ++k) {
    double v = q[k];
    if (!(v > 0.0)) v = 0.0;
    if (v > 2097151.0) v = 2097151.0;
    c[k] = (uint64_t)v;
  }
  return spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
}

void order_by(const std::vector<uint64_t>& code, int32_t* perm) {
  const size_t n = code.size();
  std::vector<int32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return code[a] < code[b]; });
  std::copy(idx.begin(), idx.end(), perm);
}

// Parity of a permutation of (0, 1, 2, 3): true if even.
inline bool even4(const int q[4]) {
  int inv = 0;
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j) inv += q[i] > q[j];
  return (inv & 1) == 0;
}

inline uint8_t pack4(const int q[4]) {
  return (uint8_t)(q[0] | (q[1] << 2) | (q[2] << 4) | (q[3] << 6));
}

}  // namespace

extern "C" {

int xpbd_morton_order(const double* pts, int32_t n_verts, const int32_t* tets, int32_t n_tets, int32_t* vert_perm,
                      int32_t* tet_perm) {
  if (!pts || n_verts <= 0 || n_tets < 0 || (n_tets > 0 && !tets)) return XPBD_ERR_INVALID_ARGUMENT;
  for (int64_t k = 0; k < 4ll * n_tets; ++k)
    if (tets[k] < 0 || tets[k] >= n_verts) return XPBD_ERR_BAD_MESH;
  Box b;
  for (int k = 0; k < 3; ++k) {
    double lo = pts[k], hi = pts[k];
    for (int32_t i = 1; i < n_verts; ++i) {
      lo = std::min(lo, pts[3 * i + k]);
      hi = std::max(hi, pts[3 * i + k]);
    }
    b.lo[k] = lo;
    b.scale[k] = hi > lo ? 2097151.0 / (hi - lo) : 0.0;
  }
  if (tet_perm && n_tets > 0) {
    std::vector<uint64_t> code(n_tets);
    for (int32_t t = 0; t < n_tets; ++t) {
      double c[3] = {0.0, 0.0, 0.0};
      for (int q = 0; q < 4; ++q) {
        const int32_t v = tets[4 * t + q];
        if (v < 0 || v >= n_verts) return XPBD_ERR_BAD_MESH;
        for (int k = 0; k < 3; ++k) c[k] += 0.25 * pts[3 * v + k];
      }
      code[t] = morton(b, c[0], c[1], c[2]);
    }
    order_by(code, tet_perm);
  }
  if (vert_perm) {
    // Vertices are numbered in order of first use by the Morton-sorted tets,
    // so the corners of consecutive tets are close in memory; vertices no tet
    // uses follow in Morton order of their positions.
    std::vector<uint64_t> code(n_verts);
    for (int32_t i = 0; i < n_verts; ++i) code[i] = morton(b, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    std::vector<int32_t> by_code(n_verts);
    order_by(code, by_code.data());
    std::vector<char> seen(n_verts, 0);
    int32_t k = 0;
    if (tet_perm) {
      for (int32_t t = 0; t < n_tets; ++t)
        for (int q = 0; q < 4; ++q) {
          const int32_t v = tets[4 * tet_perm[t] + q];
          if (!seen[v]) {
            seen[v] = 1;
            vert_perm[k++] = v;
          }
        }
    }
    for (int32_t i = 0; i < n_verts; ++i)
      if (!seen[by_code[i]]) vert_perm[k++] = by_code[i];
  }
  return XPBD_OK;
}

int xpbd_build_patches(const int32_t* tets, int32_t n_tets, int32_t n_verts, int32_t patch_tets,
                       int32_t* patch_voff, int32_t* patch_verts, uint32_t* tet_lid, int32_t* max_patch_verts) {
  if (!tets || n_tets <= 0 || n_verts <= 0 || patch_tets <= 0 || !patch_voff || !patch_verts || !tet_lid ||
      !max_patch_verts)
    return XPBD_ERR_INVALID_ARGUMENT;
  const int32_t np = (n_tets + patch_tets - 1) / patch_tets;
  std::vector<int32_t> uniq;
  uniq.reserve(4 * patch_tets);
  int32_t total = 0, mx = 0;
  patch_voff[0] = 0;
  for (int32_t p = 0; p < np; ++p) {
    const int32_t t0 = p * patch_tets;
    const int32_t t1 = std::min(n_tets, t0 + patch_tets);
    uniq.clear();
    for (int64_t k = 4ll * t0; k < 4ll * t1; ++k) {
      const int32_t v = tets[k];
      if (v < 0 || v >= n_verts) return XPBD_ERR_BAD_MESH;
      uniq.push_back(v);
    }
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    const int32_t nv = (int32_t)uniq.size();
    mx = std::max(mx, nv);
    std::copy(uniq.begin(), uniq.end(), patch_verts + total);
    for (int32_t t = t0; t < t1; ++t) {
      uint32_t packed = 0;
      for (int q = 0; q < 4; ++q) {
        const int32_t loc = (int32_t)(std::lower_bound(uniq.begin(), uniq.end(), tets[4 * t + q]) - uniq.begin());
        packed |= (uint32_t)(loc & 0xff) << (8 * q);
      }
      tet_lid[t] = packed;
    }
    total += nv;
    patch_voff[p + 1] = total;
  }
  *max_patch_verts = mx;
  return XPBD_OK;
}

int xpbd_build_patch_csr(const int32_t* patch_voff, const uint32_t* tet_lid, int32_t n_tets, int32_t patch_tets,
                         uint16_t* pv_start, uint16_t* pv_slots) {
  if (!patch_voff || !tet_lid || !pv_start || !pv_slots || n_tets <= 0 || patch_tets <= 0 || patch_tets > 256)
    return XPBD_ERR_INVALID_ARGUMENT;
  const int32_t np = (n_tets + patch_tets - 1) / patch_tets;
  std::fill(pv_slots, pv_slots + (size_t)4 * np * patch_tets, (uint16_t)0xffff);
  std::vector<int32_t> cnt, fill;
  for (int32_t p = 0; p < np; ++p) {
    const int32_t vb = patch_voff[p], nv = patch_voff[p + 1] - vb;
    if (nv < 0 || nv > 256) return XPBD_ERR_BAD_MESH;
    const int32_t t0 = p * patch_tets, t1 = std::min(n_tets, t0 + patch_tets);
    cnt.assign(nv + 1, 0);
    for (int32_t t = t0; t < t1; ++t)
      for (int q = 0; q < 4; ++q) {
        const int32_t l = (tet_lid[t] >> (8 * q)) & 0xff;
        if (l >= nv) return XPBD_ERR_BAD_MESH;
        cnt[l + 1]++;
      }
    for (int32_t k = 0; k < nv; ++k) cnt[k + 1] += cnt[k];
    fill.assign(cnt.begin(), cnt.end() - 1);
    for (int32_t k = 0; k < nv; ++k) pv_start[vb + k] = (uint16_t)cnt[k];
    uint16_t* slots = pv_slots + (size_t)4 * p * patch_tets;
    for (int32_t t = t0; t < t1; ++t)
      for (int q = 0; q < 4; ++q) {
        const int32_t l = (tet_lid[t] >> (8 * q)) & 0xff;
        slots[fill[l]++] = (uint16_t)(4 * (t - t0) + q);
      }
  }
  return XPBD_OK;
}

int xpbd_build_vertex_csr(const int32_t* tets, int32_t n_tets, int32_t n_verts, int32_t* offsets, int32_t* slots) {
  if (!tets || !offsets || !slots || n_tets < 0 || n_verts <= 0) return XPBD_ERR_INVALID_ARGUMENT;
  std::fill(offsets, offsets + n_verts + 1, 0);
  for (int64_t k = 0; k < 4ll * n_tets; ++k) {
    const int32_t v = tets[k];
    if (v < 0 || v >= n_verts) return XPBD_ERR_BAD_MESH;
    offsets[v + 1]++;
  }
  for (int32_t v = 0; v < n_verts; ++v) offsets[v + 1] += offsets[v];
  std::vector<int32_t> fill(offsets, offsets + n_verts);
  for (int64_t k = 0; k < 4ll * n_tets; ++k) slots[fill[tets[k]]++] = (int32_t)k;
  return XPBD_OK;
}

int xpbd_pair_tets(const int32_t* tets, int32_t n_tets, int32_t n_verts, int32_t* order, uint8_t* corner_perm,
                   int32_t* n_pairs) {
  if (n_tets < 0 || n_verts <= 0 || !order || !corner_perm || !n_pairs || (n_tets > 0 && !tets))
    return XPBD_ERR_INVALID_ARGUMENT;
  for (int64_t k = 0; k < 4ll * n_tets; ++k)
    if (tets[k] < 0 || tets[k] >= n_verts) return XPBD_ERR_BAD_MESH;
  *n_pairs = 0;
  const uint8_t identity = (uint8_t)(0 | (1 << 2) | (2 << 4) | (3 << 6));
  if (n_verts >= (1 << 21)) {  // face keys pack three 21-bit ids: no pairing
    for (int32_t t = 0; t < n_tets; ++t) {
      order[t] = t;
      corner_perm[t] = identity;
    }
    return XPBD_OK;
  }
  // faces: sorted vertex triple of the face opposite corner j of tet t
  struct Face {
    uint64_t key;
    int32_t t;
    int32_t j;
  };
  std::vector<Face> faces((size_t)4 * n_tets);
  for (int32_t t = 0; t < n_tets; ++t)
    for (int j = 0; j < 4; ++j) {
      int32_t v[3], m = 0;
      for (int c = 0; c < 4; ++c)
        if (c != j) v[m++] = tets[4 * (int64_t)t + c];
      std::sort(v, v + 3);
      faces[4 * (size_t)t + j] = {((uint64_t)v[0] << 42) | ((uint64_t)v[1] << 21) | (uint64_t)v[2], t, j};
    }
  std::sort(faces.begin(), faces.end(), [](const Face& a, const Face& b) {
    return a.key < b.key || (a.key == b.key && a.t < b.t);
  });
  std::vector<int32_t> nb((size_t)4 * n_tets, -1);  // tet across the face opposite corner j
  for (size_t k = 0; k + 1 < faces.size(); ++k)
    if (faces[k].key == faces[k + 1].key && faces[k].t != faces[k + 1].t) {
      nb[4 * (size_t)faces[k].t + faces[k].j] = faces[k + 1].t;
      nb[4 * (size_t)faces[k + 1].t + faces[k + 1].j] = faces[k].t;
    }
  // corner orders of a pair (a, b) sharing the face opposite a's corner ja:
  // a' = (u, v, w, a*), b' = (v, u, w, b*), both even; false if b' is odd
  auto orders = [&](int32_t a, int ja, int32_t b, int qa[4], int qb[4]) {
    int m = 0;
    for (int c = 0; c < 4; ++c)
      if (c != ja) qa[m++] = c;
    qa[3] = ja;
    if (!even4(qa)) std::swap(qa[0], qa[1]);
    const int32_t* A = tets + 4 * (int64_t)a;
    const int32_t* B = tets + 4 * (int64_t)b;
    const int32_t want[3] = {A[qa[1]], A[qa[0]], A[qa[2]]};
    bool used[4] = {false, false, false, false};
    for (int k = 0; k < 3; ++k) {
      qb[k] = -1;
      for (int c = 0; c < 4; ++c)
        if (B[c] == want[k]) qb[k] = c;
      if (qb[k] < 0) return false;
      used[qb[k]] = true;
    }
    for (int c = 0; c < 4; ++c)
      if (!used[c]) qb[3] = c;
    return even4(qb);
  };
  // Greedy in the given (Morton) order; a partner is a face neighbour within
  // kWindow positions, the nearest one, so that pairs keep the order's locality.
  constexpr int64_t kWindow = 48;
  std::vector<int32_t> partner(n_tets, -1);
  std::vector<uint8_t> perm(n_tets, identity);
  for (int32_t t = 0; t < n_tets; ++t) {
    if (partner[t] >= 0) continue;
    int32_t best = -1;
    int64_t best_d = 0;
    int qa[4], qb[4], ba[4] = {0, 1, 2, 3}, bb[4] = {0, 1, 2, 3};
    for (int j = 0; j < 4; ++j) {
      const int32_t u = nb[4 * (size_t)t + j];
      if (u < 0 || partner[u] >= 0) continue;
      const int64_t d = u > t ? (int64_t)u - t : (int64_t)t - u;
      if (d > kWindow || (best >= 0 && d >= best_d)) continue;
      if (!orders(t, j, u, qa, qb)) continue;
      best = u;
      best_d = d;
      std::copy(qa, qa + 4, ba);
      std::copy(qb, qb + 4, bb);
    }
    if (best < 0) continue;
    partner[t] = best;
    partner[best] = t;
    perm[t] = pack4(ba);
    perm[best] = pack4(bb);
  }
  // Units of two slots: face pairs, and the remaining tets two by two in
  // order (their corners unchanged); units in the order of their first tet.
  struct Unit {
    int32_t a, b;  // b < 0: a lone last tet
  };
  std::vector<Unit> units;
  units.reserve(n_tets / 2 + 1);
  int32_t pending = -1, np = 0;
  for (int32_t t = 0; t < n_tets; ++t) {
    const int32_t u = partner[t];
    if (u >= 0) {
      if (u > t) {
        units.push_back({t, u});
        ++np;
      }
    } else if (pending < 0) {
      pending = t;
    } else {
      units.push_back({pending, t});
      pending = -1;
    }
  }
  std::stable_sort(units.begin(), units.end(), [](const Unit& x, const Unit& y) { return x.a < y.a; });
  if (pending >= 0) units.push_back({pending, -1});
  int32_t k = 0;
  for (const Unit& un : units) {
    order[k] = un.a;
    corner_perm[k++] = perm[un.a];
    if (un.b >= 0) {
      order[k] = un.b;
      corner_perm[k++] = perm[un.b];
    }
  }
  *n_pairs = np;
  return XPBD_OK;
}

}  // extern "C"

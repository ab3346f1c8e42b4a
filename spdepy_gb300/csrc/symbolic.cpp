// Symbolic analysis of the SPDE precision on a regular lattice.
//
// The reference factorises Q with CHOLMOD (fill-reducing ordering + supernodal
// analysis inside `cholesky(Q)`, spdes/advection_diffusion2D.py:117,193).  The
// pattern of Q only depends on the lattice (Q14: coefficients are time-invariant,
// and S^T S is diagonal so Q_c shares Q's pattern), so here the ordering is a
// geometric nested dissection of the (x, y, t) box: thickness-2 separators
// across x or y (spatial stencil radius 2), thickness-1 separators across t
// (temporal radius 1), whichever is smallest.  Every box of the dissection tree
// is one dense front: its separator columns S and the rows B = the box's halo
// (lattice nodes outside the box within stencil reach), which all belong to
// ancestor separators.  The result is computed once per lattice and reused for
// Q, Q_c and every theta.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "spde_internal.h"

namespace spde {

void slot_offsets(int nslots, int* dx, int* dy, int* dt) {
  int s = 0;
  if (nslots == kSlotsSep) {
    for (int c = -1; c <= 1; ++c)
      for (int a = -2; a <= 2; ++a)
        for (int b = -2; b <= 2; ++b) { dx[s] = b; dy[s] = a; dt[s] = c; ++s; }
    return;
  }
  if (nslots == kSlotsST) {
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b) { dx[s] = b; dy[s] = a; dt[s] = -1; ++s; }
  }
  for (int a = -2; a <= 2; ++a)
    for (int b = -2; b <= 2; ++b) { dx[s] = b; dy[s] = a; dt[s] = 0; ++s; }
  if (nslots == kSlotsST) {
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b) { dx[s] = b; dy[s] = a; dt[s] = 1; ++s; }
  }
}

namespace {

inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

struct NDBuilder {
  Symbolic* S;
  int Mx, Ny, T, leaf_max;
  int rt = 1;  // spatial reach of the coupling to the neighbouring time slices
  int next_new = 0;

  inline int nat(int x, int y, int t) const { return (t * Ny + y) * Mx + x; }

  void assign(const int* b) {
    for (int t = b[4]; t < b[5]; ++t)
      for (int y = b[2]; y < b[3]; ++y)
        for (int x = b[0]; x < b[1]; ++x) S->perm[nat(x, y, t)] = next_new++;
  }

  // returns front id
  int build(const int* box, int depth) {
    int a = box[1] - box[0], b = box[3] - box[2], c = box[5] - box[4];
    int64_t vol = int64_t(a) * b * c;
    const int64_t INF = INT64_MAX;
    int64_t cx = (a >= 4) ? int64_t(2) * b * c : INF;
    int64_t cy = (b >= 4) ? int64_t(2) * a * c : INF;
    int64_t ct = (T > 1 && c >= 3) ? int64_t(a) * b : INF;
    int64_t cmin = std::min(cx, std::min(cy, ct));
    Front fr;
    fr.depth = depth;
    std::memcpy(fr.box, box, sizeof(fr.box));
    if (vol <= leaf_max || cmin == INF) {
      fr.leaf = true;
      fr.s0 = next_new;
      fr.ns = int(vol);
      assign(box);
      S->fronts.push_back(fr);
      return int(S->fronts.size()) - 1;
    }
    int k1[6], k2[6], sp[6];
    std::memcpy(k1, box, sizeof(k1));
    std::memcpy(k2, box, sizeof(k2));
    std::memcpy(sp, box, sizeof(sp));
    if (cmin == cx) {
      int m = box[0] + (a - 2) / 2;
      k1[1] = m; sp[0] = m; sp[1] = m + 2; k2[0] = m + 2;
    } else if (cmin == cy) {
      int m = box[2] + (b - 2) / 2;
      k1[3] = m; sp[2] = m; sp[3] = m + 2; k2[2] = m + 2;
    } else {
      int m = box[4] + (c - 1) / 2;
      k1[5] = m; sp[4] = m; sp[5] = m + 1; k2[4] = m + 1;
    }
    int c1 = build(k1, depth + 1);
    int c2 = build(k2, depth + 1);
    fr.child[0] = c1;
    fr.child[1] = c2;
    fr.nchild = 2;
    fr.s0 = next_new;
    fr.ns = (sp[1] - sp[0]) * (sp[3] - sp[2]) * (sp[5] - sp[4]);
    assign(sp);
    S->fronts.push_back(fr);
    int id = int(S->fronts.size()) - 1;
    S->fronts[c1].parent = id;
    S->fronts[c2].parent = id;
    return id;
  }

  // Halo of a box: lattice nodes outside it within stencil reach, as new indices.
  void halo(const int* b, std::vector<int>& out) const {
    out.clear();
    int xa = std::max(0, b[0] - 2), xb = std::min(Mx, b[1] + 2);
    int ya = std::max(0, b[2] - 2), yb = std::min(Ny, b[3] + 2);
    for (int t = b[4]; t < b[5]; ++t)
      for (int y = ya; y < yb; ++y)
        for (int x = xa; x < xb; ++x) {
          bool inside = x >= b[0] && x < b[1] && y >= b[2] && y < b[3];
          if (!inside) out.push_back(S->perm[nat(x, y, t)]);
        }
    if (T > 1) {
      int xa1 = std::max(0, b[0] - rt), xb1 = std::min(Mx, b[1] + rt);
      int ya1 = std::max(0, b[2] - rt), yb1 = std::min(Ny, b[3] + rt);
      for (int t : {b[4] - 1, b[5]}) {
        if (t < 0 || t >= T) continue;
        for (int y = ya1; y < yb1; ++y)
          for (int x = xa1; x < xb1; ++x) out.push_back(S->perm[nat(x, y, t)]);
      }
    }
    std::sort(out.begin(), out.end());
  }
};

// Position of new index `v` inside front f (S part first, then sorted B), or -1.
int front_pos(const Symbolic& S, const Front& f, int v) {
  if (v >= f.s0 && v < f.s0 + f.ns) return v - f.s0;
  const int* beg = S.blist.data() + f.b_off;
  const int* end = beg + f.nb;
  const int* it = std::lower_bound(beg, end, v);
  if (it == end || *it != v) return -1;
  return f.ns + int(it - beg);
}

}  // namespace

int build_symbolic(int Mx, int Ny, int T, int leaf_max, int nbk, Symbolic* out, bool separable) {
  if (Mx < 1 || Ny < 1 || T < 1 || leaf_max < 1 || nbk < 8 || (separable && T < 2)) return -1;
  Symbolic& S = *out;
  S = Symbolic();
  S.Mx = Mx; S.Ny = Ny; S.T = T;
  int64_t n64 = int64_t(Mx) * Ny * T;
  if (n64 > INT32_MAX / 64) return -2;
  S.n = int(n64);
  S.nslots = separable ? kSlotsSep : (T > 1 ? kSlotsST : kSlotsS);
  S.nbk = nbk;
  S.leaf_max = leaf_max;
  S.perm.assign(S.n, -1);
  NDBuilder B{&S, Mx, Ny, T, leaf_max};
  B.rt = separable ? 2 : 1;
  int root[6] = {0, Mx, 0, Ny, 0, T};
  B.build(root, 0);
  if (B.next_new != S.n) return -3;
  S.iperm.assign(S.n, 0);
  for (int k = 0; k < S.n; ++k) S.iperm[S.perm[k]] = k;
  S.front_of.assign(S.n, -1);
  const int nf = int(S.fronts.size());
  std::vector<int> h;
  for (int f = 0; f < nf; ++f) {
    Front& fr = S.fronts[f];
    for (int v = fr.s0; v < fr.s0 + fr.ns; ++v) S.front_of[v] = f;
    B.halo(fr.box, h);
    fr.nb = int(h.size());
    fr.b_off = int64_t(S.blist.size());
    S.blist.insert(S.blist.end(), h.begin(), h.end());
    S.max_depth = std::max(S.max_depth, fr.depth);
  }
  // every B node must be a later node (ancestor separator)
  for (int f = 0; f < nf; ++f) {
    const Front& fr = S.fronts[f];
    for (int i = 0; i < fr.nb; ++i)
      if (S.blist[fr.b_off + i] < fr.s0 + fr.ns) return -4;
  }
  // extend-add maps
  S.rmap.assign(S.blist.size(), -1);
  for (int f = 0; f < nf; ++f) {
    const Front& fr = S.fronts[f];
    if (fr.parent < 0) { if (fr.nb) return -5; continue; }
    const Front& pa = S.fronts[fr.parent];
    for (int i = 0; i < fr.nb; ++i) {
      int p = front_pos(S, pa, S.blist[fr.b_off + i]);
      if (p < 0) return -6;
      S.rmap[fr.b_off + i] = p;
    }
  }
  // arenas: panels grouped by depth (deepest first) so a depth is contiguous
  S.by_depth.assign(S.max_depth + 1, {});
  for (int f = 0; f < nf; ++f) S.by_depth[S.fronts[f].depth].push_back(f);
  int64_t off = 0, doff = 0;
  for (int d = S.max_depth; d >= 0; --d) {
    int64_t uoff = 0, zoff = 0, woff = 0;
    for (int f : S.by_depth[d]) {
      Front& fr = S.fronts[f];
      fr.ld = int(round_up(fr.ns, 4));
      fr.ldu = int(round_up(std::max(fr.nb, 1), 4));
      fr.ldz = int(round_up(fr.ns + fr.nb, 4));
      fr.p_off = off;
      off = round_up(off + int64_t(fr.ns + fr.nb) * fr.ld, 32);
      fr.u_off = uoff;
      uoff = round_up(uoff + int64_t(fr.nb) * fr.ldu, 32);
      fr.z_off = zoff;
      zoff = round_up(zoff + int64_t(fr.ns + fr.nb) * fr.ldz, 32);
      fr.w_base = woff;
      woff += fr.nb;
      fr.d_off = doff;
      doff += int64_t((fr.ns + nbk - 1) / nbk) * nbk * nbk;
      S.max_front = std::max(S.max_front, fr.ns + fr.nb);
      S.max_ns = std::max(S.max_ns, fr.ns);
      S.max_nb = std::max(S.max_nb, fr.nb);
      double s = fr.ns, b = fr.nb;
      S.factor_flops += s * s * s / 3.0 + b * s * s + b * b * s;
      S.selinv_flops += b * s * s + 2.0 * b * b * s + 2.0 * s * s * s / 3.0 + 2.0 * s * s * b;
      S.nnz_l += s * (s + 1) / 2 + s * b;
    }
    S.u_pool[d & 1] = std::max(S.u_pool[d & 1], uoff);
    S.z_pool[d & 1] = std::max(S.z_pool[d & 1], zoff);
    S.w_pool[d & 1] = std::max(S.w_pool[d & 1], woff);
  }
  S.l_size = off;
  S.dinv_size = doff;
  // assembly map: (natural node, slot) -> offset in its front panel
  std::vector<int> dx(S.nslots), dy(S.nslots), dt(S.nslots);
  slot_offsets(S.nslots, dx.data(), dy.data(), dt.data());
  S.amap.assign(int64_t(S.n) * S.nslots, -1);
  for (int t = 0; t < T; ++t)
    for (int y = 0; y < Ny; ++y)
      for (int x = 0; x < Mx; ++x) {
        int k = (t * Ny + y) * Mx + x;
        int vk = S.perm[k];
        const Front& fr = S.fronts[S.front_of[vk]];
        int col = vk - fr.s0;
        for (int s = 0; s < S.nslots; ++s) {
          int xx = x + dx[s], yy = y + dy[s], tt = t + dt[s];
          if (xx < 0 || xx >= Mx || yy < 0 || yy >= Ny || tt < 0 || tt >= T) continue;
          int vn = S.perm[(tt * Ny + yy) * Mx + xx];
          if (vn < vk) continue;
          int row = front_pos(S, fr, vn);
          if (row < 0) return -7;
          S.amap[int64_t(k) * S.nslots + s] = row * fr.ld + col;
        }
      }
  return 0;
}

}  // namespace spde

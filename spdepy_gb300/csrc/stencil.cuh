// Device restatement of the reference stencils, one cell per call.
//
// Diffusion (9 entries, order 0:(0,0) 1:(+1,0) 2:(-1,0) 3:(0,+1) 4:(0,-1)
// 5:(+1,+1) 6:(-1,-1) 7:(-1,+1) 8:(+1,-1)) follows AcH_2D_b{1,3}.cpp / AH_2D_b{1,3}.cpp;
// advection (5 entries, the first five offsets) follows Acw_2D_b{1,3}.cpp /
// Aw_2D_b{1,3}.cpp.  Arithmetic is written operation by operation with _rn
// intrinsics so the compiler cannot contract it into FMAs: the triplet entry
// points reproduce the reference's doubles bit for bit.
#pragma once
#include <cuda_runtime.h>

namespace spde {

struct CellH {  // the eight face coefficients the 9-point stencil reads
  double W00, E00, N01, S01, N11, S11, E10, W10;
};

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dd(double a, double b) { return __ddiv_rn(a, b); }

// Face coefficients of cell c = (i, j).  field: Hc points at this cell's
// (4, 2, 2) block with faces W,E,S,N; otherwise Hc is one 2x2 matrix (row-major)
// whose [1][0] entry stands for every cross term with bc = 1
// (AcH_2D_b1.cpp:42-49) while bc = 3 reads [0][1] on the N/S faces
// (AcH_2D_b3.cpp:41-44).  bc == 1 applies the Neumann face zeroing: for the
// constant stencil on the current boundary cell (AcH_2D_b1.cpp:51-68), for the
// field stencil only on cell 0, the single cell the reference's loop order
// zeroes before use (AH_2D_b1.cpp:34-52).
__device__ __forceinline__ CellH cell_h(const double* Hc, bool field, int c, int i, int j, int M, int N, int bc) {
  CellH h;
  const double* H = Hc;
  if (field) {
    const double* q = Hc;
    h.W00 = q[0 * 4 + 0]; h.W10 = q[0 * 4 + 2];
    h.E00 = q[1 * 4 + 0]; h.E10 = q[1 * 4 + 2];
    h.S01 = q[2 * 4 + 1]; h.S11 = q[2 * 4 + 3];
    h.N01 = q[3 * 4 + 1]; h.N11 = q[3 * 4 + 3];
    if (bc == 1 && c == 0) { h.W00 = 0.0; h.W10 = 0.0; h.S11 = 0.0; h.S01 = 0.0; }
  } else {
    h.W00 = H[0]; h.E00 = H[0];
    h.N01 = H[2]; h.S01 = H[2]; h.E10 = H[2]; h.W10 = H[2];
    h.N11 = H[3]; h.S11 = H[3];
    if (bc == 3) { h.N01 = H[1]; h.S01 = H[1]; }
    if (bc == 1) {
      if (i == 0) { h.W00 = 0.0; h.W10 = 0.0; }
      else if (i == M - 1) { h.E00 = 0.0; h.E10 = 0.0; }
      if (j == 0) { h.S11 = 0.0; h.S01 = 0.0; }
      else if (j == N - 1) { h.N11 = 0.0; h.N01 = 0.0; }
    }
  }
  return h;
}

// Raw 9-point diffusion triplets of cell (i, j): values, columns, and whether
// the entry is kept (false = the reference's row == M*N sentinel).
__device__ __forceinline__ void diffusion_cell(const CellH& h, double hx, double hy, int i, int j, int M, int N,
                                               int bc, double* v, int* col, bool* keep) {
  const double ha = dd(hy, hx), hb = dd(hx, hy);
  double t1a = dm(ha, h.E00), t1b = dm(0.25, ds(h.N01, h.S01));
  double t2a = dm(ha, h.W00), t2b = dm(-0.25, ds(h.N01, h.S01));
  double t3a = dm(hb, h.N11), t3b = dm(0.25, ds(h.E10, h.W10));
  double t4a = dm(hb, h.S11), t4b = dm(-0.25, ds(h.E10, h.W10));
  double t5 = dm(0.25, da(h.N01, h.E10));
  double t6 = dm(0.25, da(h.S01, h.W10));
  double t7 = dm(-0.25, da(h.N01, h.W10));
  double t8 = dm(-0.25, da(h.S01, h.E10));
  // -hy/hx*(E+W) - hx/hy*(N+S), evaluated as ((-hy)/hx)*(E+W) - (hx/hy)*(N+S)
  double v0 = ds(dm(dd(-hy, hx), da(h.E00, h.W00)), dm(hb, da(h.N11, h.S11)));
  v[1] = da(t1a, t1b); v[2] = da(t2a, t2b); v[3] = da(t3a, t3b); v[4] = da(t4a, t4b);
  v[5] = t5; v[6] = t6; v[7] = t7; v[8] = t8;
  const int k = j * M + i;
  for (int p = 0; p < 9; ++p) keep[p] = true;
  if (bc == 1) {
    int in = i - 1, ip = i + 1, jn = j - 1, jp = j + 1;
    if (i == 0) in = i; else if (i == M - 1) ip = i;
    if (j == 0) jn = j; else if (j == N - 1) jp = j;
    col[0] = k; col[1] = j * M + ip; col[2] = j * M + in; col[3] = jp * M + i; col[4] = jn * M + i;
    col[5] = jp * M + ip; col[6] = jn * M + in; col[7] = jp * M + in; col[8] = jn * M + ip;
    double rem = 0.0;
    if (col[1] == k) { rem = da(da(rem, t1a), t1b); keep[1] = false; }
    if (col[2] == k) { rem = da(da(rem, t2a), t2b); keep[2] = false; }
    if (col[3] == k) { rem = da(da(rem, t3a), t3b); keep[3] = false; }
    if (col[4] == k) { rem = da(da(rem, t4a), t4b); keep[4] = false; }
    if (col[5] == k) { rem = da(rem, t5); keep[5] = false; }
    if (col[6] == k) { rem = da(rem, t6); keep[6] = false; }
    if (col[7] == k) { rem = da(rem, t7); keep[7] = false; }
    if (col[8] == k) { rem = da(rem, t8); keep[8] = false; }
    v[0] = da(v0, rem);
  } else {
    col[0] = k; col[1] = j * M + i + 1; col[2] = j * M + i - 1; col[3] = (j + 1) * M + i;
    col[4] = (j - 1) * M + i; col[5] = (j + 1) * M + i + 1; col[6] = (j - 1) * M + i - 1;
    col[7] = (j + 1) * M + i - 1; col[8] = (j - 1) * M + i + 1;
    v[0] = da(v0, 0.0);
    if (i == 0) { keep[2] = keep[6] = keep[7] = false; }
    else if (i == M - 1) { keep[1] = keep[5] = keep[8] = false; }
    if (j == 0) { keep[4] = keep[6] = keep[8] = false; }
    else if (j == N - 1) { keep[3] = keep[5] = keep[7] = false; }
  }
}

__device__ __forceinline__ double sgn_div(double g) { return g / fabs(g); }  // NaN at 0, as the reference

// Raw 5-point advection triplets.  field == false: constant G = (wx, wy) in
// G[0], G[1] (Acw_2D_b*.cpp).  field == true: G, dG hold this cell's four face
// values ordered E,N,W,S (Aw_2D_b*.cpp); bc == 1 zeroes the folded faces of the
// current cell first.
__device__ __forceinline__ void advection_cell(const double* G, const double* dG, bool field, double hx, double hy,
                                               int i, int j, int M, int N, int bc, int diff, double* v, int* col,
                                               bool* keep) {
  const int k = j * M + i;
  for (int p = 0; p < 5; ++p) keep[p] = true;
  int in = i - 1, ip = i + 1, jn = j - 1, jp = j + 1;
  if (!field) {
    const double g0 = G[0], g1 = G[1];
    const double a0 = fabs(g0), a1 = fabs(g1);
    if (diff == 1) {
      double s0 = sgn_div(g0);
      v[0] = dm(s0, hy);
      v[1] = dd(dm(-ds(s0, 1.0), hy), 2.0);
      v[2] = dd(dm(-da(s0, 1.0), hy), 2.0);
      v[3] = 0.0; v[4] = 0.0;
    } else if (diff == 2) {
      double s1 = sgn_div(g1);
      v[0] = dm(s1, hx);
      v[1] = 0.0; v[2] = 0.0;
      v[3] = dd(dm(-ds(s1, 1.0), hx), 2.0);
      v[4] = dd(dm(-da(s1, 1.0), hx), 2.0);
    } else {
      v[0] = da(dm(a0, hy), dm(a1, hx));
      v[1] = dd(dm(-ds(a0, g0), hy), 2.0);
      v[2] = dd(dm(-da(a0, g0), hy), 2.0);
      v[3] = dd(dm(-ds(a1, g1), hx), 2.0);
      v[4] = dd(dm(-da(a1, g1), hx), 2.0);
    }
    if (bc == 1) {
      if (i == 0) { in = i; v[0] = ds(v[0], dd(dm(a0, hy), 2.0)); keep[2] = false; }
      else if (i == M - 1) { ip = i; v[0] = ds(v[0], dd(dm(a0, hy), 2.0)); keep[1] = false; }
      if (j == 0) { jn = j; v[0] = ds(v[0], dd(dm(a1, hx), 2.0)); keep[4] = false; }
      else if (j == N - 1) { jp = j; v[0] = ds(v[0], dd(dm(a1, hx), 2.0)); keep[3] = false; }
    } else {
      v[0] = da(v[0], 0.0);
      if (i == M - 1) keep[1] = false;
      if (i == 0) keep[2] = false;
      if (j == N - 1) keep[3] = false;
      if (j == 0) keep[4] = false;
    }
  } else {
    double g[4], d[4];
    for (int f = 0; f < 4; ++f) { g[f] = G[f]; d[f] = dG ? dG[f] : 0.0; }
    if (bc == 1) {
      if (i == 0) in = i; else if (i == M - 1) ip = i;
      if (j == 0) jn = j; else if (j == N - 1) jp = j;
      if (j * M + ip == k) { g[0] = 0.0; d[0] = 0.0; keep[1] = false; }
      if (j * M + in == k) { g[2] = 0.0; d[2] = 0.0; keep[2] = false; }
      if (jp * M + i == k) { g[1] = 0.0; d[1] = 0.0; keep[3] = false; }
      if (jn * M + i == k) { g[3] = 0.0; d[3] = 0.0; keep[4] = false; }
    } else {
      if (i == M - 1) keep[1] = false;
      if (i == 0) keep[2] = false;
      if (j == N - 1) keep[3] = false;
      if (j == 0) keep[4] = false;
    }
    if (diff == 1) {
      double s0 = sgn_div(g[0]), s2 = sgn_div(g[2]);
      v[0] = dd(dm(ds(da(da(dm(s0, d[0]), d[0]), dm(s2, d[2])), d[2]), hy), 2.0);
      v[1] = dd(dm(-ds(dm(s0, d[0]), d[0]), hy), 2.0);
      v[2] = dd(dm(-da(dm(s2, d[2]), d[2]), hy), 2.0);
      v[3] = 0.0; v[4] = 0.0;
    } else if (diff == 2) {
      double s1 = sgn_div(g[1]), s3 = sgn_div(g[3]);
      v[0] = dd(dm(ds(da(da(dm(s1, d[1]), d[1]), dm(s3, d[3])), d[3]), hx), 2.0);
      v[1] = 0.0; v[2] = 0.0;
      v[3] = dd(dm(-ds(dm(s1, d[1]), d[1]), hx), 2.0);
      v[4] = dd(dm(-da(dm(s3, d[3]), d[3]), hx), 2.0);
    } else {
      double a0 = fabs(g[0]), a1 = fabs(g[1]), a2 = fabs(g[2]), a3 = fabs(g[3]);
      v[0] = da(dd(dm(ds(da(da(a0, g[0]), a2), g[2]), hy), 2.0), dd(dm(ds(da(da(a1, g[1]), a3), g[3]), hx), 2.0));
      v[1] = dd(dm(-ds(a0, g[0]), hy), 2.0);
      v[2] = dd(dm(-da(a2, g[2]), hy), 2.0);
      v[3] = dd(dm(-ds(a1, g[1]), hx), 2.0);
      v[4] = dd(dm(-da(a3, g[3]), hx), 2.0);
    }
  }
  col[0] = k; col[1] = j * M + ip; col[2] = j * M + in; col[3] = jp * M + i; col[4] = jn * M + i;
}

// Geometric 3x3 slot of column `c` relative to cell (i, j): (dy+1)*3 + (dx+1).
__device__ __forceinline__ int geo9(int c, int i, int j, int M) {
  int cj = c / M, ci = c - cj * M;
  return (cj - j + 1) * 3 + (ci - i + 1);
}

}  // namespace spde

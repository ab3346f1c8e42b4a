// Internal declarations shared by the host symbolic analysis and the CUDA kernels.
//
// Lattice: nodes (x, y, t), x < Mx, y < Ny, t < T, natural index
// k = t*Mx*Ny + y*Mx + x (the reference's block-t, cell j*M+i numbering,
// spdes/advection_diffusion2D.py:112-116).  The precision Q couples a node to
// spatial offsets |dx|,|dy| <= 2 in its own time slice (25-point, A^T D A) and
// |dx|,|dy| <= 1 in the neighbouring slices (9-point, -Qs V^-1 A).
#pragma once
#include <cstdint>
#include <vector>

namespace spde {

// Stencil slots of one node: dt = -1 (9), dt = 0 (25), dt = +1 (9); T == 1 keeps
// only the 25 same-slice slots.  Separable space-time models (Q = Qt (x) Qs,
// spdes/seperable_spatial_temporal2D.py:64-83) couple |dx|,|dy| <= 2 in the
// neighbouring slices too: 3 x 25 slots, slot = (dt + 1) 25 + (dy + 2) 5 + dx + 2.
// The slot count identifies the layout.
constexpr int kSlotsST = 43;
constexpr int kSlotsS = 25;
constexpr int kSlotsSep = 75;

struct Front {
  int parent = -1;
  int depth = 0;
  int child[2] = {-1, -1};
  int nchild = 0;
  int s0 = 0;        // first new index of the separator (or leaf) nodes
  int ns = 0;        // |S|
  int nb = 0;        // |B| (rows below the separator block)
  int ld = 0;        // row stride of the front panel P (>= ns, multiple of 4)
  int ldu = 0;       // row stride of the update block U (>= nb, multiple of 4)
  int ldz = 0;       // row stride of the full front inverse ZF (>= ns+nb)
  int64_t p_off = 0; // panel offset in the factor arena (elements)
  int64_t u_off = 0; // update block offset in pool (depth & 1)
  int64_t z_off = 0; // full-front inverse offset in pool (depth & 1)
  int64_t b_off = 0; // offset of the sorted B list / rmap in the index arrays
  int64_t d_off = 0; // offset of this front's inverse diagonal blocks (nb x nb each)
  int64_t w_base = 0; // offset, per right-hand side, of this front's solve vectors in its depth pool
  int box[6] = {0, 0, 0, 0, 0, 0};  // x0,x1,y0,y1,t0,t1 of the subtree box
  bool leaf = false;
};

struct Symbolic {
  int Mx = 0, Ny = 0, T = 1;
  int n = 0;
  int nslots = kSlotsS;
  int nbk = 64;                 // diagonal block size of the blocked factorisation
  int leaf_max = 0;             // largest box (nodes) kept as a leaf front
  std::vector<Front> fronts;    // post-order (children before parents)
  std::vector<int> perm;        // natural -> new
  std::vector<int> iperm;       // new -> natural
  std::vector<int> front_of;    // new index -> front id
  std::vector<int> blist;       // concatenated sorted B lists (new indices)
  std::vector<int> rmap;        // concatenated positions of B in the parent front
  std::vector<int> amap;        // natural node * nslots + slot -> panel offset (-1: none)
  std::vector<std::vector<int>> by_depth;  // front ids per depth
  int max_depth = 0;
  int64_t l_size = 0;           // factor arena (elements)
  int64_t u_pool[2] = {0, 0};   // update pools by depth parity (elements)
  int64_t z_pool[2] = {0, 0};   // full-front inverse pools by depth parity (elements)
  int64_t dinv_size = 0;        // inverse diagonal blocks (elements)
  int64_t w_pool[2] = {0, 0};   // solve-vector pools by depth parity (elements per right-hand side)
  int max_front = 0, max_ns = 0, max_nb = 0;
  double factor_flops = 0.0;    // algorithmic flops of one numeric factorisation
  double selinv_flops = 0.0;    // algorithmic flops of one selected inversion
  double nnz_l = 0.0;           // entries of L (lower, dense fronts)
};

// Stencil offset table of a layout with `nslots` slots: slot -> (dx, dy, dt).
void slot_offsets(int nslots, int* dx, int* dy, int* dt);

// Build the symbolic analysis for an Mx x Ny x T lattice.  `leaf_max` bounds the
// node count of an undivided box; `nbk` is the diagonal block size; `separable`
// selects the 75-slot layout (T >= 2).
int build_symbolic(int Mx, int Ny, int T, int leaf_max, int nbk, Symbolic* out, bool separable = false);

}  // namespace spde

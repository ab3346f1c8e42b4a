// The plan: symbolic analysis, device arenas, precomputed launch schedules.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "assemble.cuh"
#include "kernels.cuh"
#include "spde_internal.h"

namespace spde {

enum OpKind {
  OP_MEMSET = 0, OP_EXTEND, OP_DIAG, OP_GEMM, OP_SGATHER_FWD, OP_SGATHER_BWD, OP_ZGATHER, OP_MIRROR, OP_ZEXTRACT,
  OP_FWD_CHAIN, OP_BWD_CHAIN
};
// profile class of a tiled product that ran on the tensor cores (the others count as OP_GEMM)
constexpr int kProfTensorCore = 9;
constexpr int kProfClasses = 10;

// learned preconditioner (pcg.cu): 42 features, two hidden layers of 32, 27 stencil weights
constexpr int kPcFeat = 42, kPcHidden = 32, kPcOffsets = 27;
constexpr int kPcParams = kPcHidden * kPcFeat + kPcHidden + kPcHidden * kPcHidden + kPcHidden +
                          kPcOffsets * kPcHidden + kPcOffsets;
enum BufId { B_NONE = 0, B_L, B_DINV, B_P0, B_P1, B_X, B_W0, B_W1, B_G0, B_G1, B_SX };

// Call sites of the tiled product (for per-site timing).
enum GemmSite {
  S_NONE = 0, S_F_TRSM, S_F_UPD, S_F_SYRK, S_V_FWD_D, S_V_FWD_S, S_V_FWD_B, S_V_BWD_0, S_V_BWD_D, S_V_BWD_U,
  S_Z_XSOLVE, S_Z_XUPD, S_Z_BS, S_Z_XJ, S_Z_RJ, S_Z_JJ, S_Z_JJ2, S_Z_SS, S_COUNT
};

struct Op {
  double flops = 0.0;  // algorithmic flops of a GEMM launch (2 m n k summed over its tiles)
  int site = 0;
  int tc = 1;          // product path (GemmPath): CUDA-core tiles, tensor-core tiles (FP32), narrow
  int nmax = 0;        // largest task n of a narrow launch
  int kind = 0;
  int64_t off = 0;  // first task in the array of this kind
  int count = 0;
  int mode = 0, al = 0, bl = 0;
  int abuf = B_NONE, bbuf = B_NONE, cbuf = B_NONE;
  int64_t elems = 0;  // memset length
  int depth = 0;
};

// 32 x 32 block copy, rows x cols of src: dst[j*ldd + i] = src[i*lds + j] when
// trans, else dst[i*ldd + j] = src[i*lds + j].
struct MirrorTask {
  int64_t src, dst;
  int lds, ldd, rows, cols, trans;
};
// Front-wide task over a row range (gathers, extraction).
struct RowTask {
  int front, r0, r1;
};

// A TMA tensor map the cluster-pair product reads an operand through: the
// row-major region of buffer `buf` starting at element `base`, row stride `ld`
// (both multiples of 4), rows up to the end of the buffer.
struct MapReq {
  int buf;
  int64_t base;
  int ld;
};

struct Schedule {
  std::vector<Op> ops;
  std::vector<GemmTask> gemm;
  std::vector<DiagTask> diag;
  std::vector<ExtendTask> ext;
  std::vector<RowTask> rows;
  std::vector<MirrorTask> mirror;
  std::vector<MapReq> maps;
  std::map<std::tuple<int, int64_t, int>, int> map_index;
  // device copies
  GemmTask* d_gemm = nullptr;
  DiagTask* d_diag = nullptr;
  ExtendTask* d_ext = nullptr;
  RowTask* d_rows = nullptr;
  MirrorTask* d_mirror = nullptr;
  CUtensorMap* d_maps = nullptr;
  int launches = 0;
  void upload();
  void release();
};

// Separable models Q = Qt (x) Qs: the tridiagonal AR(1) precision Qt as its end
// diagonal, interior diagonal and off-diagonal, from the temporal parameters
// (p1, p2) of the canonical vector, and their derivatives in p1 (d1) and p2 (d2):
//   temporal 1 (seperable_spatial_temporal2D.py:186-212): rho = exp(p1),
//     (1, 1 + rho^2, -rho) / (1 - rho^2); p2 unused;
//   temporal 2 (seperable_spatial_temporal_idiffusion2D.py:166-189): a = p1,
//     sigma = exp(p2), (sigma, (1 + a^2) sigma, -a sigma).
// Returns false when rho >= 1 (Qt would not be positive definite).
inline bool separable_qt(int temporal, double p1, double p2, double* qt, double* d1 = nullptr,
                         double* d2 = nullptr) {
  double e1[3], e2[3];
  if (temporal == 1) {
    const double rho = std::exp(p1), r2 = rho * rho, q = 1.0 - r2;
    if (!(q > 0.0)) return false;
    qt[0] = 1.0 / q; qt[1] = (1.0 + r2) / q; qt[2] = -rho / q;
    // rho d/drho
    e1[0] = 2.0 * r2 / (q * q); e1[1] = 4.0 * r2 / (q * q); e1[2] = -rho * (1.0 + r2) / (q * q);
    e2[0] = e2[1] = e2[2] = 0.0;
  } else {
    const double a = p1, sigma = std::exp(p2);
    qt[0] = sigma; qt[1] = (1.0 + a * a) * sigma; qt[2] = -a * sigma;
    e1[0] = 0.0; e1[1] = 2.0 * a * sigma; e1[2] = -sigma;
    e2[0] = qt[0]; e2[1] = qt[1]; e2[2] = qt[2];
  }
  for (int i = 0; i < 3; ++i) {
    if (d1) d1[i] = e1[i];
    if (d2) d2[i] = e2[i];
  }
  return true;
}

// The spatial operator of a separable model: its model description as T == 1.
inline DevModel spatial_view(const DevModel& m) {
  DevModel s = m;
  s.T = 1;
  s.adv = 0;
  s.nw = 0;
  return s;
}

struct Plan {
  Symbolic sym;
  int device = 0;     // CUDA device current when the plan was created
  int precision = 1;  // 0: FP64 throughout ("plain"); 1: FP32 factor, FP64 pivots/refinement ("mixed")
  int tile_m = 64, tile_n = 64;
  // wall-clock limit of the tensor-core kernels' pipeline waits (failure-detection tests lower it)
  unsigned long long tc_wait_ns = kTcWaitNs;
  cudaStream_t stream = nullptr;
  // symbolic data on the device
  DevFront* d_fronts = nullptr;
  int *d_perm = nullptr, *d_iperm = nullptr, *d_front_of = nullptr, *d_blist = nullptr, *d_rmap = nullptr;
  int* d_amap = nullptr;
  // numeric arenas (element type = double for precision 0, float for 1)
  void* d_L = nullptr;
  void* d_dinv = nullptr;
  void* d_pool[2] = {nullptr, nullptr};
  void* d_sx = nullptr;  // selected-inversion scratch (triangular inverse, X^T)
  int64_t pool_elems[2] = {0, 0};
  double* d_logpiv = nullptr;
  int* d_err = nullptr;
  // one-column triangular sweeps (engine.cu, fwd_chain_kernel / bwd_chain_kernel):
  // word 0 the block ticket counter, words 64.. one completion flag per 64-row
  // block of every front (the epoch of the sweep that finished it); the error
  // word is set when a wait on a flag gives up
  unsigned* d_chain = nullptr;
  unsigned chain_epoch = 0;
  int* d_chain_err = nullptr;
  double* d_scalar = nullptr;  // small reduction outputs
  double* d_part = nullptr;    // block partial sums (1024)
  // page-locked host buffer for the scalars and partial sums read back during a
  // factorisation, solve or inversion: doubles 0-1023 partial sums, 1024 the
  // log-pivot sum; ints at double 1536: the pivot error, the tensor-core flag
  double* h_pin = nullptr;
  int* pin_int() { return reinterpret_cast<int*>(h_pin + 1536); }
  // model / assembly state (FP64)
  DevModel model{};
  bool model_set = false;
  double *d_bs = nullptr, *d_bsH = nullptr, *d_bsA = nullptr, *d_ww = nullptr, *d_theta = nullptr;
  double *d_Ageo = nullptr, *d_A0geo = nullptr, *d_kap = nullptr, *d_qs = nullptr;
  double *d_Q0 = nullptr, *d_QA = nullptr, *d_QO = nullptr, *d_cQs = nullptr;
  bool assembled = false;
  double cfac = 1.0;
  // separable models (sym.nslots == kSlotsSep): Qt end / interior diagonal and
  // off-diagonal, and the temporal parametrisation (1: log rho, 2: a, log sigma)
  int temporal = 0;
  double qt[3] = {0.0, 0.0, 0.0};
  std::vector<double> theta;
  // observations
  double* d_obs_cnt = nullptr;  // per natural node: summed observation weights (the count when unweighted)
  int* d_obs_idx = nullptr;   // observed natural nodes (m)
  int nobs = 0;
  // the distinct observed nodes as a bitmask over the nodes (bit p & 31 of word
  // p >> 5), the number of set bits before each word, and their list in node
  // order: the learned preconditioner's compact weights give observed nodes
  // their own rows (the observation term changes their row of A)
  uint32_t* d_obs_mask = nullptr;
  int* d_obs_rank = nullptr;
  int* d_obs_nodes = nullptr;
  int nob = 0;
  int obs_version = 0;  // incremented by every new observation set
  // factor state
  int factored = 0;  // 0 none, 1 Q, 2 Q + tau S^T S
  double factored_tau = 0.0;
  double logdet = 0.0;
  // schedules
  Schedule sched_factor, sched_selinv;
  std::map<int, std::unique_ptr<Schedule>> sched_fwd, sched_bwd;
  // solve buffers (sized for the largest nrhs seen)
  int solve_cap = 0;
  void* d_X = nullptr;
  void* d_W[2] = {nullptr, nullptr};
  void* d_G[2] = {nullptr, nullptr};
  int64_t w_elems_per_rhs[2] = {0, 0};
  double *d_r = nullptr, *d_x64 = nullptr, *d_b64 = nullptr;
  int64_t r_cap = 0;
  // counters and optional per-launch timing (CUDA events on the plan's stream)
  int64_t launches_total = 0;
  bool profile = false;
  bool profile_tc_only = false;  // time only the tensor-core products
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, double>> ev_pending;  // (op kind, flops) per recorded pair
  size_t ev_used = 0;
  double prof_ms[16] = {0};
  double prof_flops[16] = {0};
  int64_t prof_count[16] = {0};
  double site_ms[S_COUNT] = {0};
  double site_flops[S_COUNT] = {0};
  int64_t site_tiles[S_COUNT] = {0};
  std::vector<int> ev_site;
  std::string last_error;
  // iterative solver / preconditioner scratch (pcg.cu)
  void* d_pc = nullptr;
  size_t pc_cap = 0;
  void* d_pc32 = nullptr;  // FP32 PCG scratch (vectors and coefficient copies)
  size_t pc32_cap = 0;

  QStencil qstencil() const {
    QStencil q;
    q.Q0 = d_Q0; q.QA = d_QA; q.QO = d_QO; q.cQs = d_cQs;
    q.Mx = sym.Mx; q.Ny = sym.Ny; q.T = sym.T; q.Ns = sym.Mx * sym.Ny;
    q.sep = sym.nslots == kSlotsSep ? 1 : 0;
    q.qt_end = qt[0]; q.qt_mid = qt[1]; q.qt_off = qt[2];
    return q;
  }
  size_t esize() const { return precision == 0 ? sizeof(double) : sizeof(float); }
};

// engine entry points used by the C ABI
int plan_build(Plan* p);
int plan_factor(Plan* p, int with_obs, double tau);
int plan_solve(Plan* p, const double* b_dev, double* x_dev, int nrhs, int refine_iters, double tol, double* resid);
int plan_selinv(Plan* p, double* zq_dev);
int plan_sample(Plan* p, const double* z_dev, double* x_dev, int nrhs);
void prof_collect(Plan* p);

// learned preconditioner and PCG (pcg.cu)
int pc_weights(Plan* p, int with_obs, double tau, const float* prm, float* w, float* act);
int pc_grad(Plan* p, int with_obs, double tau, const float* prm, const float* w, const float* act, const double* z,
            int k, double* loss, float* grad);
int pc_adam(const float* g, float* prm, float* m, float* v, int n, float lr, float b1, float b2, float eps, int t,
            cudaStream_t st);
int qsqrt_apply(Plan* p, int transpose, const double* x, double* y, int nrhs);
int jacobi_smooth(Plan* p, int with_obs, double tau, double omega, int sweeps, double* z, int nrhs);
int pcg_solve(Plan* p, int with_obs, double tau, int kind, const float* w, const double* b, double* x, int nrhs,
              double tol, int maxit, int check_every, int* iters, double* relres);
// learned preconditioner, compact weights: one row of G per (spatial cell, time
// class: first step, interior, last step) and one per distinct observed node
int64_t pc_compact_floats(const Plan* p);
int pc_weights_compact(Plan* p, int with_obs, double tau, const float* prm, float* w);

// adjoint (adjoint.cu)
void launch_adjoint(const Plan* p, const double* gbar, double* grad_dev, double* work, cudaStream_t st);
// doubles of adjoint work per spatial cell: 84 reduced stencil values + 22 partials
constexpr int64_t kAdjointCellElems = 106;
int64_t adjoint_work_elems(const Plan* p);
// device address and size of the allocation-free adjoint's static scratch on
// device `dev` (looked up once per device with that device current)
int noalloc_scratch(int dev, double** ptr, int64_t* elems);

}  // namespace spde

// C ABI of libspde_gb300 (declared in include/spde_gb300.h).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <cstring>
#include <string>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "../../include/spde_gb300.h"
#include "engine.cuh"

using namespace spde;


#define API_CUDA(x)                                                      \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    if (e_ != cudaSuccess) {                                             \
      plan->p.last_error = std::string(#x) + ": " + cudaGetErrorString(e_); \
      return SPDE_ERR_CUDA;                                              \
    }                                                                    \
  } while (0)

namespace {

// relative residual the FP64 refinement of the conditional-mean solve stops at
constexpr double kRefineTol = 1e-10;

__global__ void obs_rhs_kernel(const int* __restrict__ idx, int m, int r, double tau, const double* __restrict__ y,
                               const double* __restrict__ mu0, double* __restrict__ b) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(m) * r) return;
  const int i = int(e / r), c = int(e % r);
  const int k = idx[i];
  double v = y[e];
  if (mu0) v -= mu0[int64_t(k) * r + c];
  atomicAdd(&b[int64_t(k) * r + c], tau * v);
}

// block partial sums of a[i]*b[i] (b == nullptr: a[i]^2)
__global__ void dot_partial_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                                   double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * 256 + threadIdx.x; i < n; i += int64_t(gridDim.x) * 256)
    s += b ? a[i] * b[i] : a[i] * a[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = 128; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// residual of the observations: d[i, c] = y[i, c] - mu[idx_i, c]
__global__ void obs_resid_kernel(const int* __restrict__ idx, int m, int r, const double* __restrict__ y,
                                 const double* __restrict__ mu, double* __restrict__ d) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= int64_t(m) * r) return;
  d[e] = y[e] - mu[int64_t(idx[e / r]) * r + e % r];
}

// Gbar = a * (ZQ - ZQc) - 1/2 sum_c mu mu^T on the stencil (exact traces), or with
// Hutchinson probes: a/nh1 * sym(Delta V^T) where Delta = TrQ - TrQc.
__global__ void gbar_kernel(int Mx, int Ny, int T, int nslots, double a, const double* __restrict__ zq,
                            const double* __restrict__ zqc, const double* __restrict__ dlt,
                            const double* __restrict__ V, int nh1, const double* __restrict__ mu, int r,
                            double* __restrict__ g) {
  const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = int64_t(Mx) * Ny * T;
  if (e >= n * nslots) return;
  const int k = int(e / nslots), s = int(e % nslots);
  int dx, dy, dt;
  stencil_slot(nslots, s, &dx, &dy, &dt);
  const int t = k / (Mx * Ny), c = k - t * Mx * Ny, y = c / Mx, x = c - y * Mx;
  if (x + dx < 0 || x + dx >= Mx || y + dy < 0 || y + dy >= Ny || t + dt < 0 || t + dt >= T) {
    g[e] = 0.0;
    return;
  }
  const int64_t nb = (int64_t(t + dt) * Ny + y + dy) * Mx + x + dx;
  double v = 0.0;
  if (zq) {
    v = a * (zq[e] - zqc[e]);
  } else {
    double acc = 0.0;
    for (int p = 0; p < nh1; ++p)
      acc += dlt[int64_t(k) * nh1 + p] * V[nb * nh1 + p] + dlt[nb * nh1 + p] * V[int64_t(k) * nh1 + p];
    v = a * 0.5 * acc / nh1;
  }
  double mm = 0.0;
  for (int cc = 0; cc < r; ++cc) mm += mu[int64_t(k) * r + cc] * mu[nb * r + cc];
  g[e] = v - 0.5 * mm;
}

// sum over observations of z[idx_i, centre] (exact) or sum_p TrQc[idx_i,p] V[idx_i,p]
__global__ void obs_trace_kernel(const int* __restrict__ idx, int m, const double* __restrict__ zqc, int nslots,
                                 int centre, const double* __restrict__ trc, const double* __restrict__ V, int nh1,
                                 double* __restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < m; i += gridDim.x * 256) {
    const int64_t k = idx[i];
    if (zqc) s += zqc[k * nslots + centre];
    else
      for (int p = 0; p < nh1; ++p) s += trc[k * nh1 + p] * V[k * nh1 + p];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int q = 128; q > 0; q >>= 1) {
    if (threadIdx.x < q) red[threadIdx.x] += red[threadIdx.x + q];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void sub_kernel(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) a[i] -= b[i];
}

struct DevBuf {
  double* p = nullptr;
  size_t n = 0;
  ~DevBuf() { cudaFree(p); }
  cudaError_t ensure(size_t elems) {
    if (elems <= n) return cudaSuccess;
    cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, elems * sizeof(double));
    if (e == cudaSuccess) n = elems;
    return e;
  }
};

double host_sum_partials(const double* dpart, int nblk, cudaStream_t st) {
  std::vector<double> h(nblk);
  cudaMemcpyAsync(h.data(), dpart, nblk * sizeof(double), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  double s = 0.0;
  for (double v : h) s += v;
  return s;
}

int ntheta_of(const Plan& p) { return 4 * p.model.nk + p.model.nw + 6; }

}  // namespace

// Optional phase timeline of spde_loglike: with SPDE_PHASE_LOG set, the end of
// each phase of the two pipelines (factor, solve, inverse) is recorded with a
// CUDA event on the phase's stream and printed to stderr in ms from the end of
// the assembly.
struct PhaseLog {
  bool on = false;
  cudaEvent_t t0 = nullptr;
  std::vector<std::pair<const char*, cudaEvent_t>> marks;
  std::mutex mu;
  explicit PhaseLog(cudaStream_t st) {
    on = std::getenv("SPDE_PHASE_LOG") != nullptr;
    if (!on) return;
    cudaEventCreate(&t0);
    cudaEventRecord(t0, st);
  }
  void mark(const char* what, cudaStream_t st) {
    if (!on) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, st);
    std::lock_guard<std::mutex> g(mu);
    marks.emplace_back(what, e);
  }
  ~PhaseLog() {
    if (!on) return;
    std::string line = "phases (ms):";
    for (auto& m : marks) {
      float ms = 0.0f;
      cudaEventSynchronize(m.second);
      cudaEventElapsedTime(&ms, t0, m.second);
      char buf[96];
      std::snprintf(buf, sizeof(buf), " %s %.2f", m.first, ms);
      line += buf;
      cudaEventDestroy(m.second);
    }
    cudaEventDestroy(t0);
    std::fprintf(stderr, "%s\n", line.c_str());
  }
};

struct LoglikeScratch {
  DevBuf zq, zqc, b, mu, qmu, part, gbar, gradv, work, trq, trc, d;
};

struct SpdePlan {
  Plan p;
  LoglikeScratch s;
  // Second pipeline of spde_loglike: Q + tau S^T S is factored, solved and
  // inverted on its own arenas and stream while Q runs on the plan's own, so the
  // latency-bound top levels of the two overlap.  It shares the assembled model
  // and the observations of `p` (read only) and is built on first use.
  std::unique_ptr<Plan> twin;
  int pipelines = 2;
  // phase streams of the two pipelines: [pipeline][0 factor / solve, 1 inverse],
  // and the events that order a pipeline's phases across them
  cudaStream_t phase[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  cudaEvent_t phase_ev[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
};

// Moves a plan's subsequent work to stream `to`, after everything enqueued so far.
static void move_to(Plan* p, cudaStream_t to, cudaEvent_t ev) {
  if (to == p->stream) return;
  cudaEventRecord(ev, p->stream);
  cudaStreamWaitEvent(to, ev, 0);
  p->stream = to;
}

// Creates the phase streams: the factorisations and the solve, chains of
// latency-bound launches, at the greatest priority; the selected inversions,
// long runs of large tensor-core products, at the least, so that they fill the
// SMs the chains leave idle without delaying them.
static int ensure_phase_streams(SpdePlan* plan) {
  if (plan->phase[0][0]) return SPDE_OK;
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  for (int q = 0; q < 2; ++q)
    for (int k = 0; k < 2; ++k)
      if (cudaStreamCreateWithPriority(&plan->phase[q][k], cudaStreamNonBlocking, k == 0 ? greatest : least) !=
          cudaSuccess)
        return SPDE_ERR_CUDA;
  for (int q = 0; q < 2; ++q)
    for (int k = 0; k < 3; ++k)
      if (cudaEventCreateWithFlags(&plan->phase_ev[q][k], cudaEventDisableTiming) != cudaSuccess) return SPDE_ERR_CUDA;
  return SPDE_OK;
}

extern "C" {

int spde_diffusion_triplets(int M, int N, const double* H, int field, double hx, double hy, int bc, int* row, int* col,
                            double* val, void* stream) {
  if (M < 1 || N < 1 || (bc != 1 && bc != 3) || !H || !row || !col || !val) return SPDE_ERR_ARG;
  launch_diffusion_triplets(M, N, H, field, hx, hy, bc, row, col, val, static_cast<cudaStream_t>(stream));
  return cudaGetLastError() == cudaSuccess ? SPDE_OK : SPDE_ERR_CUDA;
}

int spde_advection_triplets(int M, int N, const double* G, const double* dG, int field, double hx, double hy, int bc,
                            int diff, int* row, int* col, double* val, void* stream) {
  if (M < 1 || N < 1 || (bc != 1 && bc != 3) || diff < 1 || diff > 3 || !G || !row || !col || !val)
    return SPDE_ERR_ARG;
  launch_advection_triplets(M, N, G, dG, field, hx, hy, bc, diff, row, col, val, static_cast<cudaStream_t>(stream));
  return cudaGetLastError() == cudaSuccess ? SPDE_OK : SPDE_ERR_CUDA;
}

static void fill_info(const Symbolic& S, SpdePlanInfo* info) {
  info->n = S.n;
  info->nfronts = int64_t(S.fronts.size());
  info->max_depth = S.max_depth;
  info->max_front = S.max_front;
  info->nslots = S.nslots;
  info->factor_flops = S.factor_flops;
  info->selinv_flops = S.selinv_flops;
  info->nnz_l = S.nnz_l;
}

int spde_symbolic_info(int Mx, int Ny, int T, int leaf_max, SpdePlanInfo* info) {
  if (!info) return SPDE_ERR_ARG;
  Symbolic S;
  if (build_symbolic(Mx, Ny, T, leaf_max, 64, &S) != 0) return SPDE_ERR_ARG;
  std::memset(info, 0, sizeof(*info));
  fill_info(S, info);
  info->precision = -1;
  info->bytes_factor = double(S.l_size);
  info->bytes_work = double(std::max(S.u_pool[0], S.z_pool[0]) + std::max(S.u_pool[1], S.z_pool[1]));
  return SPDE_OK;
}

int spde_symbolic_export(int Mx, int Ny, int T, int leaf_max, int32_t* perm, int32_t* front_ns, int32_t* front_nb,
                         int32_t* front_parent, int64_t cap) {
  Symbolic S;
  if (build_symbolic(Mx, Ny, T, leaf_max, 64, &S) != 0) return SPDE_ERR_ARG;
  if (perm) std::memcpy(perm, S.perm.data(), S.perm.size() * sizeof(int32_t));
  if (int64_t(S.fronts.size()) > cap) return SPDE_ERR_ARG;
  for (size_t f = 0; f < S.fronts.size(); ++f) {
    if (front_ns) front_ns[f] = S.fronts[f].ns;
    if (front_nb) front_nb[f] = S.fronts[f].nb;
    if (front_parent) front_parent[f] = S.fronts[f].parent;
  }
  return SPDE_OK;
}

// Frees what plan_build and the solve / iterative paths allocated for a plan
// (not its model or observation arrays).
static void release_numeric(Plan& p) {
  void* ptrs[] = {p.d_fronts, p.d_perm, p.d_iperm, p.d_front_of, p.d_blist, p.d_rmap, p.d_amap, p.d_L, p.d_dinv,
                  p.d_pool[0], p.d_pool[1], p.d_logpiv, p.d_err, p.d_scalar, p.d_X, p.d_W[0], p.d_W[1], p.d_G[0],
                  p.d_G[1], p.d_r, p.d_x64, p.d_b64, p.d_part, p.d_sx, p.d_pc, p.d_chain, p.d_chain_err};
  for (void* q : ptrs) cudaFree(q);
  cudaFreeHost(p.h_pin);
  p.h_pin = nullptr;
  for (cudaEvent_t e : p.ev_pool) cudaEventDestroy(e);
  p.ev_pool.clear();
  p.sched_factor.release();
  p.sched_selinv.release();
  for (auto& kv : p.sched_fwd) kv.second->release();
  for (auto& kv : p.sched_bwd) kv.second->release();
}

static void destroy_twin(SpdePlan* plan) {
  if (!plan->twin) return;
  Plan& t = *plan->twin;
  cudaStreamSynchronize(t.stream);
  release_numeric(t);
  if (t.stream) cudaStreamDestroy(t.stream);
  plan->twin.reset();
}

static int ensure_twin(SpdePlan* plan) {
  if (plan->twin) return SPDE_OK;
  Plan& p = plan->p;
  std::unique_ptr<Plan> t(new (std::nothrow) Plan());
  if (!t) return SPDE_ERR_NO_MEMORY;
  t->precision = p.precision;
  t->sym = p.sym;
  // the second pipeline carries the conditional-mean solve, a chain of small
  // latency-bound launches on the evaluation's critical path: highest priority
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (cudaStreamCreateWithPriority(&t->stream, cudaStreamNonBlocking, greatest) != cudaSuccess) {
    p.last_error = "could not create the second pipeline's stream";
    return SPDE_ERR_CUDA;
  }
  const int rc = plan_build(t.get());
  if (rc) {
    p.last_error = "second pipeline: " + t->last_error;
    release_numeric(*t);
    cudaStreamDestroy(t->stream);
    return rc == 4 ? SPDE_ERR_NO_MEMORY : SPDE_ERR_CUDA;
  }
  plan->twin = std::move(t);
  return SPDE_OK;
}

// The twin reads the plan's assembled model and observations (same device arrays).
static void share_model(const Plan& p, Plan& t) {
  t.model = p.model;
  t.model_set = p.model_set;
  t.d_Q0 = p.d_Q0; t.d_QA = p.d_QA; t.d_QO = p.d_QO; t.d_cQs = p.d_cQs;
  t.cfac = p.cfac;
  t.temporal = p.temporal;
  t.qt[0] = p.qt[0]; t.qt[1] = p.qt[1]; t.qt[2] = p.qt[2];
  t.assembled = p.assembled;
  t.d_obs_cnt = p.d_obs_cnt;
  t.d_obs_idx = p.d_obs_idx;
  t.nobs = p.nobs;
  t.profile = p.profile;
  t.profile_tc_only = p.profile_tc_only;
  t.tc_wait_ns = p.tc_wait_ns;
}

// The learned preconditioner reads the 43-slot spatio-temporal stencil and the
// square root of Q is the implicit-Euler factor: neither applies to separable plans.
static int not_separable(Plan& p, const char* what) {
  if (p.sym.nslots != kSlotsSep) return SPDE_OK;
  p.last_error = std::string(what) + " is not available for separable models";
  return SPDE_ERR_STATE;
}

static int no_factor(SpdePlan* plan) {
  plan->p.last_error = "this plan was created for iterative solves only (no factorisation)";
  return SPDE_ERR_STATE;
}

static int plan_create(int Mx, int Ny, int T, int precision, int leaf_max, bool separable, SpdePlan** out) {
  if (!out || precision < 0 || precision > 2) return SPDE_ERR_ARG;
  if (separable && (precision == SPDE_PRECISION_ITERATIVE || T < 2)) return SPDE_ERR_ARG;
  *out = nullptr;
  SpdePlan* plan = new (std::nothrow) SpdePlan();
  if (!plan) return SPDE_ERR_NO_MEMORY;
  plan->p.precision = precision;
  if (cudaGetDevice(&plan->p.device) != cudaSuccess) plan->p.device = 0;
  if (precision == SPDE_PRECISION_ITERATIVE) {
    // assembly, products and iterative solves only: no ordering, no factor arenas
    if (Mx < 3 || Ny < 3 || T < 1 || int64_t(Mx) * Ny * T > (int64_t(1) << 31) - 1) {
      delete plan;
      return SPDE_ERR_ARG;
    }
    Symbolic& S = plan->p.sym;
    S.Mx = Mx; S.Ny = Ny; S.T = T; S.n = Mx * Ny * T; S.nslots = T == 1 ? 25 : 43;
    *out = plan;
    return SPDE_OK;
  }
  if (build_symbolic(Mx, Ny, T, leaf_max > 0 ? leaf_max : 128, 64, &plan->p.sym, separable) != 0) {
    delete plan;
    return SPDE_ERR_ARG;
  }
  int rc = plan_build(&plan->p);
  if (rc != 0) {
    spde_plan_destroy(plan);
    return rc == 4 ? SPDE_ERR_NO_MEMORY : SPDE_ERR_CUDA;
  }
  *out = plan;
  return SPDE_OK;
}

int spde_plan_create(int Mx, int Ny, int T, int precision, int leaf_max, SpdePlan** out) {
  return plan_create(Mx, Ny, T, precision, leaf_max, false, out);
}

int spde_plan_create_separable(int Mx, int Ny, int T, int precision, int leaf_max, SpdePlan** out) {
  return plan_create(Mx, Ny, T, precision, leaf_max, true, out);
}

int spde_plan_destroy(SpdePlan* plan) {
  if (!plan) return SPDE_OK;
  destroy_twin(plan);
  Plan& p = plan->p;
  cudaStreamSynchronize(p.stream);
  for (auto& row : plan->phase)
    for (cudaStream_t& q : row)
      if (q) { cudaStreamSynchronize(q); cudaStreamDestroy(q); }
  for (auto& row : plan->phase_ev)
    for (cudaEvent_t& e : row)
      if (e) cudaEventDestroy(e);
  void* ptrs[] = {p.d_fronts, p.d_perm, p.d_iperm, p.d_front_of, p.d_blist, p.d_rmap, p.d_amap, p.d_L, p.d_dinv,
                  p.d_pool[0], p.d_pool[1], p.d_logpiv, p.d_err, p.d_scalar, p.d_bs, p.d_bsH, p.d_bsA, p.d_ww,
                  p.d_theta, p.d_Ageo, p.d_A0geo, p.d_kap, p.d_qs, p.d_Q0, p.d_QA, p.d_QO, p.d_cQs, p.d_obs_cnt,
                  p.d_obs_idx, p.d_X, p.d_W[0], p.d_W[1], p.d_G[0], p.d_G[1], p.d_r, p.d_x64, p.d_b64,
                  p.d_obs_mask, p.d_obs_rank, p.d_obs_nodes, p.d_pc32, p.d_chain, p.d_chain_err};
  for (void* q : ptrs) cudaFree(q);
  cudaFreeHost(p.h_pin);
  p.h_pin = nullptr;
  cudaFree(p.d_part);
  cudaFree(p.d_sx);
  cudaFree(p.d_pc);
  for (cudaEvent_t e : p.ev_pool) cudaEventDestroy(e);
  p.sched_factor.release();
  p.sched_selinv.release();
  for (auto& kv : p.sched_fwd) kv.second->release();
  for (auto& kv : p.sched_bwd) kv.second->release();
  delete plan;
  return SPDE_OK;
}

int spde_plan_set_stream(SpdePlan* plan, void* stream) {
  if (!plan) return SPDE_ERR_ARG;
  plan->p.stream = static_cast<cudaStream_t>(stream);
  return SPDE_OK;
}

int spde_plan_info(const SpdePlan* plan, SpdePlanInfo* info) {
  if (!plan || !info) return SPDE_ERR_ARG;
  const Plan& p = plan->p;
  std::memset(info, 0, sizeof(*info));
  fill_info(p.sym, info);
  info->precision = p.precision;
  info->bytes_factor = double(p.sym.l_size) * p.esize();
  info->bytes_work = double(p.pool_elems[0] + p.pool_elems[1]) * p.esize();
  info->launches = p.launches_total + (plan->twin ? plan->twin->launches_total : 0);
  return SPDE_OK;
}

const char* spde_last_error(const SpdePlan* plan) { return plan ? plan->p.last_error.c_str() : "null plan"; }

int spde_plan_set_profiling(SpdePlan* plan, int enable) {
  if (!plan) return SPDE_ERR_ARG;
  if (enable < 0 || enable > 2) return SPDE_ERR_ARG;
  Plan* ps[2] = {&plan->p, plan->twin.get()};
  for (Plan* q : ps) {
    if (!q) continue;
    prof_collect(q);
    q->profile = enable != 0;
    q->profile_tc_only = enable == 2;
  }
  return SPDE_OK;
}

int spde_plan_read_sites(SpdePlan* plan, double* ms, double* flops, int64_t* tiles, int reset) {
  if (!plan) return SPDE_ERR_ARG;
  Plan* ps[2] = {&plan->p, plan->twin.get()};
  for (Plan* q : ps)
    if (q) prof_collect(q);
  for (int k = 0; k < S_COUNT; ++k) {
    double a = 0.0, b = 0.0;
    int64_t c = 0;
    for (Plan* q : ps) {
      if (!q) continue;
      a += q->site_ms[k]; b += q->site_flops[k]; c += q->site_tiles[k];
      if (reset) { q->site_ms[k] = 0; q->site_flops[k] = 0; q->site_tiles[k] = 0; }
    }
    if (ms) ms[k] = a;
    if (flops) flops[k] = b;
    if (tiles) tiles[k] = c;
  }
  return SPDE_OK;
}

int spde_plan_read_profile(SpdePlan* plan, double* ms, double* flops, int64_t* count, int reset) {
  if (!plan) return SPDE_ERR_ARG;
  Plan* ps[2] = {&plan->p, plan->twin.get()};
  for (Plan* q : ps)
    if (q) prof_collect(q);
  for (int k = 0; k < kProfClasses; ++k) {
    double a = 0.0, b = 0.0;
    int64_t c = 0;
    for (Plan* q : ps) {
      if (!q) continue;
      a += q->prof_ms[k]; b += q->prof_flops[k]; c += q->prof_count[k];
      if (reset) { q->prof_ms[k] = 0; q->prof_flops[k] = 0; q->prof_count[k] = 0; }
    }
    if (ms) ms[k] = a;
    if (flops) flops[k] = b;
    if (count) count[k] = c;
  }
  return SPDE_OK;
}

int spde_set_model(SpdePlan* plan, const SpdeModelDesc* d) {
  if (!plan || !d) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (d->Mx != p.sym.Mx || d->Ny != p.sym.Ny || d->T != p.sym.T) { p.last_error = "grid mismatch"; return SPDE_ERR_ARG; }
  if ((d->bc != 1 && d->bc != 3) || d->diff_form < 0 || d->diff_form > 2 || d->adv < 0 || d->adv > 3) {
    p.last_error = "unsupported model flags";
    return SPDE_ERR_ARG;
  }
  const bool sep = p.sym.nslots == kSlotsSep;
  if (sep) {
    if (d->adv != 0 || (d->temporal != 1 && d->temporal != 2)) {
      p.last_error = "a separable plan needs a model without advection and temporal = 1 (rho) or 2 (a, sigma)";
      return SPDE_ERR_ARG;
    }
  } else if (d->temporal != 0) {
    p.last_error = "separable models need a plan from spde_plan_create_separable";
    return SPDE_ERR_ARG;
  } else if ((d->T == 1) != (d->adv == 0)) {
    p.last_error = "spatial models have no advection, spatio-temporal ones do";
    return SPDE_ERR_ARG;
  }
  p.temporal = d->temporal;
  const int Ns = d->Mx * d->Ny;
  const int nb = std::max(d->nbasis, 1);
  auto up = [&](double*& dst, const double* src, size_t n) -> int {
    cudaFree(dst);
    dst = nullptr;
    if (!src) return 0;
    if (cudaMalloc(&dst, n * sizeof(double)) != cudaSuccess) return 1;
    return cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess;
  };
  if ((d->var_h && (!d->bs || !d->bsH)) || (d->adv == 2 && !d->bsA) || (d->adv == 3 && !d->ww)) {
    p.last_error = "missing basis or velocity field";
    return SPDE_ERR_ARG;
  }
  if (up(p.d_bs, d->var_h ? d->bs : nullptr, size_t(Ns) * nb) || up(p.d_bsH, d->var_h ? d->bsH : nullptr, size_t(Ns) * 4 * nb) ||
      up(p.d_bsA, d->adv == 2 ? d->bsA : nullptr, size_t(Ns) * 4 * nb) || up(p.d_ww, d->adv == 3 ? d->ww : nullptr, size_t(Ns) * 4)) {
    p.last_error = "device allocation failed (model)";
    return SPDE_ERR_NO_MEMORY;
  }
  DevModel& m = p.model;
  m.Mx = d->Mx; m.Ny = d->Ny; m.T = d->T; m.Ns = Ns; m.bc = d->bc; m.mod0_bc = d->mod0_bc ? d->mod0_bc : d->bc;
  m.hx = d->hx; m.hy = d->hy; m.dt = d->dt; m.V = d->hx * d->hy;
  m.diff = d->diff_form; m.mod0_diff = d->mod0_diff_form; m.var_h = d->var_h; m.adv = d->adv; m.nbasis = nb;
  m.nk = d->var_h ? nb : 1;
  m.nw = d->adv == 1 ? 2 : d->adv == 2 ? 2 * nb : d->adv == 3 ? 1 : 0;
  m.bs = p.d_bs; m.bsH = p.d_bsH; m.bsA = p.d_bsA; m.ww = p.d_ww;
  double** arrs9[] = {&p.d_Ageo, &p.d_A0geo};
  for (double** a : arrs9) { cudaFree(*a); API_CUDA(cudaMalloc(a, size_t(Ns) * 9 * sizeof(double))); }
  double** arrs1[] = {&p.d_kap, &p.d_qs, &p.d_cQs};
  for (double** a : arrs1) { cudaFree(*a); API_CUDA(cudaMalloc(a, size_t(Ns) * sizeof(double))); }
  cudaFree(p.d_Q0); API_CUDA(cudaMalloc(&p.d_Q0, size_t(Ns) * 25 * sizeof(double)));
  cudaFree(p.d_QA); API_CUDA(cudaMalloc(&p.d_QA, size_t(Ns) * 25 * sizeof(double)));
  cudaFree(p.d_QO); API_CUDA(cudaMalloc(&p.d_QO, size_t(Ns) * 9 * sizeof(double)));
  cudaFree(p.d_theta); API_CUDA(cudaMalloc(&p.d_theta, size_t(ntheta_of(p)) * sizeof(double)));
  m.theta = p.d_theta;
  p.model_set = true;
  p.assembled = false;
  p.factored = 0;
  return SPDE_OK;
}

int spde_assemble(SpdePlan* plan, const double* theta, int ntheta) {
  if (!plan || !theta) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.model_set) { p.last_error = "set a model first"; return SPDE_ERR_STATE; }
  if (ntheta != ntheta_of(p)) { p.last_error = "theta length does not match the model"; return SPDE_ERR_ARG; }
  for (int i = 0; i < ntheta; ++i)
    if (!std::isfinite(theta[i])) { p.last_error = "non-finite parameter"; return SPDE_ERR_ARG; }
  p.theta.assign(theta, theta + ntheta);
  API_CUDA(cudaMemcpyAsync(p.d_theta, theta, ntheta * sizeof(double), cudaMemcpyHostToDevice, p.stream));
  const int to = 4 * p.model.nk + p.model.nw;  // log sigma, or the first temporal parameter
  if (p.temporal) {
    // Q = Qt (x) Qs: Qs through the spatial assembly, Qt from the temporal
    // parameters (spdes/seperable_spatial_temporal2D.py:186-212,
    // seperable_spatial_temporal_idiffusion2D.py:166-189)
    if (!separable_qt(p.temporal, theta[to], theta[to + 1], p.qt)) {
      p.last_error = "rho = exp(par) must be below 1";
      return SPDE_ERR_ARG;
    }
    p.cfac = 1.0;
    const DevModel ms = spatial_view(p.model);
    launch_fields(ms, p.d_Ageo, p.d_A0geo, p.d_kap, p.d_qs, p.stream);
    launch_qstencil(ms, p.d_Ageo, p.d_A0geo, p.d_kap, p.d_qs, p.d_Q0, p.d_QA, p.d_QO, p.d_cQs, 1.0, p.stream);
  } else {
    p.cfac = p.sym.T > 1 ? 1.0 / (p.model.dt * std::exp(theta[to])) : 1.0;
    launch_fields(p.model, p.d_Ageo, p.d_A0geo, p.d_kap, p.d_qs, p.stream);
    launch_qstencil(p.model, p.d_Ageo, p.d_A0geo, p.d_kap, p.d_qs, p.d_Q0, p.d_QA, p.d_QO, p.d_cQs, p.cfac,
                    p.stream);
  }
  p.launches_total += 2;
  API_CUDA(cudaGetLastError());
  p.assembled = true;
  p.factored = 0;
  return SPDE_OK;
}

int spde_export_q(SpdePlan* plan, int with_obs, double tau, double* q) {
  if (!plan || !q) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (with_obs && !p.d_obs_cnt) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  launch_qexport(p.qstencil(), p.sym.nslots, with_obs ? p.d_obs_cnt : nullptr, tau, q, p.stream);
  API_CUDA(cudaGetLastError());
  return SPDE_OK;
}

int spde_spmv(SpdePlan* plan, int with_obs, double tau, const double* x, double* y, int nrhs) {
  if (!plan || !x || !y || nrhs < 1) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (with_obs && !p.d_obs_cnt) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  launch_spmv(p.qstencil(), with_obs ? p.d_obs_cnt : nullptr, tau, x, y, nrhs, p.stream);
  API_CUDA(cudaGetLastError());
  return SPDE_OK;
}

// Observation set with per-observation weights (nullptr: 1 each): node k's
// weight is the sum over the observations at k, so tau * weight is what
// tau S^T S adds to Q's diagonal.
static int set_obs(SpdePlan* plan, const int64_t* idx, const double* wts, int m) {
  if (!plan || (m > 0 && !idx) || m < 0) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  std::vector<double> cnt(p.sym.n, 0.0);
  std::vector<int> id(std::max(m, 1), 0);
  for (int i = 0; i < m; ++i) {
    if (idx[i] < 0 || idx[i] >= p.sym.n) { p.last_error = "observation index out of range"; return SPDE_ERR_ARG; }
    if (wts && !(std::isfinite(wts[i]) && wts[i] >= 0.0)) {
      p.last_error = "observation weights must be finite and non-negative";
      return SPDE_ERR_ARG;
    }
    cnt[idx[i]] += wts ? wts[i] : 1.0;
    id[i] = int(idx[i]);
  }
  // distinct observed nodes: bitmask, per-word rank and list (node order)
  const int64_t nwords = (int64_t(p.sym.n) + 31) / 32;
  std::vector<uint32_t> mask(nwords, 0u);
  std::vector<int> rank(nwords, 0), nodes;
  for (int64_t k = 0; k < p.sym.n; ++k)
    if (cnt[k] > 0.0) {
      mask[k >> 5] |= 1u << (k & 31);
      nodes.push_back(int(k));
    }
  for (int64_t w = 1; w < nwords; ++w) rank[w] = rank[w - 1] + __builtin_popcount(mask[w - 1]);
  if (nodes.empty()) nodes.push_back(0);
  cudaFree(p.d_obs_cnt); cudaFree(p.d_obs_idx);
  cudaFree(p.d_obs_mask); cudaFree(p.d_obs_rank); cudaFree(p.d_obs_nodes);
  p.d_obs_cnt = nullptr; p.d_obs_idx = nullptr;
  p.d_obs_mask = nullptr; p.d_obs_rank = nullptr; p.d_obs_nodes = nullptr;
  p.nob = 0;
  API_CUDA(cudaMalloc(&p.d_obs_cnt, cnt.size() * sizeof(double)));
  API_CUDA(cudaMalloc(&p.d_obs_idx, id.size() * sizeof(int)));
  API_CUDA(cudaMemcpy(p.d_obs_cnt, cnt.data(), cnt.size() * sizeof(double), cudaMemcpyHostToDevice));
  API_CUDA(cudaMemcpy(p.d_obs_idx, id.data(), id.size() * sizeof(int), cudaMemcpyHostToDevice));
  API_CUDA(cudaMalloc(&p.d_obs_mask, size_t(nwords) * sizeof(uint32_t)));
  API_CUDA(cudaMalloc(&p.d_obs_rank, size_t(nwords) * sizeof(int)));
  API_CUDA(cudaMalloc(&p.d_obs_nodes, nodes.size() * sizeof(int)));
  API_CUDA(cudaMemcpy(p.d_obs_mask, mask.data(), size_t(nwords) * sizeof(uint32_t), cudaMemcpyHostToDevice));
  API_CUDA(cudaMemcpy(p.d_obs_rank, rank.data(), size_t(nwords) * sizeof(int), cudaMemcpyHostToDevice));
  API_CUDA(cudaMemcpy(p.d_obs_nodes, nodes.data(), nodes.size() * sizeof(int), cudaMemcpyHostToDevice));
  p.nob = mask.empty() ? 0 : rank[nwords - 1] + __builtin_popcount(mask[nwords - 1]);
  p.nobs = m;
  ++p.obs_version;
  if (p.factored == 2) p.factored = 0;
  return SPDE_OK;
}

int spde_set_obs(SpdePlan* plan, const int64_t* idx, int m) { return set_obs(plan, idx, nullptr, m); }

int spde_set_obs_weighted(SpdePlan* plan, const int64_t* idx, const double* weights, int m) {
  if (!weights && m > 0) return SPDE_ERR_ARG;
  return set_obs(plan, idx, weights, m);
}

int spde_factor(SpdePlan* plan, int with_obs, double tau, double* logdet) {
  if (plan && plan->p.precision == SPDE_PRECISION_ITERATIVE) return no_factor(plan);
  if (!plan) return SPDE_ERR_ARG;
  int rc = plan_factor(&plan->p, with_obs, tau);
  if (rc == 0 && logdet) *logdet = plan->p.logdet;
  return rc;
}

int spde_solve(SpdePlan* plan, const double* b, double* x, int nrhs, int iters, double tol, double* resid) {
  if (plan && plan->p.precision == SPDE_PRECISION_ITERATIVE) return no_factor(plan);
  if (!plan || !b || !x) return SPDE_ERR_ARG;
  return plan_solve(&plan->p, b, x, nrhs, iters, tol, resid);
}

int spde_sample(SpdePlan* plan, const double* z, double* x, int nrhs) {
  if (plan && plan->p.precision == SPDE_PRECISION_ITERATIVE) return no_factor(plan);
  if (!plan || !z || !x || nrhs < 1) return SPDE_ERR_ARG;
  return plan_sample(&plan->p, z, x, nrhs);
}

int spde_selinv(SpdePlan* plan, double* zq) {
  if (plan && plan->p.precision == SPDE_PRECISION_ITERATIVE) return no_factor(plan);
  if (!plan || !zq) return SPDE_ERR_ARG;
  return plan_selinv(&plan->p, zq);
}

int spde_adjoint(SpdePlan* plan, const double* gbar, double* grad_host) {
  if (!plan || !gbar || !grad_host) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  const int nt = ntheta_of(p) - 1;
  DevBuf work, g;  // freed on every return
  API_CUDA(work.ensure(size_t(adjoint_work_elems(&p))));
  API_CUDA(g.ensure(size_t(nt)));
  launch_adjoint(&p, gbar, g.p, work.p, p.stream);
  cudaError_t e = cudaMemcpyAsync(grad_host, g.p, nt * sizeof(double), cudaMemcpyDeviceToHost, p.stream);
  cudaStreamSynchronize(p.stream);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) { p.last_error = "adjoint failed"; return SPDE_ERR_CUDA; }
  return SPDE_OK;
}

int spde_adjoint_noalloc(SpdePlan* plan, const double* gbar, double* grad_dev) {
  if (!plan || !gbar || !grad_dev) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  double* scratch = nullptr;
  int64_t cap = 0;
  // the plan's own device's copy of the array, whichever device is current
  if (noalloc_scratch(p.device, &scratch, &cap)) {
    p.last_error = "fixed scratch not reachable on the plan's device";
    return SPDE_ERR_CUDA;
  }
  const int64_t need = adjoint_work_elems(&p);
  if (need > cap) {
    p.last_error = "grid too large for the fixed adjoint scratch (needs " + std::to_string(need) +
                   " doubles, limit " + std::to_string(cap) + ", i.e. Mx*Ny <= " +
                   std::to_string(cap / kAdjointCellElems) + ")";
    return SPDE_ERR_ARG;
  }
  // enqueue on the plan's device (its array, its stream), then restore the caller's
  struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
      if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
      else prev = -1;
    }
    ~DeviceGuard() {
      if (prev >= 0) cudaSetDevice(prev);
    }
  } guard(p.device);
  // the kernels write every scratch entry they later read; clear anyway so no
  // value from an earlier call can leak into this one
  API_CUDA(cudaMemsetAsync(scratch, 0, size_t(need) * sizeof(double), p.stream));
  launch_adjoint(&p, gbar, grad_dev, scratch, p.stream);
  API_CUDA(cudaGetLastError());
  return SPDE_OK;
}

int spde_conditional_mean(SpdePlan* plan, double tau, const double* y, const double* mu0, double* mu) {
  if (plan && plan->p.precision == SPDE_PRECISION_ITERATIVE) return no_factor(plan);
  if (!plan || !y || !mu) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.d_obs_idx) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  int rc = plan_factor(&p, 1, tau);
  if (rc) return rc;
  DevBuf buf;  // right-hand side; freed on every return
  API_CUDA(buf.ensure(size_t(p.sym.n)));
  double* b = buf.p;
  API_CUDA(cudaMemsetAsync(b, 0, size_t(p.sym.n) * sizeof(double), p.stream));
  obs_rhs_kernel<<<(p.nobs + 255) / 256 + 1, 256, 0, p.stream>>>(p.d_obs_idx, p.nobs, 1, tau, y, mu0, b);
  double resid = 0.0;
  rc = plan_solve(&p, b, mu, 1, p.precision == 0 ? 1 : 10, kRefineTol, &resid);
  if (rc == 0 && mu0) {
    // mu += mu0, written as mu - (0 - mu0) with the subtraction kernel
    API_CUDA(cudaMemsetAsync(b, 0, size_t(p.sym.n) * sizeof(double), p.stream));
    sub_kernel<<<int((p.sym.n + 255) / 256), 256, 0, p.stream>>>(b, mu0, p.sym.n);
    sub_kernel<<<int((p.sym.n + 255) / 256), 256, 0, p.stream>>>(mu, b, p.sym.n);
  }
  cudaStreamSynchronize(p.stream);  // before buf is freed
  return rc;
}

int spde_loglike(SpdePlan* plan, const double* theta, int ntheta, const double* y, int r, int grad_mode,
                 const double* V, int nh1, double* f_out, double* jac) {
  if (plan && plan->p.precision == SPDE_PRECISION_ITERATIVE) return no_factor(plan);
  if (!plan || !theta || !y || r < 1 || !f_out || grad_mode < 0 || grad_mode > 2) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.d_obs_idx || p.nobs < 1) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  if (grad_mode == 2 && (!V || nh1 < 1)) { p.last_error = "Hutchinson mode needs probes"; return SPDE_ERR_ARG; }
  if (grad_mode && !jac) return SPDE_ERR_ARG;
  int rc = spde_assemble(plan, theta, ntheta);
  if (rc) return rc;
  cudaStream_t st = p.stream;
  const int n = p.sym.n, ns = p.sym.nslots, m = p.nobs;
  const double tau = std::exp(theta[ntheta - 1]);
  LoglikeScratch& S = plan->s;
  const int nblk = 256;
  API_CUDA(S.part.ensure(nblk));
  const bool exact = grad_mode == 1, hutch = grad_mode == 2;
  if (exact) { API_CUDA(S.zq.ensure(size_t(n) * ns)); API_CUDA(S.zqc.ensure(size_t(n) * ns)); }
  if (hutch) { API_CUDA(S.trq.ensure(size_t(n) * nh1)); API_CUDA(S.trc.ensure(size_t(n) * nh1)); }
  const int iters = p.precision == 0 ? 1 : 10;
  const double tol = kRefineTol;
  API_CUDA(S.b.ensure(size_t(n) * r));
  API_CUDA(S.mu.ensure(size_t(n) * r));
  API_CUDA(S.qmu.ensure(size_t(n) * r));
  API_CUDA(S.d.ensure(size_t(m) * r));
  // Q_c = Q + tau S^T S on the second pipeline when there is one (its own
  // arenas, stream and host thread), else after Q on this plan
  Plan* qc = &p;
  if (plan->pipelines > 1) {
    if ((rc = ensure_twin(plan))) return rc;
    qc = plan->twin.get();
    share_model(p, *qc);
    cudaEvent_t ready;
    API_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    API_CUDA(cudaEventRecord(ready, st));  // assembly done
    API_CUDA(cudaStreamWaitEvent(qc->stream, ready, 0));
    cudaEventDestroy(ready);
  }
  double ldq = 0.0, ldqc = 0.0, res = 0.0, res_c = 0.0;
  int rc_c = 0;
  PhaseLog plog(st);
  // with two pipelines, each runs its phases on the plan's phase streams and
  // returns to its own stream at the end
  bool phased = qc != &p;
  if (phased && (rc = ensure_phase_streams(plan))) return rc;
  cudaStream_t qc_home = qc->stream;
  auto run_qc = [&]() {
    if (phased) move_to(qc, plan->phase[1][0], plan->phase_ev[1][0]);
    if ((rc_c = plan_factor(qc, 1, tau))) return;
    plog.mark("qc_factor", qc->stream);
    ldqc = qc->logdet;
    cudaMemsetAsync(S.b.p, 0, size_t(n) * r * sizeof(double), qc->stream);
    obs_rhs_kernel<<<int((int64_t(m) * r + 255) / 256), 256, 0, qc->stream>>>(p.d_obs_idx, m, r, tau, y, nullptr,
                                                                               S.b.p);
    if ((rc_c = plan_solve(qc, S.b.p, S.mu.p, r, iters, tol, &res_c))) return;
    plog.mark("qc_solve", qc->stream);
    if (hutch && (rc_c = plan_solve(qc, V, S.trc.p, nh1, iters, tol, &res_c))) return;
    if (phased) move_to(qc, plan->phase[1][1], plan->phase_ev[1][1]);
    if (exact && (rc_c = plan_selinv(qc, S.zqc.p))) return;
    plog.mark("qc_inverse", qc->stream);
  };
  std::thread worker;
  if (qc != &p) {
    try {
      worker = std::thread(run_qc);
    } catch (...) {
      qc = &p;  // no thread available: both on this plan, one after the other
      phased = false;
    }
  }
  // Q: log-determinant, then its inverse on the pattern (or Hutchinson solves)
  if (phased) move_to(&p, plan->phase[0][0], plan->phase_ev[0][0]);
  rc = plan_factor(&p, 0, 0.0);
  plog.mark("q_factor", p.stream);
  if (!rc) ldq = p.logdet;
  if (phased) move_to(&p, plan->phase[0][1], plan->phase_ev[0][1]);
  if (!rc && exact) rc = plan_selinv(&p, S.zq.p);
  plog.mark("q_inverse", p.stream);
  if (!rc && hutch) rc = plan_solve(&p, V, S.trq.p, nh1, iters, tol, &res);
  if (qc != &p) worker.join();
  else if (!rc) run_qc();
  if (phased) {
    // back to the caller's stream, after both pipelines' work
    move_to(qc, qc_home, plan->phase_ev[1][2]);
    cudaStreamWaitEvent(st, plan->phase_ev[1][2], 0);
    move_to(&p, st, plan->phase_ev[0][2]);
  }
  if (rc) return rc;
  if (rc_c) {
    if (qc != &p) p.last_error = qc->last_error;
    return rc_c;
  }
  // quadratic terms
  launch_spmv(p.qstencil(), nullptr, 0.0, S.mu.p, S.qmu.p, r, st);
  dot_partial_kernel<<<nblk, 256, 0, st>>>(S.mu.p, S.qmu.p, int64_t(n) * r, S.part.p);
  const double muqmu = host_sum_partials(S.part.p, nblk, st);
  obs_resid_kernel<<<int((int64_t(m) * r + 255) / 256), 256, 0, st>>>(p.d_obs_idx, m, r, y, S.mu.p, S.d.p);
  dot_partial_kernel<<<nblk, 256, 0, st>>>(S.d.p, nullptr, int64_t(m) * r, S.part.p);
  const double rss = host_sum_partials(S.part.p, nblk, st);
  p.launches_total += 5;  // obs rhs, spmv, two dot partials, obs residual
  const double like = 0.5 * ldq * r + m * r * std::log(tau) / 2 - 0.5 * ldqc * r - 0.5 * muqmu - tau / 2 * rss;
  *f_out = -like / (double(m) * r);
  if (!grad_mode) return SPDE_OK;
  API_CUDA(S.gbar.ensure(size_t(n) * ns));
  if (hutch) {
    int64_t tot = int64_t(n) * nh1;
    sub_kernel<<<int((tot + 255) / 256), 256, 0, st>>>(S.trq.p, S.trc.p, tot);  // trq <- TrQ - TrQc
  }
  {
    int64_t tot = int64_t(n) * ns;
    gbar_kernel<<<int((tot + 255) / 256), 256, 0, st>>>(p.sym.Mx, p.sym.Ny, p.sym.T, ns, 0.5 * r, exact ? S.zq.p : nullptr,
                                                        S.zqc.p, S.trq.p, V, nh1, S.mu.p, r, S.gbar.p);
  }
  API_CUDA(S.work.ensure(size_t(adjoint_work_elems(&p))));
  API_CUDA(S.gradv.ensure(size_t(ntheta)));
  launch_adjoint(&p, S.gbar.p, S.gradv.p, S.work.p, st);
  std::vector<double> g(ntheta, 0.0);
  API_CUDA(cudaMemcpyAsync(g.data(), S.gradv.p, (ntheta - 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
  const int centre = p.sym.nslots / 2;  // the (0, 0, 0) slot of every layout
  obs_trace_kernel<<<nblk, 256, 0, st>>>(p.d_obs_idx, m, exact ? S.zqc.p : nullptr, ns, centre, S.trc.p, V, nh1,
                                         S.part.p);
  const double tr = host_sum_partials(S.part.p, nblk, st);
  plog.mark("gradient", st);
  p.launches_total += 5 + (hutch ? 1 : 0);  // gbar, adjoint (3), obs trace, probe difference
  API_CUDA(cudaGetLastError());
  const double trace_term = exact ? tr : tr / nh1;
  g[ntheta - 1] = m * r / 2.0 - 0.5 * r * tau * trace_term - tau / 2 * rss;
  for (int i = 0; i < ntheta; ++i) jac[i] = -g[i] / (double(m) * r);
  return SPDE_OK;
}

int spde_plan_set_wait_limit(SpdePlan* plan, int64_t ns) {
  if (!plan || ns < 0) return SPDE_ERR_ARG;
  const unsigned long long v = ns == 0 ? kTcWaitNs : static_cast<unsigned long long>(ns);
  plan->p.tc_wait_ns = v;
  if (plan->twin) plan->twin->tc_wait_ns = v;
  return SPDE_OK;
}

int spde_plan_set_pipelines(SpdePlan* plan, int pipelines) {
  if (!plan || pipelines < 1 || pipelines > 2) return SPDE_ERR_ARG;
  plan->pipelines = pipelines;
  if (pipelines == 1) destroy_twin(plan);
  return SPDE_OK;
}

// ------------------------------------------------------------ learned PCG
int spde_precond_nparams(void) { return kPcParams; }

int spde_precond_weights(SpdePlan* plan, int with_obs, double tau, const float* params, float* w, float* act) {
  if (!plan || !params || !w) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (int rc = not_separable(p, "the learned preconditioner")) return rc;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (with_obs && !p.d_obs_cnt) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  return pc_weights(&p, with_obs, tau, params, w, act) ? SPDE_ERR_CUDA : SPDE_OK;
}

int spde_precond_compact_size(const SpdePlan* plan, int64_t* nfloats) {
  if (!plan || !nfloats) return SPDE_ERR_ARG;
  *nfloats = pc_compact_floats(&plan->p);
  return SPDE_OK;
}

int spde_precond_weights_compact(SpdePlan* plan, int with_obs, double tau, const float* params, float* w) {
  if (!plan || !params || !w) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (int rc = not_separable(p, "the learned preconditioner")) return rc;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (with_obs && !p.d_obs_cnt) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  return pc_weights_compact(&p, with_obs, tau, params, w) ? SPDE_ERR_CUDA : SPDE_OK;
}

int spde_precond_grad(SpdePlan* plan, int with_obs, double tau, const float* params, const float* w,
                      const float* act, const double* z, int k, double* loss, float* grad) {
  if (!plan || !params || !w || !act || !z || k < 1 || !loss || !grad) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (int rc = not_separable(p, "the learned preconditioner")) return rc;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (with_obs && !p.d_obs_cnt) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  const int rc = pc_grad(&p, with_obs, tau, params, w, act, z, k, loss, grad);
  if (rc == 4) { p.last_error = "scratch allocation failed"; return SPDE_ERR_NO_MEMORY; }
  if (rc == 1) { p.last_error = "n x nrhs must stay below 2^31"; return SPDE_ERR_ARG; }
  return rc ? SPDE_ERR_CUDA : SPDE_OK;
}

int spde_adam_step(SpdePlan* plan, float* params, const float* grad, float* m, float* v, int n, double lr, double b1,
                   double b2, double eps, int t) {
  if (!plan || !params || !grad || !m || !v || n < 1 || t < 1) return SPDE_ERR_ARG;
  return pc_adam(grad, params, m, v, n, float(lr), float(b1), float(b2), float(eps), t, plan->p.stream)
             ? SPDE_ERR_CUDA
             : SPDE_OK;
}

int spde_qsqrt(SpdePlan* plan, int transpose, const double* x, double* y, int nrhs) {
  if (!plan || !x || !y || nrhs < 1) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (int rc = not_separable(p, "the square root of Q")) return rc;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  const int rc = qsqrt_apply(&p, transpose, x, y, nrhs);
  if (rc == 1) { p.last_error = "n x nrhs must stay below 2^31"; return SPDE_ERR_ARG; }
  return rc ? SPDE_ERR_CUDA : SPDE_OK;
}

int spde_jacobi_smooth(SpdePlan* plan, int with_obs, double tau, double omega, int sweeps, double* z, int nrhs) {
  if (!plan || !z || nrhs < 1 || sweeps < 0) return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (with_obs && !p.d_obs_cnt) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  const int rc = jacobi_smooth(&p, with_obs, tau, omega, sweeps, z, nrhs);
  if (rc == 4) { p.last_error = "scratch allocation failed"; return SPDE_ERR_NO_MEMORY; }
  if (rc == 1) { p.last_error = "n x nrhs must stay below 2^31"; return SPDE_ERR_ARG; }
  return rc ? SPDE_ERR_CUDA : SPDE_OK;
}

int spde_loglike_grad_pcg(SpdePlan* plan, double tau, const double* y, int r, const double* V, int nh1, int precond,
                          const float* w_q, const float* w_qc, double tol, int maxit, double* jac, int* iters) {
  if (!plan || !y || r < 1 || !V || nh1 < 1 || !jac || maxit < 1 || precond < 0 || precond > 3 ||
      (precond >= 2 && (!w_q || !w_qc)))
    return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (precond >= 2)
    if (int rc = not_separable(p, "the learned preconditioner")) return rc;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (!p.d_obs_idx || p.nobs < 1) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  cudaStream_t st = p.stream;
  const int n = p.sym.n, ns = p.sym.nslots, m = p.nobs, ntheta = ntheta_of(p);
  LoglikeScratch& S = plan->s;
  const int nblk = 256;
  API_CUDA(S.part.ensure(nblk));
  API_CUDA(S.trq.ensure(size_t(n) * nh1));
  API_CUDA(S.trc.ensure(size_t(n) * nh1));
  API_CUDA(S.b.ensure(size_t(n) * r));
  API_CUDA(S.mu.ensure(size_t(n) * r));
  API_CUDA(S.d.ensure(size_t(m) * r));
  API_CUDA(S.gbar.ensure(size_t(n) * ns));
  int it_total = 0, it = 0;
  double rel = 0.0;
  auto solve = [&](int with_obs, const float* w, const double* b, double* x, int nrhs) -> int {
    const int rc = pcg_solve(&p, with_obs, tau, precond, w, b, x, nrhs, tol, maxit, 8, &it, &rel);
    it_total += it;
    if (rc == 7) {
      p.last_error = "compact preconditioner weights do not match this solve (with or without observations, or another observation set)";
      return SPDE_ERR_STATE;
    }
    if (rc == 4) { p.last_error = "scratch allocation failed"; return SPDE_ERR_NO_MEMORY; }
    if (rc == 1) { p.last_error = "n x nrhs must stay below 2^31"; return SPDE_ERR_ARG; }
    if (rc == 6) { p.last_error = "PCG did not reach the tolerance"; return SPDE_ERR_NOT_CONVERGED; }
    return rc ? SPDE_ERR_CUDA : SPDE_OK;
  };
  // conditional mean mu = (Q + tau S^T S)^-1 tau S^T y
  API_CUDA(cudaMemsetAsync(S.b.p, 0, size_t(n) * r * sizeof(double), st));
  obs_rhs_kernel<<<int((int64_t(m) * r + 255) / 256), 256, 0, st>>>(p.d_obs_idx, m, r, tau, y, nullptr, S.b.p);
  int rc = solve(1, w_qc, S.b.p, S.mu.p, r);
  if (rc) return rc;
  // Hutchinson solves Q^-1 V and (Q + tau S^T S)^-1 V
  if ((rc = solve(0, w_q, V, S.trq.p, nh1))) return rc;
  if ((rc = solve(1, w_qc, V, S.trc.p, nh1))) return rc;
  obs_resid_kernel<<<int((int64_t(m) * r + 255) / 256), 256, 0, st>>>(p.d_obs_idx, m, r, y, S.mu.p, S.d.p);
  dot_partial_kernel<<<nblk, 256, 0, st>>>(S.d.p, nullptr, int64_t(m) * r, S.part.p);
  const double rss = host_sum_partials(S.part.p, nblk, st);
  {
    const int64_t tot = int64_t(n) * nh1;
    sub_kernel<<<int((tot + 255) / 256), 256, 0, st>>>(S.trq.p, S.trc.p, tot);
  }
  {
    const int64_t tot = int64_t(n) * ns;
    gbar_kernel<<<int((tot + 255) / 256), 256, 0, st>>>(p.sym.Mx, p.sym.Ny, p.sym.T, ns, 0.5 * r, nullptr, nullptr,
                                                        S.trq.p, V, nh1, S.mu.p, r, S.gbar.p);
  }
  API_CUDA(S.work.ensure(size_t(adjoint_work_elems(&p))));
  API_CUDA(S.gradv.ensure(size_t(ntheta)));
  launch_adjoint(&p, S.gbar.p, S.gradv.p, S.work.p, st);
  std::vector<double> g(ntheta, 0.0);
  API_CUDA(cudaMemcpyAsync(g.data(), S.gradv.p, (ntheta - 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
  const int centre = p.sym.nslots / 2;  // the (0, 0, 0) slot of every layout
  obs_trace_kernel<<<nblk, 256, 0, st>>>(p.d_obs_idx, m, nullptr, ns, centre, S.trc.p, V, nh1, S.part.p);
  const double tr = host_sum_partials(S.part.p, nblk, st);
  API_CUDA(cudaGetLastError());
  g[ntheta - 1] = m * r / 2.0 - 0.5 * r * tau * tr / nh1 - tau / 2 * rss;
  for (int i = 0; i < ntheta; ++i) jac[i] = -g[i] / (double(m) * r);
  if (iters) *iters = it_total;
  return SPDE_OK;
}

int spde_pcg(SpdePlan* plan, int with_obs, double tau, int precond, const float* w, const double* b, double* x,
             int nrhs, double tol, int maxit, int* iters, double* relres) {
  if (!plan || !b || !x || nrhs < 1 || maxit < 1 || !iters || !relres || precond < 0 || precond > 4 ||
      ((precond == 2 || precond == 3) && !w))
    return SPDE_ERR_ARG;
  Plan& p = plan->p;
  if (precond >= 2)
    if (int rc = not_separable(p, "the learned preconditioner")) return rc;
  if (!p.assembled) { p.last_error = "no assembled model"; return SPDE_ERR_STATE; }
  if (with_obs && !p.d_obs_cnt) { p.last_error = "no observations set"; return SPDE_ERR_STATE; }
  const int rc = pcg_solve(&p, with_obs, tau, precond, w, b, x, nrhs, tol, maxit, 8, iters, relres);
  if (rc == 7) {
    p.last_error = "compact preconditioner weights do not match this solve (with or without observations, or another observation set)";
    return SPDE_ERR_STATE;
  }
  if (rc == 8) {
    p.last_error = "IC(0) needs a spatio-temporal (not separable) plan with Mx >= 5, Ny >= 4, T >= 2";
    return SPDE_ERR_STATE;
  }
  if (rc == 9) { p.last_error = "incomplete Cholesky broke down for every diagonal shift"; return SPDE_ERR_NOT_SPD; }
  if (rc == 4) { p.last_error = "scratch allocation failed"; return SPDE_ERR_NO_MEMORY; }
  if (rc == 1) { p.last_error = "n x nrhs must stay below 2^31"; return SPDE_ERR_ARG; }
  if (rc == 6) { p.last_error = "PCG did not reach the tolerance"; return SPDE_ERR_NOT_CONVERGED; }
  return rc ? SPDE_ERR_CUDA : SPDE_OK;
}

}  // extern "C"


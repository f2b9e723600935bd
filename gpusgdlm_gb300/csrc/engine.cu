// The SGDLM engine behind the C ABI of include/sgdlm.h.
//
// Plays the role of the reference's SGDLM::HostWrapperImpl<double>
// (rSGDLM/src/SGDLM/HostWrapperImpl.cu): owns the device state, the simulation
// buffers and the stream, enforces the prior/posterior state machine, and
// sequences the kernels of each filtering call.  Differences by design:
//   * one GPU (no per-device loops, no host-side combine of per-GPU moments);
//   * flat, strided buffers instead of device pointer arrays;
//   * draw buffers are series-major and no random-number caches exist (Philox
//     in registers), so simulation memory is lambda + theta + one LU slab per
//     resident CTA instead of 2*nsim_batch dense m x m matrices;
//   * nsim_batch is accepted and reported for API compatibility; it does not
//     change results (neither does it in the reference) nor memory here.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <set>
#include <string>
#include <type_traits>
#include <vector>

#include <cmath>

#include <cuda_bf16.h>

#include "../../include/sgdlm.h"
#include "elimination.hpp"
#include "kernels.hpp"
#include "proposal.hpp"

using namespace sgdlm;

namespace {

// Levels and default of the reference's logger (rSGDLM/src/logger.hpp:16-30,
// logger.cpp:11).
enum LogLevel { LOG_ERROR = 0, LOG_WARNING = 5, LOG_INFO = 10, LOG_RESULT = 20, LOG_DEBUG = 50, LOG_SYSDEBUG = 100 };

template <typename T> struct DevBuf {
  T *ptr = nullptr;
  size_t count = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  cudaError_t alloc(size_t n) {
    release();
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&ptr, n * sizeof(T));
    if (e != cudaSuccess) {
      ptr = nullptr;
      return e;
    }
    count = n;
    return cudaMemset(ptr, 0, n * sizeof(T));
  }
  // at least n elements: the present allocation when it is large enough (its
  // contents kept), else a new one
  cudaError_t reserve(size_t n) { return (ptr && count >= n) ? cudaSuccess : alloc(n); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
};

constexpr size_t kMaxP = 64;

// The learned importance proposal's configuration, network, replay buffer and
// per-call buffers (proposal.hpp).
struct ProposalState {
  sgdlm_proposal_config cfg{SGDLM_PROPOSAL_PLAIN, 500, 4, 4096, 1e-3, 0.5, 20261204u};
  size_t m = 0, P = 0;  // dimensions the buffers were made for
  MlpLayout L{};
  long cap = 0, count = 0, pos = 0;
  sgdlm_proposal_info info{};
  DevBuf<float> w, grad, m1, m2;
  DevBuf<__nv_bfloat16> w16;
  DevBuf<float> X, Y, M;                 // m rows: features (normalised in X), targets, mask
  DevBuf<float> bX, bY, bM;              // replay ring, cap rows
  DevBuf<float> Xb, Yb, Mb;              // training batch
  DevBuf<float> Z1, A1, Z2, A2, Out, dOut, dA, dA2;  // activations, max(batch, m) rows
  DevBuf<double> fsum, loss;
  DevBuf<double> mq, nq, sq, Uq64, cst, lr, logw;
  DevBuf<float> Uq32;
  MlpActs acts() {
    return MlpActs{Z1.ptr, A1.ptr, Z2.ptr, A2.ptr, Out.ptr, dOut.ptr, dA.ptr, dA2.ptr};
  }
  void release() {
    for (auto *b : {&w, &grad, &m1, &m2, &X, &Y, &M, &bX, &bY, &bM, &Xb, &Yb, &Mb, &Z1, &A1, &Z2,
                    &A2, &Out, &dOut, &dA, &dA2, &Uq32})
      b->release();
    for (auto *b : {&fsum, &loss, &mq, &nq, &sq, &Uq64, &cst, &lr, &logw}) b->release();
    w16.release();
    m = P = 0;
    cap = count = pos = 0;
    info = sgdlm_proposal_info{};
  }
};

}  // namespace

struct sgdlm_engine {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  size_t no_gpus = 1;
  size_t m = 0, P = 0;
  bool mem_init = false, sim_init = false, is_prior = false;
  bool use_evo = false;  // state evolution matrices enabled (manageEvoMemory)
  size_t nsim = 0, nsim_batch = 0;
  int precision = SGDLM_PRECISION_MIXED;
  unsigned compat = SGDLM_COMPAT_REFERENCE;
  uint64_t seed = 1234;  // HostWrapperImpl.cu:63-64 seeds device 0 with 1234
  uint64_t epoch = 0;
  int log_level = LOG_RESULT;
  std::string last_error;
  uint64_t launches = 0;
  sgdlm_stats stats{};

  // state
  DevBuf<double> m_t, C_t, n_t, s_t, W_t, beta, delta;
  DevBuf<unsigned> p, sp;
  DevBuf<int> g_rowptr;
  DevBuf<int2> g_ent;
  DevBuf<int> g_jac_order;  // the rows by decreasing length (iterative forecast solves)
  DevBuf<int> g_extptr, g_extk;
  // evolution matrices G (P x P x m, FP64 and the FP32 copy the draws use)
  DevBuf<double> G_t;
  DevBuf<float> G32;
  DevBuf<float> x32;  // FP32 copy of a forecast's x (the right-hand sides of FP32 draws)
  // sparse pre-elimination plan of (I - Gamma) (elimination.hpp)
  int elim_levels = 4;
  EliminationPlanHost eplan;
  DevBuf<int> elim_buf;
  EliminationPlan elim_dev{};
  DevBuf<double> y_t, F_t, x_t;
  DevBuf<double> fm_t, fC_t, fn_t, fs_t, fW_t;
  DevBuf<double> U64;
  DevBuf<float> U32;
  std::vector<unsigned> h_p, h_sp;
  // simulation
  DevBuf<unsigned char> lambda, theta, lu_scratch;
  // the draws' Gamma entries draw-major (GammaDraws), room for m * P per draw
  DevBuf<unsigned char> theta_g;
  int g_nnz = 0;  // Gamma entries (rows' CSR length)
  DevBuf<double> logdet, w, y_fc, nu_fc, stats6, wpart, part_a, part_b;
  DevBuf<int> draw_flags, series_flags;
  DevBuf<int> pivot_list;  // nsim + 1: count, then the draws flagged for the redo
  DevBuf<double> mean_m, mean_C, mean_n, mean_s, mean_lambda, mean_log_lambda, mean_Q;
  DevBuf<uint32_t> dev_epoch;
  LuPlan plan{};
  LuOptions lu_opt{};
  JacobiPlan jac{};        // iterative forecast solves of FP32 draws
  int forecast_iterative = 1;
  DevBuf<int> jac_list;    // nsim + 1: count, then the forecast draws left to factor
  ProposalState prop;
  int chunks = 0;          // VB draw chunks and draws per chunk (vb_chunking)
  long chunk_draws = 0;
  cudaEvent_t ev[8] = {};

  void log(int level, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (level == LOG_ERROR) last_error = buf;
    if (level <= log_level)
      fprintf(stderr, "%s%s\n",
              level == LOG_ERROR ? "Error: " : (level == LOG_WARNING ? "Warning: " : ""), buf);
  }
  int fail(int status, const char *msg) {
    log(LOG_ERROR, "%s", msg);
    return status;
  }
  int cuda_fail(cudaError_t e, const char *where) {
    char buf[256];
    snprintf(buf, sizeof buf, "CUDA error in %s: %s", where, cudaGetErrorString(e));
    log(LOG_ERROR, "%s", buf);
    return e == cudaErrorMemoryAllocation ? SGDLM_ERR_OUT_OF_MEMORY : SGDLM_ERR_DEVICE;
  }
  // HostWrapperImpl.cu:1240-1246
  bool check_initialized() {
    if (!mem_init) {
      log(LOG_ERROR, "The device memory is not initialized.");
      return false;
    }
    return true;
  }
  // HostWrapperImpl.cu:1249-1255
  bool check_sim_initialized() {
    if (!sim_init) {
      log(LOG_ERROR, "The simulation device memory is not initialized.");
      return false;
    }
    return true;
  }
  // HostWrapperImpl.cu:1258-1265
  bool check_use_evo() {
    if (!use_evo) {
      log(LOG_ERROR, "The use of state evolution matrices is disabled.");
      return false;
    }
    return true;
  }
  // HostWrapperImpl.cu:1268-1286
  bool check_prior(bool want_prior) {
    if (want_prior && !is_prior) {
      log(LOG_ERROR, "This function can only be executed when the parameters are prior parameters.");
      return false;
    }
    if (!want_prior && is_prior) {
      log(LOG_ERROR, "This function can only be executed when the parameters are posterior parameters.");
      return false;
    }
    return true;
  }
  size_t tsize() const { return precision == SGDLM_PRECISION_FP64 ? sizeof(double) : sizeof(float); }
  RngKey key(uint32_t ep) const {
    return RngKey{(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32), ep, nullptr};
  }
};

namespace {

#define CK(expr)                                                     \
  do {                                                               \
    cudaError_t _e = (expr);                                         \
    if (_e != cudaSuccess) return h->cuda_fail(_e, #expr);           \
  } while (0)

int h2d(sgdlm_engine *h, void *dst, const void *src, size_t bytes) {
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
  return SGDLM_OK;
}
int d2h(sgdlm_engine *h, void *dst, const void *src, size_t bytes) {
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
  return SGDLM_OK;
}
int sync(sgdlm_engine *h) {
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaGetLastError());
  return SGDLM_OK;
}
float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// Row-wise CSR of the Gamma entries (see GammaRows), from the host copy of sp.
int upload_gamma_rows(sgdlm_engine *h) {
  const size_t m = h->m, P = h->P, mm = m * m;
  std::vector<int> rowptr(m + 1, 0);
  std::vector<int2> ent;
  for (size_t e = 0; e < m * P; ++e)
    if ((size_t)h->h_sp[e] < mm) rowptr[h->h_sp[e] % m + 1]++;
  for (size_t r = 0; r < m; ++r) rowptr[r + 1] += rowptr[r];
  ent.resize(rowptr[m] > 0 ? rowptr[m] : 1);
  std::vector<int> fill(rowptr.begin(), rowptr.end() - 1);
  for (size_t e = 0; e < m * P; ++e) {
    const unsigned pos = h->h_sp[e];
    if ((size_t)pos < mm) ent[fill[pos % m]++] = make_int2((int)e, (int)(pos / m));
  }
  CK(h->g_rowptr.alloc(m + 1));
  CK(h->g_ent.alloc(ent.size()));
  CK(cudaMemcpy(h->g_rowptr.ptr, rowptr.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->g_ent.ptr, ent.data(), ent.size() * sizeof(int2), cudaMemcpyHostToDevice));
  std::vector<int> extptr(m + 1, 0), extk;
  for (size_t j = 0; j < m; ++j) {
    for (size_t k = 0; k < P; ++k)
      if ((size_t)h->h_sp[j * P + k] >= mm) extk.push_back((int)k);
    extptr[j + 1] = (int)extk.size();
  }
  if (extk.empty()) extk.push_back(0);
  CK(h->g_extptr.alloc(m + 1));
  CK(h->g_extk.alloc(extk.size()));
  CK(cudaMemcpy(h->g_extptr.ptr, extptr.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->g_extk.ptr, extk.data(), extk.size() * sizeof(int), cudaMemcpyHostToDevice));
  h->g_nnz = rowptr[m];
  int max_row = 0;
  for (size_t r = 0; r < m; ++r) max_row = std::max(max_row, rowptr[r + 1] - rowptr[r]);
  std::vector<int> order(m);
  for (size_t r = 0; r < m; ++r) order[r] = (int)r;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return rowptr[a + 1] - rowptr[a] > rowptr[b + 1] - rowptr[b];
  });
  CK(h->g_jac_order.alloc(m));
  CK(cudaMemcpy(h->g_jac_order.ptr, order.data(), m * sizeof(int), cudaMemcpyHostToDevice));
  h->jac = plan_jacobi((int)m, max_row, h->num_sms);
  h->jac.order = h->g_jac_order.ptr;
  return SGDLM_OK;
}

// Plans the sparse pre-elimination for the current parental sets and uploads it
// as one int array.
int upload_elimination(sgdlm_engine *h) {
  const int m = (int)h->m, P = (int)h->P;
  h->eplan = plan_elimination(m, P, h->h_sp, h->elim_levels);
  const EliminationPlanHost &pl = h->eplan;
  std::vector<int> buf;
  std::vector<size_t> offs;
  auto put = [&](const void *data, size_t n_ints) {
    while (buf.size() % 4) buf.push_back(0);
    offs.push_back(buf.size());
    const int *p = static_cast<const int *>(data);
    buf.insert(buf.end(), p, p + n_ints);
  };
  put(pl.diag_slot.data(), pl.diag_slot.size());
  put(pl.l0_e.data(), pl.l0_e.size());
  put(pl.l0_slot.data(), pl.l0_slot.size());
  put(pl.lev_piv.data(), pl.lev_piv.size());
  put(pl.piv.data(), pl.piv.size());
  put(pl.lev_scale.data(), pl.lev_scale.size());
  put(pl.scale.data(), pl.scale.size());
  put(pl.lev_chunk.data(), pl.lev_chunk.size());
  put(pl.chunk_tofs.data(), pl.chunk_tofs.size());
  put(pl.ent.data(), pl.ent.size());
  put(pl.terms.data(), pl.terms.size());
  put(pl.lev_fwd_nodes.data(), pl.lev_fwd_nodes.size());
  put(pl.fwd_node.data(), pl.fwd_node.size());
  put(pl.fwd_ptr.data(), pl.fwd_ptr.size());
  put(pl.fwd.data(), pl.fwd.size());
  put(pl.lev_bwd_nodes.data(), pl.lev_bwd_nodes.size());
  put(pl.bwd_node.data(), pl.bwd_node.size());
  put(pl.bwd_diag.data(), pl.bwd_diag.size());
  put(pl.bwd_ptr.data(), pl.bwd_ptr.size());
  put(pl.bwd.data(), pl.bwd.size());
  put(pl.core_node.data(), pl.core_node.size());
  put(pl.core_map.data(), (pl.core_map.size() + 1) / 2);  // two 16-bit slots per int
  while (buf.size() % 4) buf.push_back(0);
  CK(h->elim_buf.alloc(buf.size()));
  CK(cudaMemcpy(h->elim_buf.ptr, buf.data(), buf.size() * sizeof(int), cudaMemcpyHostToDevice));
  const int *b = h->elim_buf.ptr;
  auto u = [&](size_t k) { return reinterpret_cast<const unsigned *>(b + offs[k]); };
  EliminationPlan &d = h->elim_dev;
  d = EliminationPlan{};
  d.m = m;
  d.P = P;
  d.nlev = pl.nlev;
  d.nv = pl.nlev > 0 ? pl.nv : 0;
  d.n_solve = pl.nlev > 0 ? pl.n_solve : 0;
  d.nnz0 = (int)pl.l0_e.size();
  d.core_n = pl.nlev > 0 ? pl.core_n : m;
  size_t k = 0;
  d.diag_slot = b + offs[k++];
  d.l0_e = b + offs[k++];
  d.l0_slot = b + offs[k++];
  d.lev_piv = b + offs[k++];
  d.piv = b + offs[k++];
  d.lev_scale = b + offs[k++];
  d.scale = u(k++);
  d.lev_chunk = b + offs[k++];
  d.chunk_tofs = b + offs[k++];
  d.ent = u(k++);
  d.terms = u(k++);
  d.prog = b + offs[k];
  d.prog_len = (int)(offs[k + 9] - offs[k]);  // lev_fwd_nodes .. bwd (core_node follows)
  d.lev_fwd_nodes = b + offs[k++];
  d.fwd_node = b + offs[k++];
  d.fwd_ptr = b + offs[k++];
  d.fwd = u(k++);
  d.lev_bwd_nodes = b + offs[k++];
  d.bwd_node = b + offs[k++];
  d.bwd_diag = b + offs[k++];
  d.bwd_ptr = b + offs[k++];
  d.bwd = u(k++);
  d.core_node = b + offs[k++];
  // without levels the whole matrix is the dense core, built from the parental sets
  d.core_map = pl.nlev > 0 ? reinterpret_cast<const uint16_t *>(b + offs[k]) : nullptr;
  return SGDLM_OK;
}

int alloc_state(sgdlm_engine *h) {
  const size_t m = h->m, P = h->P;
  CK(h->m_t.alloc(P * m));
  CK(h->C_t.alloc(P * P * m));
  CK(h->n_t.alloc(m));
  CK(h->s_t.alloc(m));
  CK(h->W_t.alloc(P * P * m));
  CK(h->beta.alloc(m));
  CK(h->delta.alloc(P * P * m));
  CK(h->p.alloc(m));
  CK(h->sp.alloc(P * m));
  CK(h->y_t.alloc(m));
  CK(h->F_t.alloc(P * m));
  CK(h->x_t.alloc(P * m));
  CK(h->fm_t.alloc(P * m));
  CK(h->fC_t.alloc(P * P * m));
  CK(h->fn_t.alloc(m));
  CK(h->fs_t.alloc(m));
  CK(h->fW_t.alloc(P * P * m));
  CK(h->U64.alloc(P * P * m));
  CK(h->U32.alloc(P * P * m));
  CK(h->mean_m.alloc(P * m));
  CK(h->mean_C.alloc(P * P * m));
  CK(h->mean_n.alloc(m));
  CK(h->mean_s.alloc(m));
  CK(h->mean_lambda.alloc(m));
  CK(h->mean_log_lambda.alloc(m));
  CK(h->mean_Q.alloc(m));
  CK(h->series_flags.alloc(m));
  CK(h->stats6.alloc(8));
  CK(h->wpart.alloc(4 * (size_t)kWeightBlocks));
  CK(h->x32.alloc(P * m));
  CK(h->dev_epoch.alloc(1));
  h->h_p.assign(m, 0);
  h->h_sp.assign(P * m, 0xFFFFFFFFu);
  // Parental sets default to "no simultaneous parents" (all external).
  CK(cudaMemcpy(h->sp.ptr, h->h_sp.data(), P * m * sizeof(unsigned), cudaMemcpyHostToDevice));
  int st = upload_gamma_rows(h);
  if (st) return st;
  return upload_elimination(h);
}

void release_sim(sgdlm_engine *h) {
  h->lambda.release();
  h->theta.release();
  h->theta_g.release();
  h->lu_scratch.release();
  h->logdet.release();
  h->w.release();
  h->y_fc.release();
  h->nu_fc.release();
  h->part_a.release();
  h->part_b.release();
  h->draw_flags.release();
  h->pivot_list.release();
  h->jac_list.release();
  h->sim_init = false;
  h->nsim = 0;
  h->nsim_batch = 0;
}

void release_all(sgdlm_engine *h) {
  release_sim(h);
  for (auto *b : {&h->m_t, &h->C_t, &h->n_t, &h->s_t, &h->W_t, &h->beta, &h->delta, &h->y_t,
                  &h->F_t, &h->x_t, &h->fm_t, &h->fC_t, &h->fn_t, &h->fs_t, &h->fW_t,
                  &h->U64, &h->mean_m, &h->mean_C, &h->mean_n, &h->mean_s, &h->mean_lambda,
                  &h->mean_log_lambda, &h->mean_Q, &h->stats6, &h->wpart})
    b->release();
  h->U32.release();
  h->p.release();
  h->sp.release();
  h->g_rowptr.release();
  h->g_ent.release();
  h->g_jac_order.release();
  h->g_extptr.release();
  h->g_extk.release();
  h->G_t.release();
  h->G32.release();
  h->x32.release();
  h->elim_buf.release();
  h->elim_dev = EliminationPlan{};
  h->series_flags.release();
  h->dev_epoch.release();
  h->mem_init = false;
}

int plan_sim(sgdlm_engine *h, long n, LuPlan *out) {
  const int core_n = h->elim_dev.core_n > 0 ? h->elim_dev.core_n : (int)h->m;
  const int nv = h->elim_dev.nv;
  LuPlan pl = (h->precision == SGDLM_PRECISION_FP64)
                  ? plan_lu<double>((int)h->m, (int)h->P, n, h->num_sms, core_n, nv,
                                    h->elim_dev.n_solve, h->elim_dev.prog_len, h->lu_opt)
                  : plan_lu<float>((int)h->m, (int)h->P, n, h->num_sms, core_n, nv,
                                   h->elim_dev.n_solve, h->elim_dev.prog_len, h->lu_opt);
  if (pl.smem > 227 * 1024 - 64 || pl.smem_fallback > 227 * 1024 - 64) {
    char buf[200];
    snprintf(buf, sizeof buf,
             "m = %zu needs %zu bytes of shared memory per LU block at this precision "
             "(limit 232448); use the mixed precision or a smaller m",
             h->m, std::max(pl.smem, pl.smem_fallback));
    return h->fail(SGDLM_ERR_UNSUPPORTED, buf);
  }
  *out = pl;
  return SGDLM_OK;
}

int alloc_sim(sgdlm_engine *h, size_t nsim) {
  const size_t m = h->m, P = h->P, ts = h->tsize();
  LuPlan pl;
  int st = plan_sim(h, (long)nsim, &pl);
  if (st) return st;
  // grow-only: a smaller draw count (e.g. forecasts of fewer draws between VB
  // calls with more) keeps the allocations, so that alternating counts do not
  // free and allocate gigabytes every call; every buffer is written before it
  // is read within a call
  h->plan = pl;
  vb_chunking((long)nsim, (int)m, h->num_sms, &h->chunks, &h->chunk_draws);
  CK(h->lambda.reserve(m * nsim * ts));
  CK(h->theta.reserve(m * nsim * P * ts));
  CK(h->theta_g.reserve(m * nsim * P * ts));
  CK(h->lu_scratch.reserve(pl.scratch_elems_total * ts));
  CK(h->logdet.reserve(nsim));
  CK(h->w.reserve(nsim));
  CK(h->y_fc.reserve(nsim * m));
  CK(h->nu_fc.reserve(nsim * m));
  CK(h->draw_flags.reserve(nsim));
  CK(h->pivot_list.reserve(nsim + 1));
  CK(h->jac_list.reserve(nsim + 1));
  CK(h->part_a.reserve((size_t)h->chunks * m * (P + 2) + m * P));
  CK(h->part_b.reserve((size_t)h->chunks * m * P * P));
  h->nsim = nsim;
  return SGDLM_OK;
}

// Re-sizes the LU scratch after the elimination plan changed (simulation memory
// already allocated).
int replan_sim(sgdlm_engine *h) {
  if (!h->sim_init) return SGDLM_OK;
  LuPlan pl;
  int st = plan_sim(h, (long)h->nsim, &pl);
  if (st) return st;
  if (pl.scratch_elems_total * h->tsize() > h->lu_scratch.count) {
    CK(h->lu_scratch.alloc(pl.scratch_elems_total * h->tsize()));
  }
  h->plan = pl;
  return SGDLM_OK;
}

// Validates a parental set: p_j <= P, and the Gamma positions (sp < m*m) hit
// off-diagonal cells at most once.  The reference does not check; a diagonal
// position races with fillGammas' unit diagonal (kernel_functions.cuh:830-840)
// and a repeated one with itself, so both are rejected here.
int validate_parents(sgdlm_engine *h, const unsigned *p, const unsigned *sp) {
  const size_t m = h->m, P = h->P, mm = m * m;
  if (p)
    for (size_t j = 0; j < m; ++j)
      if (p[j] > P) return h->fail(SGDLM_ERR_BAD_ARG, "p[j] exceeds max_p");
  if (sp) {
    std::set<unsigned> seen;
    for (size_t e = 0; e < m * P; ++e) {
      const unsigned pos = sp[e];
      if ((size_t)pos >= mm) continue;
      if (pos % m == pos / m)
        return h->fail(SGDLM_ERR_BAD_ARG, "sp addresses a diagonal entry of (I - Gamma)");
      if (!seen.insert(pos).second)
        return h->fail(SGDLM_ERR_BAD_ARG, "sp addresses the same entry of (I - Gamma) twice");
    }
  }
  return SGDLM_OK;
}

template <typename T> T *as(DevBuf<unsigned char> &b) { return reinterpret_cast<T *>(b.ptr); }

// The device-side epoch counter (read by the fused step) follows the host's, so
// that API calls and fused steps never reuse an epoch.
void advance_device_epoch(sgdlm_engine *h, uint32_t delta) {
  if (h->dev_epoch.ptr) {
    launch_advance_epoch(h->stream, h->dev_epoch.ptr, delta);
    h->launches += 1;
  }
}

// The sampler's draw-major copy of the Gamma entries (read by the LU and
// iterative-solve kernels).
template <typename T> GammaDraws<T> gamma_draws(sgdlm_engine *h) {
  return GammaDraws<T>{as<T>(h->theta_g), h->g_rowptr.ptr, h->sp.ptr, h->g_nnz};
}

// sample -> LU -> fallback, from the given normal-gamma parameters (posterior
// for VB, forecasting prior for forecasts).
template <typename T>
void sample_draws(sgdlm_engine *h, const double *m_t, const double *C_t, const double *n_t,
                  const double *s_t, RngKey key) {
  const int m = (int)h->m, P = (int)h->P;
  const long n = (long)h->nsim;
  launch_cholesky(h->stream, m, P, h->p.ptr, C_t, h->U64.ptr, h->U32.ptr);
  const T *U = std::is_same<T, float>::value ? reinterpret_cast<const T *>(h->U32.ptr)
                                              : reinterpret_cast<const T *>(h->U64.ptr);
  launch_sample<T>(h->stream, m, P, n, m_t, n_t, s_t, U, key, as<T>(h->lambda), as<T>(h->theta),
                   gamma_draws<T>(h), h->draw_flags.ptr, h->p.ptr);
  h->launches += 2;
}

// Small systems: one warp per draw, partial pivoting, no redo.
bool warp_lu(const sgdlm_engine *h) { return h->m <= (size_t)kWarpLuMaxM && h->lu_opt.allow_warp; }

// Forecasts of FP32 draws are solved iteratively first (block LU path only).
template <typename T> bool iterative_forecast(const sgdlm_engine *h) {
  return std::is_same<T, float>::value && h->forecast_iterative && h->jac.ok && !warp_lu(h);
}

template <typename T>
int lu_draws(sgdlm_engine *h, const double *x, RngKey key, double *y) {
  const long n = (long)h->nsim;
  const bool refine = (h->precision != SGDLM_PRECISION_FP64);
  const GammaRows rows{h->g_rowptr.ptr, h->g_ent.ptr, h->g_extptr.ptr, h->g_extk.ptr};
  if (x) {
    const size_t nx = h->m * h->P;
    launch_to_float(h->stream, nx, x, h->x32.ptr);
    launch_forecast_nu<T>(h->stream, (int)h->m, (int)h->P, n, rows, as<T>(h->theta), x,
                          h->x32.ptr, as<T>(h->lambda), key, h->nu_fc.ptr);
    h->launches += 2;
  }
  if (warp_lu(h)) {
    launch_lu_warp<T>(h->stream, (int)h->m, (int)h->P, n, h->num_sms, h->sp.ptr, as<T>(h->theta),
                      h->logdet.ptr, h->draw_flags.ptr,
                      x ? h->nu_fc.ptr : nullptr, x ? y : nullptr);
    h->launches += 1;
    return SGDLM_OK;
  }
  // forecasts of FP32 draws: the iterative solve first; the LU kernels then
  // factor only the draws it leaves in jac_list
  const bool iterative = iterative_forecast<T>(h) && x;
  if (iterative) {
    CK(cudaMemsetAsync(h->jac_list.ptr, 0, sizeof(int), h->stream));
    launch_forecast_jacobi(h->stream, h->jac, (int)h->m, (int)h->P, n, rows,
                           reinterpret_cast<const float *>(h->theta_g.ptr), h->g_nnz, h->nu_fc.ptr, y,
                           h->logdet.ptr, h->jac_list.ptr);
    h->launches += 1;
  }
  // the fast pass appends the draws it flags to pivot_list; the redo visits those
  CK(cudaMemsetAsync(h->pivot_list.ptr, 0, sizeof(int), h->stream));
  launch_lu<T>(h->stream, h->plan, n, h->elim_dev, h->sp.ptr, as<T>(h->theta),
               as<T>(h->theta_g), as<T>(h->lu_scratch), h->logdet.ptr, h->draw_flags.ptr, x, as<T>(h->lambda), key,
               refine, y, rows, x ? h->nu_fc.ptr : nullptr, h->pivot_list.ptr,
               iterative ? h->jac_list.ptr : nullptr);
  launch_lu_fallback<T>(h->stream, h->plan, n, h->elim_dev, h->sp.ptr, as<T>(h->theta),
                        as<T>(h->theta_g), as<T>(h->lu_scratch), h->logdet.ptr, h->draw_flags.ptr, x,
                        as<T>(h->lambda), key, y, rows, h->pivot_list.ptr);
  h->launches += 2;
  return SGDLM_OK;
}

template <typename T> void vb_moments(sgdlm_engine *h, double *w) {
  const int m = (int)h->m, P = (int)h->P;
  const long n = (long)h->nsim;
  VbScratch scr{h->part_a.ptr, h->part_b.ptr, h->chunks, h->chunk_draws};
  launch_vb<T>(h->stream, m, P, n, h->p.ptr, h->n_t.ptr, h->s_t.ptr, w, as<T>(h->lambda),
               as<T>(h->theta), scr, h->mean_m.ptr, h->mean_C.ptr, h->mean_n.ptr,
               h->mean_s.ptr, h->mean_lambda.ptr, h->mean_log_lambda.ptr, h->mean_Q.ptr,
               h->series_flags.ptr);
  h->launches += 4;
}

// ---- learned importance proposal ------------------------------------------------

// splitmix64 (Steele, Lea & Flood 2014) and Box-Muller normals for the initial
// weights: the same values on every host.
uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double host_normal(uint64_t &st) {
  const double u1 = ((splitmix64(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  const double u2 = ((splitmix64(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

// Buffers and fresh weights for the current (m, max_p): W1 ~ N(0, 1/F),
// W2 ~ N(0, 1/H), W3 = 0 and zero biases, so that an untrained network leaves
// the naive posterior unchanged.
int proposal_ensure(sgdlm_engine *h) {
  ProposalState &q = h->prop;
  if (q.w.ptr && q.m == h->m && q.P == h->P) return SGDLM_OK;
  if (h->P > (size_t)kProposalMaxP)
    return h->fail(SGDLM_ERR_UNSUPPORTED, "the learned proposal serves max_p <= 24");
  cudaStreamSynchronize(h->stream);
  const sgdlm_proposal_config cfg = q.cfg;
  q.release();
  const int m = (int)h->m, P = (int)h->P, F = proposal_features(P), O = proposal_outputs(P);
  q.L = mlp_layout(F, O);
  const long H = q.L.H;
  q.cap = (long)std::max(1, cfg.train_steps) * m;
  const long rows = std::max<long>(cfg.batch, m);
  CK(q.w.alloc(q.L.total));
  CK(q.grad.alloc(q.L.total));
  CK(q.m1.alloc(q.L.total));
  CK(q.m2.alloc(q.L.total));
  CK(q.w16.alloc(q.L.total));
  CK(q.X.alloc((size_t)m * F));
  CK(q.Y.alloc((size_t)m * O));
  CK(q.M.alloc((size_t)m * O));
  CK(q.bX.alloc((size_t)q.cap * F));
  CK(q.bY.alloc((size_t)q.cap * O));
  CK(q.bM.alloc((size_t)q.cap * O));
  CK(q.Xb.alloc((size_t)cfg.batch * F));
  CK(q.Yb.alloc((size_t)cfg.batch * O));
  CK(q.Mb.alloc((size_t)cfg.batch * O));
  for (auto *b : {&q.Z1, &q.A1, &q.Z2, &q.A2, &q.dA, &q.dA2}) CK(b->alloc((size_t)rows * H));
  CK(q.Out.alloc((size_t)rows * O));
  CK(q.dOut.alloc((size_t)rows * O));
  CK(q.fsum.alloc(2 * (size_t)F + 1));
  CK(q.loss.alloc(1));
  CK(q.mq.alloc((size_t)m * P));
  CK(q.nq.alloc(m));
  CK(q.sq.alloc(m));
  CK(q.cst.alloc(m));
  CK(q.Uq64.alloc((size_t)m * P * P));
  CK(q.Uq32.alloc((size_t)m * P * P));
  std::vector<float> w(q.L.total, 0.f);
  uint64_t st = cfg.seed;
  const double s1 = 1.0 / std::sqrt((double)F), s2 = 1.0 / std::sqrt((double)H);
  for (long e = 0; e < H * F; ++e) w[q.L.w1 + e] = (float)(s1 * host_normal(st));
  for (long e = 0; e < H * H; ++e) w[q.L.w2 + e] = (float)(s2 * host_normal(st));
  CK(cudaMemcpyAsync(q.w.ptr, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  mlp_refresh_bf16(h->stream, q.L, q.w.ptr, q.w16.ptr);
  h->launches += 1;
  q.cfg = cfg;
  q.m = h->m;
  q.P = h->P;
  q.info.deployed = cfg.train_steps <= 0 ? 1 : 0;
  return sync(h);
}

// The pairs of this call (naive posterior in m_t.., VB refit in mean_..) into
// the replay buffer, then iters_per_step Adam iterations on random batches.
int proposal_train(sgdlm_engine *h) {
  ProposalState &q = h->prop;
  cudaStream_t s = h->stream;
  const int m = (int)h->m, P = (int)h->P, F = q.L.F, O = q.L.O;
  launch_proposal_features(s, m, P, h->p.ptr, h->sp.ptr, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr,
                           h->s_t.ptr, q.X.ptr);
  launch_proposal_targets(s, m, P, h->p.ptr, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr, h->s_t.ptr,
                          h->mean_m.ptr, h->mean_C.ptr, h->mean_n.ptr, h->mean_s.ptr, q.Y.ptr,
                          q.M.ptr);
  launch_replay_append(s, m, F, O, q.pos, q.cap, q.X.ptr, q.Y.ptr, q.M.ptr, q.bX.ptr, q.bY.ptr,
                       q.bM.ptr, q.fsum.ptr);
  h->launches += 3;
  q.pos = (q.pos + m) % q.cap;
  q.count = std::min(q.count + m, q.cap);
  const int B = q.cfg.batch;
  for (int it = 0; it < q.cfg.iters_per_step; ++it) {
    const uint64_t step = ++q.info.adam_steps;
    launch_replay_gather(s, B, F, O, q.count, q.cfg.seed, step, q.bX.ptr, q.bY.ptr, q.bM.ptr,
                         q.fsum.ptr, q.Xb.ptr, q.Yb.ptr, q.Mb.ptr);
    mlp_forward(s, q.L, B, q.Xb.ptr, q.w.ptr, q.w16.ptr, q.acts());
    mlp_loss_backward(s, q.L, B, q.Xb.ptr, q.Yb.ptr, q.Mb.ptr, q.w16.ptr, q.acts(), q.grad.ptr,
                      q.loss.ptr);
    mlp_adam(s, q.L, q.w.ptr, q.w16.ptr, q.grad.ptr, q.m1.ptr, q.m2.ptr, (float)q.cfg.lr,
             (long)step);
    h->launches += 16;
  }
  q.info.training_calls += 1;
  q.info.samples = (uint64_t)q.count;
  if ((long)q.info.training_calls >= q.cfg.train_steps) q.info.deployed = 1;
  double loss = NAN;
  int st = d2h(h, &loss, q.loss.ptr, sizeof(double));
  if (st) return st;
  if ((st = sync(h))) return st;
  q.info.last_loss = loss;
  return SGDLM_OK;
}

// Draws from the learned proposal and their exact log weights (in q.logw), then
// the normalised weights.  Precondition: the proposal's buffers exist.
template <typename T>
int learned_draws(sgdlm_engine *h, RngKey key) {
  ProposalState &q = h->prop;
  cudaStream_t s = h->stream;
  const int m = (int)h->m, P = (int)h->P, F = q.L.F;
  const long n = (long)h->nsim;
  if (q.lr.count != (size_t)m * n) {
    CK(q.lr.alloc((size_t)m * n));
    CK(q.logw.alloc(n));
  }
  launch_cholesky(s, m, P, h->p.ptr, h->C_t.ptr, h->U64.ptr, h->U32.ptr);
  launch_proposal_features(s, m, P, h->p.ptr, h->sp.ptr, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr,
                           h->s_t.ptr, q.X.ptr);
  launch_normalise(s, m, F, q.fsum.ptr, q.X.ptr);
  mlp_forward(s, q.L, m, q.X.ptr, q.w.ptr, q.w16.ptr, q.acts());
  T *Uq = std::is_same<T, float>::value ? reinterpret_cast<T *>(q.Uq32.ptr)
                                        : reinterpret_cast<T *>(q.Uq64.ptr);
  launch_proposal_params<T>(s, m, P, h->p.ptr, q.Out.ptr, h->m_t.ptr, h->n_t.ptr, h->s_t.ptr,
                            h->U64.ptr, q.mq.ptr, q.nq.ptr, q.sq.ptr, q.Uq64.ptr, Uq, q.cst.ptr);
  launch_sample<T>(s, m, P, n, q.mq.ptr, q.nq.ptr, q.sq.ptr, Uq, key, as<T>(h->lambda),
                   as<T>(h->theta), gamma_draws<T>(h), h->draw_flags.ptr, h->p.ptr);
  h->launches += 8;
  CK(cudaEventRecord(h->ev[1], s));
  int st = lu_draws<T>(h, nullptr, key, nullptr);
  if (st) return st;
  CK(cudaEventRecord(h->ev[2], s));
  const T *U = std::is_same<T, float>::value ? reinterpret_cast<const T *>(h->U32.ptr)
                                              : reinterpret_cast<const T *>(h->U64.ptr);
  launch_log_ratio<T>(s, m, P, n, h->p.ptr, as<T>(h->theta), as<T>(h->lambda), h->m_t.ptr,
                      h->n_t.ptr, h->s_t.ptr, U, q.mq.ptr, q.nq.ptr, q.sq.ptr, Uq, q.cst.ptr,
                      h->logdet.ptr, q.lr.ptr, q.logw.ptr);
  launch_weights(s, n, q.logw.ptr, h->w.ptr, h->stats6.ptr, h->wpart.ptr);
  h->launches += 5;
  return SGDLM_OK;
}

// Reads back the per-draw and per-series status words into the stats block.
int collect_flags(sgdlm_engine *h, bool with_series) {
  std::vector<int> f(h->nsim);
  CK(cudaMemcpyAsync(f.data(), h->draw_flags.ptr, h->nsim * sizeof(int), cudaMemcpyDeviceToHost,
                     h->stream));
  std::vector<int> sf;
  if (with_series) {
    sf.resize(h->m);
    CK(cudaMemcpyAsync(sf.data(), h->series_flags.ptr, h->m * sizeof(int),
                       cudaMemcpyDeviceToHost, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  uint64_t piv = 0, piv_full = 0, sing = 0, cap = 0, newton = 0;
  for (int v : f) {
    piv += (v & DRAW_FLAG_REDONE) ? 1 : 0;
    piv_full += (v & DRAW_FLAG_FULL_PIVOT) ? 1 : 0;
    sing += (v & DRAW_FLAG_SINGULAR) ? 1 : 0;
    cap += (v & DRAW_FLAG_GAMMA_CAP) ? 1 : 0;
  }
  for (int v : sf) newton += (v & 2) ? 1 : 0;
  h->stats.draws_pivoted = piv;
  h->stats.draws_pivoted_full = piv_full;
  h->stats.draws_singular = sing;
  h->stats.gamma_cap_hits = cap;
  if (with_series) h->stats.newton_fallbacks = newton;
  if (sing) h->log(LOG_WARNING, "%llu draws had a singular (I - Gamma)", (unsigned long long)sing);
  if (cap) h->log(LOG_WARNING, "%llu gamma draws hit the sampler's attempt cap", (unsigned long long)cap);
  return SGDLM_OK;
}

template <typename T>
int vb_posterior(sgdlm_engine *h, double *o_m, double *o_C, double *o_n, double *o_s,
                 double *o_w, double *o_sum) {
  const size_t m = h->m, P = h->P, n = h->nsim;
  cudaStream_t s = h->stream;
  int st;
  ProposalState &q = h->prop;
  const bool use_learned = q.cfg.mode == SGDLM_PROPOSAL_LEARNED;
  if (use_learned && (st = proposal_ensure(h))) return st;
  const bool learned = use_learned && q.info.deployed;
  const RngKey key = h->key((uint32_t)h->epoch);
  h->epoch += 1;
  advance_device_epoch(h, 1);
  q.info.ess_learned = q.info.ess_plain = 0.0;
  q.info.used_learned = 0;
  CK(cudaEventRecord(h->ev[0], s));
  CK(cudaMemsetAsync(h->draw_flags.ptr, 0, n * sizeof(int), s));
  bool plain = !learned;
  if (learned) {
    if ((st = learned_draws<T>(h, key))) return st;
    CK(cudaEventRecord(h->ev[3], s));
    double st6[6];
    if ((st = d2h(h, st6, h->stats6.ptr, 6 * sizeof(double)))) return st;
    if ((st = sync(h))) return st;
    q.info.learned_calls += 1;
    q.info.ess_learned = st6[1];
    if (!(st6[1] >= q.cfg.ess_fraction * (double)n)) {
      // fallback: the plain proposal on an independent stream (the key's high
      // word flipped), as the caller would run it
      q.info.fallbacks += 1;
      plain = true;
      CK(cudaMemsetAsync(h->draw_flags.ptr, 0, n * sizeof(int), s));
    } else {
      q.info.used_learned = 1;
    }
  }
  if (plain) {
    RngKey kp = key;
    if (learned) kp.k1 ^= 0x80000000u;
    sample_draws<T>(h, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr, h->s_t.ptr, kp);
    CK(cudaEventRecord(h->ev[1], s));
    if ((st = lu_draws<T>(h, nullptr, kp, nullptr))) return st;
    CK(cudaEventRecord(h->ev[2], s));
    launch_weights(s, (long)n, h->logdet.ptr, h->w.ptr, h->stats6.ptr, h->wpart.ptr);
    h->launches += 3;
    CK(cudaEventRecord(h->ev[3], s));
  }
  vb_moments<T>(h, h->w.ptr);
  CK(cudaEventRecord(h->ev[4], s));
  if (o_m && (st = d2h(h, o_m, h->mean_m.ptr, P * m * sizeof(double)))) return st;
  if (o_C && (st = d2h(h, o_C, h->mean_C.ptr, P * P * m * sizeof(double)))) return st;
  if (o_n && (st = d2h(h, o_n, h->mean_n.ptr, m * sizeof(double)))) return st;
  if (o_s && (st = d2h(h, o_s, h->mean_s.ptr, m * sizeof(double)))) return st;
  if (o_w && (st = d2h(h, o_w, h->w.ptr, n * sizeof(double)))) return st;
  double st6[8];
  if ((st = d2h(h, st6, h->stats6.ptr, 6 * sizeof(double)))) return st;
  if ((st = sync(h))) return st;
  if (o_sum) *o_sum = st6[0];
  h->stats.sum_det_weights = st6[0];
  h->stats.ess = st6[1];
  h->stats.max_log_det = st6[2];
  if (plain) q.info.ess_plain = st6[1];
  h->stats.ms_sample = elapsed(h->ev[0], h->ev[1]);
  h->stats.ms_lu = elapsed(h->ev[1], h->ev[2]);
  h->stats.ms_weights = elapsed(h->ev[2], h->ev[3]);
  h->stats.ms_vb = elapsed(h->ev[3], h->ev[4]);
  h->stats.ms_total = elapsed(h->ev[0], h->ev[4]);
  if ((st = collect_flags(h, true))) return st;
  // training pairs: calls before deployment whose ESS passes the README's gate
  if (use_learned && !q.info.deployed && st6[1] > 0.5 * (double)n) return proposal_train(h);
  return SGDLM_OK;
}

template <typename T>
int forecast(sgdlm_engine *h, double *o_y, const double *x, double *o_lambda, double *o_theta,
             bool use_existing) {
  const size_t m = h->m, P = h->P, n = h->nsim;
  cudaStream_t s = h->stream;
  int st;
  if ((st = h2d(h, h->x_t.ptr, x, P * m * sizeof(double)))) return st;
  const RngKey key = h->key((uint32_t)h->epoch);
  h->epoch += 1;
  advance_device_epoch(h, 1);
  CK(cudaEventRecord(h->ev[0], s));
  CK(cudaMemsetAsync(h->draw_flags.ptr, 0, n * sizeof(int), s));
  if (!use_existing)
    sample_draws<T>(h, h->fm_t.ptr, h->fC_t.ptr, h->fn_t.ptr, h->fs_t.ptr, key);
  CK(cudaEventRecord(h->ev[1], s));
  // a page-locked, device-mapped destination receives the draws straight from the
  // LU kernels (over the host link while they run); any other goes through y_fc
  double *ydst = h->y_fc.ptr;
  if (o_y) {
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, o_y) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
        pa.devicePointer != nullptr)
      ydst = static_cast<double *>(pa.devicePointer);
    else
      (void)cudaGetLastError();  // pageable memory is not an error here
  }
  if ((st = lu_draws<T>(h, h->x_t.ptr, key, ydst))) return st;
  CK(cudaEventRecord(h->ev[2], s));
  int factored = (int)n;
  if (iterative_forecast<T>(h) && (st = d2h(h, &factored, h->jac_list.ptr, sizeof(int))))
    return st;
  if (o_y && ydst == h->y_fc.ptr && (st = d2h(h, o_y, h->y_fc.ptr, n * m * sizeof(double))))
    return st;
  std::vector<T> lam, th;
  if (o_lambda) {
    lam.resize(m * n);
    if ((st = d2h(h, lam.data(), h->lambda.ptr, m * n * sizeof(T)))) return st;
  }
  if (o_theta) {
    th.resize(m * n * P);
    if ((st = d2h(h, th.data(), h->theta.ptr, m * n * P * sizeof(T)))) return st;
  }
  if ((st = sync(h))) return st;
  // debug exports use the reference's draw-major layouts:
  // lambdas (m, nsim), thetas (max_p, m, nsim)   (RcppWrapper.cpp:557-569)
  if (o_lambda)
    for (size_t j = 0; j < m; ++j)
      for (size_t i = 0; i < n; ++i) o_lambda[i * m + j] = (double)lam[j * n + i];
  if (o_theta)
    for (size_t j = 0; j < m; ++j)
      for (size_t i = 0; i < n; ++i)
        for (size_t k = 0; k < P; ++k) o_theta[(i * m + j) * P + k] = (double)th[(j * n + i) * P + k];
  h->stats.ms_sample = elapsed(h->ev[0], h->ev[1]);
  h->stats.ms_lu_forecast = elapsed(h->ev[1], h->ev[2]);
  h->stats.forecast_draws_factored = (uint64_t)factored;
  h->stats.ms_total = elapsed(h->ev[0], h->ev[2]);
  return collect_flags(h, false);
}

// Device memory of the evolution matrices (P x P x m, FP64 and FP32), zeroed
// (manageEvoMemory, HostWrapperImpl.cu:231-279).
int alloc_evolution_matrix(sgdlm_engine *h) {
  const size_t n = h->P * h->P * h->m;
  if (h->G_t.count != n) {
    CK(h->G_t.alloc(n));
    CK(h->G32.alloc(n));
    CK(cudaMemsetAsync(h->G_t.ptr, 0, n * sizeof(double), h->stream));
    CK(cudaMemsetAsync(h->G32.ptr, 0, n * sizeof(float), h->stream));
  }
  return SGDLM_OK;
}

// Copies the evolution matrices (P x P x m, column-major per series) to the device
// (setEvolutionMatrix, HostWrapperImpl.cu:737-754), with an FP32 copy.
int upload_evolution_matrix(sgdlm_engine *h, const double *G) {
  const size_t n = h->P * h->P * h->m;
  int st = alloc_evolution_matrix(h);
  if (st) return st;
  CK(cudaMemcpyAsync(h->G_t.ptr, G, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  launch_to_float(h->stream, n, h->G_t.ptr, h->G32.ptr);
  h->launches += 1;
  return SGDLM_OK;
}

template <typename T> int evolve(sgdlm_engine *h, bool with_G = false) {
  const int m = (int)h->m, P = (int)h->P;
  const long n = (long)h->nsim;
  const RngKey key = h->key((uint32_t)h->epoch);
  h->epoch += 1;
  advance_device_epoch(h, 1);
  // chol(W) of the forecasting copy (SGDLM.cu:742-747); the forecasting r, c and
  // W are not re-discounted between steps (HostWrapperImpl.cu:891-900)
  launch_cholesky(h->stream, m, P, h->p.ptr, h->fW_t.ptr, h->U64.ptr, h->U32.ptr);
  const T *UW = std::is_same<T, float>::value ? reinterpret_cast<const T *>(h->U32.ptr)
                                               : reinterpret_cast<const T *>(h->U64.ptr);
  launch_evolve<T>(h->stream, m, P, n, h->p.ptr, h->fn_t.ptr, h->fs_t.ptr, h->beta.ptr, UW,
                   key, (h->compat & SGDLM_COMPAT_UNSCALED_EVOLUTION) != 0,
                   (h->compat & SGDLM_COMPAT_BETA_NO_BOOST) != 0, as<T>(h->lambda),
                   as<T>(h->theta), gamma_draws<T>(h), h->draw_flags.ptr,
                   with_G ? (std::is_same<T, float>::value
                                 ? reinterpret_cast<const T *>(h->G32.ptr)
                                 : reinterpret_cast<const T *>(h->G_t.ptr))
                          : nullptr);
  h->launches += 2;
  return sync(h);
}

int copy_forecast_priors(sgdlm_engine *h) {
  const size_t m = h->m, P = h->P;
  cudaStream_t s = h->stream;
  CK(cudaMemcpyAsync(h->fn_t.ptr, h->n_t.ptr, m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(h->fs_t.ptr, h->s_t.ptr, m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(h->fm_t.ptr, h->m_t.ptr, P * m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(h->fC_t.ptr, h->C_t.ptr, P * P * m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(h->fW_t.ptr, h->W_t.ptr, P * P * m * sizeof(double), cudaMemcpyDeviceToDevice, s));
  return SGDLM_OK;
}

// Fused step body; every launch on the stream, no host synchronisation.
template <typename T>
int filter_step(sgdlm_engine *h, const double *d_y, const double *d_F, const double *d_x,
                double ess_threshold, double *d_forecast, double *d_w, double *d_stats) {
  const int m = (int)h->m, P = (int)h->P;
  const long n = (long)h->nsim;
  cudaStream_t s = h->stream;
  RngKey key_vb = h->key(0);
  key_vb.dev_epoch = h->dev_epoch.ptr;
  RngKey key_fc = h->key(1);
  key_fc.dev_epoch = h->dev_epoch.ptr;
  double *w = d_w ? d_w : h->w.ptr;
  double *yout = d_forecast ? d_forecast : h->y_fc.ptr;
  launch_posterior(s, m, P, h->p.ptr, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr, h->s_t.ptr, d_y, d_F);
  h->launches += 1;
  CK(cudaMemsetAsync(h->draw_flags.ptr, 0, n * sizeof(int), s));
  sample_draws<T>(h, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr, h->s_t.ptr, key_vb);
  int st = lu_draws<T>(h, nullptr, key_vb, nullptr);
  if (st) return st;
  launch_weights(s, n, h->logdet.ptr, w, h->stats6.ptr, h->wpart.ptr);
  vb_moments<T>(h, w);
  launch_gate(s, m, P, h->stats6.ptr, ess_threshold, h->mean_m.ptr, h->mean_C.ptr,
              h->mean_n.ptr, h->mean_s.ptr, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr, h->s_t.ptr,
              h->stats6.ptr + 6);
  launch_prior(s, m, P, h->p.ptr, h->C_t.ptr, h->n_t.ptr, h->W_t.ptr, h->beta.ptr, h->delta.ptr);
  h->launches += 5;  // three for the weights, the gate, the prior
  if (d_x) {
    st = copy_forecast_priors(h);
    if (st) return st;
    CK(cudaMemsetAsync(h->draw_flags.ptr, 0, n * sizeof(int), s));
    sample_draws<T>(h, h->fm_t.ptr, h->fC_t.ptr, h->fn_t.ptr, h->fs_t.ptr, key_fc);
    if ((st = lu_draws<T>(h, d_x, key_fc, yout))) return st;
  }
  if (d_stats) {
    // {ESS, sum_det, accepted, max_log_det, n_finite, sum_w2}
    CK(cudaMemcpyAsync(d_stats + 0, h->stats6.ptr + 1, sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_stats + 1, h->stats6.ptr + 0, sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_stats + 2, h->stats6.ptr + 6, sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d_stats + 3, h->stats6.ptr + 2, 3 * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  launch_advance_epoch(s, h->dev_epoch.ptr, 2);
  h->launches += 1;
  h->epoch += 2;  // host copy follows the device counter (one call = one advance)
  CK(cudaGetLastError());
  return SGDLM_OK;
}

template <typename T>
int export_draws(sgdlm_engine *h, double *o_lambda, double *o_theta, double *o_logdet) {
  const size_t m = h->m, P = h->P, n = h->nsim;
  std::vector<T> lam, th;
  int st;
  if (o_lambda) {
    lam.resize(m * n);
    if ((st = d2h(h, lam.data(), h->lambda.ptr, m * n * sizeof(T)))) return st;
  }
  if (o_theta) {
    th.resize(m * n * P);
    if ((st = d2h(h, th.data(), h->theta.ptr, m * n * P * sizeof(T)))) return st;
  }
  if (o_logdet && (st = d2h(h, o_logdet, h->logdet.ptr, n * sizeof(double)))) return st;
  if ((st = sync(h))) return st;
  if (o_lambda)
    for (size_t j = 0; j < m; ++j)
      for (size_t i = 0; i < n; ++i) o_lambda[i * m + j] = (double)lam[j * n + i];
  if (o_theta)
    for (size_t j = 0; j < m; ++j)
      for (size_t i = 0; i < n; ++i)
        for (size_t k = 0; k < P; ++k) o_theta[(i * m + j) * P + k] = (double)th[(j * n + i) * P + k];
  return SGDLM_OK;
}

}  // namespace

#define HCHECK(h)                                  \
  do {                                             \
    if (!(h)) return SGDLM_ERR_BAD_ARG;            \
    cudaSetDevice((h)->device);                    \
  } while (0)

extern "C" {

int sgdlm_create(size_t no_gpus, sgdlm_handle *out) {
  if (!out) return SGDLM_ERR_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    fprintf(stderr, "[sgdlm] No cuda-enabled devices available.\n");
    return SGDLM_ERR_NO_DEVICE;
  }
  auto h = std::make_unique<sgdlm_engine>();
  // The engine lives on the calling thread's current device (device 0 unless the
  // caller selected another), as the reference's first GPU is device 0
  // (HostWrapperImpl.cu:39-40).
  if (cudaGetDevice(&h->device) != cudaSuccess) h->device = 0;
  if (no_gpus != 1)
    h->log(LOG_INFO, "no_gpus = %zu requested; this engine runs on one GPU", no_gpus);
  h->no_gpus = 1;
  cudaError_t e = cudaSetDevice(h->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  for (int k = 0; k < 8 && e == cudaSuccess; ++k) e = cudaEventCreate(&h->ev[k]);
  if (e != cudaSuccess) {
    fprintf(stderr, "[sgdlm] CUDA initialisation failed: %s\n", cudaGetErrorString(e));
    return SGDLM_ERR_DEVICE;
  }
  *out = h.release();
  return SGDLM_OK;
}

int sgdlm_destroy(sgdlm_handle h) {
  if (!h) return SGDLM_OK;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  release_all(h);
  for (auto &e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return SGDLM_OK;
}

int sgdlm_init_memory(sgdlm_handle h, size_t m, size_t max_p) {
  HCHECK(h);
  if (m < 1 || max_p < 1) return h->fail(SGDLM_ERR_BAD_DIM, "m and max_p must be positive");
  if (max_p > kMaxP) return h->fail(SGDLM_ERR_UNSUPPORTED, "max_p above 64 is not supported");
  if (m > 65535) return h->fail(SGDLM_ERR_UNSUPPORTED, "m above 65535 does not fit the sp encoding");
  cudaStreamSynchronize(h->stream);
  release_all(h);
  h->m = m;
  h->P = max_p;
  int st = alloc_state(h);
  if (!st && h->use_evo) st = alloc_evolution_matrix(h);  // HostWrapperImpl.cu:225
  if (st) {
    release_all(h);
    return st;
  }
  h->mem_init = true;
  return SGDLM_OK;
}

int sgdlm_clear_memory(sgdlm_handle h) {
  HCHECK(h);
  cudaStreamSynchronize(h->stream);
  release_all(h);
  return SGDLM_OK;
}

int sgdlm_get_no_series(sgdlm_handle h, size_t *m) {
  HCHECK(h);
  if (!m) return SGDLM_ERR_BAD_ARG;
  *m = h->m;
  return SGDLM_OK;
}
int sgdlm_get_max_p(sgdlm_handle h, size_t *max_p) {
  HCHECK(h);
  if (!max_p) return SGDLM_ERR_BAD_ARG;
  *max_p = h->P;
  return SGDLM_OK;
}
int sgdlm_get_no_gpus(sgdlm_handle h, size_t *no_gpus) {
  HCHECK(h);
  if (!no_gpus) return SGDLM_ERR_BAD_ARG;
  *no_gpus = h->no_gpus;
  return SGDLM_OK;
}

// initSimMemory (HostWrapperImpl.cu:321-332): nsim_batch is clamped to nsim.
int sgdlm_init_sim_memory(sgdlm_handle h, size_t nsim, size_t nsim_batch) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (nsim < 1) return h->fail(SGDLM_ERR_BAD_ARG, "nsim must be positive");
  if (nsim > 0x7FFFFFFFu) return h->fail(SGDLM_ERR_UNSUPPORTED, "nsim above 2^31 - 1 is not supported");
  cudaStreamSynchronize(h->stream);
  int st = alloc_sim(h, nsim);
  if (st) {
    release_sim(h);
    return st;
  }
  h->nsim_batch = nsim_batch > nsim ? nsim : nsim_batch;
  h->sim_init = true;
  return SGDLM_OK;
}

int sgdlm_clear_sim_memory(sgdlm_handle h) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  cudaStreamSynchronize(h->stream);
  release_sim(h);
  return SGDLM_OK;
}

int sgdlm_get_nsim(sgdlm_handle h, size_t *nsim) {
  HCHECK(h);
  if (!nsim) return SGDLM_ERR_BAD_ARG;
  *nsim = h->nsim;
  return SGDLM_OK;
}
int sgdlm_get_nsim_batch(sgdlm_handle h, size_t *nsim_batch) {
  HCHECK(h);
  if (!nsim_batch) return SGDLM_ERR_BAD_ARG;
  *nsim_batch = h->nsim_batch;
  return SGDLM_OK;
}
int sgdlm_is_prior(sgdlm_handle h, int *is_prior) {
  HCHECK(h);
  if (!is_prior) return SGDLM_ERR_BAD_ARG;
  *is_prior = h->is_prior ? 1 : 0;
  return SGDLM_OK;
}
int sgdlm_set_is_prior(sgdlm_handle h, int is_prior) {
  HCHECK(h);
  h->is_prior = is_prior != 0;
  return SGDLM_OK;
}

int sgdlm_get_parameters(sgdlm_handle h, double *m_t, double *C_t, double *n_t, double *s_t) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  const size_t m = h->m, P = h->P;
  int st;
  if (m_t && (st = d2h(h, m_t, h->m_t.ptr, P * m * sizeof(double)))) return st;
  if (C_t && (st = d2h(h, C_t, h->C_t.ptr, P * P * m * sizeof(double)))) return st;
  if (n_t && (st = d2h(h, n_t, h->n_t.ptr, m * sizeof(double)))) return st;
  if (s_t && (st = d2h(h, s_t, h->s_t.ptr, m * sizeof(double)))) return st;
  return sync(h);
}

int sgdlm_set_parameters(sgdlm_handle h, const double *m_t, const double *C_t,
                         const double *n_t, const double *s_t) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  const size_t m = h->m, P = h->P;
  int st;
  if (m_t && (st = h2d(h, h->m_t.ptr, m_t, P * m * sizeof(double)))) return st;
  if (C_t && (st = h2d(h, h->C_t.ptr, C_t, P * P * m * sizeof(double)))) return st;
  if (n_t && (st = h2d(h, h->n_t.ptr, n_t, m * sizeof(double)))) return st;
  if (s_t && (st = h2d(h, h->s_t.ptr, s_t, m * sizeof(double)))) return st;
  return sync(h);
}

int sgdlm_get_discount_factors(sgdlm_handle h, double *beta, double *delta) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  const size_t m = h->m, P = h->P;
  int st;
  if (beta && (st = d2h(h, beta, h->beta.ptr, m * sizeof(double)))) return st;
  if (delta && (st = d2h(h, delta, h->delta.ptr, P * P * m * sizeof(double)))) return st;
  return sync(h);
}

int sgdlm_set_discount_factors(sgdlm_handle h, const double *beta, const double *delta) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  const size_t m = h->m, P = h->P;
  int st;
  if (beta && (st = h2d(h, h->beta.ptr, beta, m * sizeof(double)))) return st;
  if (delta && (st = h2d(h, h->delta.ptr, delta, P * P * m * sizeof(double)))) return st;
  return sync(h);
}

int sgdlm_get_parental_sets(sgdlm_handle h, unsigned *p, unsigned *sp) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (p) std::memcpy(p, h->h_p.data(), h->m * sizeof(unsigned));
  if (sp) std::memcpy(sp, h->h_sp.data(), h->m * h->P * sizeof(unsigned));
  return SGDLM_OK;
}

int sgdlm_set_parental_sets(sgdlm_handle h, const unsigned *p, const unsigned *sp) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  int st = validate_parents(h, p, sp);
  if (st) return st;
  const size_t m = h->m, P = h->P;
  if (p) {
    std::memcpy(h->h_p.data(), p, m * sizeof(unsigned));
    if ((st = h2d(h, h->p.ptr, p, m * sizeof(unsigned)))) return st;
  }
  if (sp) {
    std::memcpy(h->h_sp.data(), sp, m * P * sizeof(unsigned));
    if ((st = h2d(h, h->sp.ptr, sp, m * P * sizeof(unsigned)))) return st;
    if ((st = sync(h))) return st;
    if ((st = upload_gamma_rows(h))) return st;
    if ((st = upload_elimination(h))) return st;
    if ((st = replan_sim(h))) return st;
  }
  return sync(h);
}

int sgdlm_compute_posterior(sgdlm_handle h, const double *y_t, const double *F_t) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_prior(true)) return SGDLM_ERR_WRONG_STATE;
  if (!y_t || !F_t) return h->fail(SGDLM_ERR_BAD_ARG, "null input");
  const size_t m = h->m, P = h->P;
  int st;
  if ((st = h2d(h, h->y_t.ptr, y_t, m * sizeof(double)))) return st;
  if ((st = h2d(h, h->F_t.ptr, F_t, P * m * sizeof(double)))) return st;
  launch_posterior(h->stream, (int)m, (int)P, h->p.ptr, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr,
                   h->s_t.ptr, h->y_t.ptr, h->F_t.ptr);
  h->launches += 1;
  if ((st = sync(h))) return st;
  h->is_prior = false;
  return SGDLM_OK;
}

int sgdlm_compute_vb_posterior(sgdlm_handle h, double *mean_m_t, double *mean_C_t,
                               double *mean_n_t, double *mean_s_t, double *is_weights,
                               double *sum_det_weights) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
  if (!h->check_prior(false)) return SGDLM_ERR_WRONG_STATE;
  if (h->precision == SGDLM_PRECISION_FP64)
    return vb_posterior<double>(h, mean_m_t, mean_C_t, mean_n_t, mean_s_t, is_weights,
                                sum_det_weights);
  return vb_posterior<float>(h, mean_m_t, mean_C_t, mean_n_t, mean_s_t, is_weights,
                             sum_det_weights);
}

int sgdlm_compute_prior(sgdlm_handle h, int evolve_forecast_variables) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  const int m = (int)h->m, P = (int)h->P;
  if (evolve_forecast_variables) {
    launch_prior(h->stream, m, P, h->p.ptr, h->fC_t.ptr, h->fn_t.ptr, h->fW_t.ptr, h->beta.ptr,
                 h->delta.ptr);
    h->launches += 1;
    return sync(h);
  }
  if (!h->check_prior(false)) return SGDLM_ERR_WRONG_STATE;
  launch_prior(h->stream, m, P, h->p.ptr, h->C_t.ptr, h->n_t.ptr, h->W_t.ptr, h->beta.ptr,
               h->delta.ptr);
  h->launches += 1;
  int st = sync(h);
  if (st) return st;
  h->is_prior = true;
  return SGDLM_OK;
}

int sgdlm_get_evolution_matrix_configuration(sgdlm_handle h, int *use) {
  HCHECK(h);
  if (!use) return SGDLM_ERR_BAD_ARG;
  *use = h->use_evo ? 1 : 0;
  return SGDLM_OK;
}

int sgdlm_manage_evo_memory(sgdlm_handle h, int use) {
  HCHECK(h);
  if (use) {
    if (h->mem_init) {
      int st = alloc_evolution_matrix(h);
      if (st) return st;
      if ((st = sync(h))) return st;
    }
  } else {
    cudaStreamSynchronize(h->stream);
    h->G_t.release();
    h->G32.release();
  }
  h->use_evo = use != 0;
  return SGDLM_OK;
}

int sgdlm_get_evolution_matrix(sgdlm_handle h, double *G_t) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_use_evo()) return SGDLM_ERR_EVO_DISABLED;
  if (!G_t) return SGDLM_OK;  // a NULL destination copies nothing (HostWrapperImpl.cu:727)
  int st = alloc_evolution_matrix(h);
  if (st) return st;
  if ((st = d2h(h, G_t, h->G_t.ptr, h->P * h->P * h->m * sizeof(double)))) return st;
  return sync(h);
}

int sgdlm_set_evolution_matrix(sgdlm_handle h, const double *G_t) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_use_evo()) return SGDLM_ERR_EVO_DISABLED;
  if (!G_t) return SGDLM_OK;
  int st = upload_evolution_matrix(h, G_t);
  if (st) return st;
  return sync(h);
}

int sgdlm_compute_evo_prior(sgdlm_handle h, const double *G_tp1, int evolve_forecast_variables) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_use_evo()) return SGDLM_ERR_EVO_DISABLED;
  if (!G_tp1) return h->fail(SGDLM_ERR_BAD_ARG, "null evolution matrix");
  if (!evolve_forecast_variables && !h->check_prior(false)) return SGDLM_ERR_WRONG_STATE;
  int st = upload_evolution_matrix(h, G_tp1);
  if (st) return st;
  const int m = (int)h->m, P = (int)h->P;
  double *m_t = evolve_forecast_variables ? h->fm_t.ptr : h->m_t.ptr;
  double *C_t = evolve_forecast_variables ? h->fC_t.ptr : h->C_t.ptr;
  double *n_t = evolve_forecast_variables ? h->fn_t.ptr : h->n_t.ptr;
  double *W_t = evolve_forecast_variables ? h->fW_t.ptr : h->W_t.ptr;
  launch_prior(h->stream, m, P, h->p.ptr, C_t, n_t, W_t, h->beta.ptr, h->delta.ptr);
  launch_evo_prior(h->stream, m, P, h->p.ptr, m_t, C_t, h->G_t.ptr);
  h->launches += 2;
  if ((st = sync(h))) return st;
  if (!evolve_forecast_variables) h->is_prior = true;
  return SGDLM_OK;
}

int sgdlm_evolve_forecast_samples_evo(sgdlm_handle h, const double *G_tp1) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_use_evo()) return SGDLM_ERR_EVO_DISABLED;
  if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
  if (!G_tp1) return h->fail(SGDLM_ERR_BAD_ARG, "null evolution matrix");
  int st = upload_evolution_matrix(h, G_tp1);
  if (st) return st;
  return h->precision == SGDLM_PRECISION_FP64 ? evolve<double>(h, true) : evolve<float>(h, true);
}

int sgdlm_init_forecast_priors(sgdlm_handle h) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  int st = copy_forecast_priors(h);
  if (st) return st;
  return sync(h);
}

int sgdlm_evolve_forecast_samples(sgdlm_handle h) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
  return h->precision == SGDLM_PRECISION_FP64 ? evolve<double>(h) : evolve<float>(h);
}

int sgdlm_compute_forecast(sgdlm_handle h, double *y_tp1, const double *x_tp1, double *lambdas,
                           double *thetas, int use_existing_lambdas_and_thetas) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
  if (!h->check_prior(true)) return SGDLM_ERR_WRONG_STATE;
  if (!x_tp1) return h->fail(SGDLM_ERR_BAD_ARG, "null predictors");
  const bool ue = use_existing_lambdas_and_thetas != 0;
  return h->precision == SGDLM_PRECISION_FP64
             ? forecast<double>(h, y_tp1, x_tp1, lambdas, thetas, ue)
             : forecast<float>(h, y_tp1, x_tp1, lambdas, thetas, ue);
}

int sgdlm_get_draws(sgdlm_handle h, double *lambdas, double *thetas, double *log_dets) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
  return h->precision == SGDLM_PRECISION_FP64 ? export_draws<double>(h, lambdas, thetas, log_dets)
                                              : export_draws<float>(h, lambdas, thetas, log_dets);
}

int sgdlm_set_precision(sgdlm_handle h, int precision) {
  HCHECK(h);
  if (precision != SGDLM_PRECISION_FP64 && precision != SGDLM_PRECISION_MIXED)
    return h->fail(SGDLM_ERR_BAD_ARG, "unknown precision");
  if (precision == h->precision) return SGDLM_OK;
  const int old = h->precision;
  h->precision = precision;
  if (h->sim_init) {
    const size_t nsim = h->nsim, batch = h->nsim_batch;
    cudaStreamSynchronize(h->stream);
    int st = alloc_sim(h, nsim);
    if (st) {
      h->precision = old;
      alloc_sim(h, nsim);
      h->nsim_batch = batch;
      h->sim_init = true;
      return st;
    }
    h->nsim_batch = batch;
    h->sim_init = true;
  }
  return SGDLM_OK;
}
int sgdlm_set_elimination_levels(sgdlm_handle h, int levels) {
  HCHECK(h);
  if (levels < 0 || levels > 16) return h->fail(SGDLM_ERR_BAD_ARG, "levels must be in 0..16");
  h->elim_levels = levels;
  if (!h->mem_init) return SGDLM_OK;
  cudaStreamSynchronize(h->stream);
  int st = upload_elimination(h);
  if (st) return st;
  return replan_sim(h);
}

int sgdlm_get_elimination_info(sgdlm_handle h, int *levels, int *core_n) {
  HCHECK(h);
  if (levels) *levels = h->eplan.nlev;
  if (core_n) *core_n = h->eplan.core_n;
  return SGDLM_OK;
}

int sgdlm_get_precision(sgdlm_handle h, int *precision) {
  HCHECK(h);
  if (!precision) return SGDLM_ERR_BAD_ARG;
  *precision = h->precision;
  return SGDLM_OK;
}
int sgdlm_set_compat(sgdlm_handle h, unsigned flags) {
  HCHECK(h);
  h->compat = flags & SGDLM_COMPAT_REFERENCE;
  return SGDLM_OK;
}
int sgdlm_get_compat(sgdlm_handle h, unsigned *flags) {
  HCHECK(h);
  if (!flags) return SGDLM_ERR_BAD_ARG;
  *flags = h->compat;
  return SGDLM_OK;
}
int sgdlm_set_rng_state(sgdlm_handle h, uint64_t seed, uint64_t epoch) {
  HCHECK(h);
  h->seed = seed;
  h->epoch = epoch;
  if (h->dev_epoch.ptr) {
    const uint32_t e32 = (uint32_t)epoch;
    cudaMemcpyAsync(h->dev_epoch.ptr, &e32, sizeof e32, cudaMemcpyHostToDevice, h->stream);
    return sync(h);
  }
  return SGDLM_OK;
}
int sgdlm_get_rng_state(sgdlm_handle h, uint64_t *seed, uint64_t *epoch) {
  HCHECK(h);
  if (!seed || !epoch) return SGDLM_ERR_BAD_ARG;
  *seed = h->seed;
  *epoch = h->epoch;
  return SGDLM_OK;
}
int sgdlm_get_stats(sgdlm_handle h, sgdlm_stats *out) {
  HCHECK(h);
  if (!out) return SGDLM_ERR_BAD_ARG;
  *out = h->stats;
  return SGDLM_OK;
}
// configureLogLevel (rSGDLM/src/logger.hpp:118-140): snap to the largest level <= level.
int sgdlm_set_log_level(sgdlm_handle h, int level) {
  HCHECK(h);
  const int levels[] = {LOG_SYSDEBUG, LOG_DEBUG, LOG_RESULT, LOG_INFO, LOG_WARNING};
  int chosen = LOG_ERROR;
  for (int l : levels)
    if (level >= l) {
      chosen = l;
      break;
    }
  h->log_level = chosen;
  return SGDLM_OK;
}
int sgdlm_get_log_level(sgdlm_handle h, int *level) {
  HCHECK(h);
  if (!level) return SGDLM_ERR_BAD_ARG;
  *level = h->log_level;
  return SGDLM_OK;
}
const char *sgdlm_last_error(sgdlm_handle h) { return h ? h->last_error.c_str() : ""; }

int sgdlm_set_proposal(sgdlm_handle h, const sgdlm_proposal_config *cfg) {
  HCHECK(h);
  sgdlm_proposal_config c{SGDLM_PROPOSAL_PLAIN, 500, 4, 4096, 1e-3, 0.5, 20261204u};
  if (cfg) c = *cfg;
  if ((c.mode != SGDLM_PROPOSAL_PLAIN && c.mode != SGDLM_PROPOSAL_LEARNED) || c.train_steps < 0 ||
      c.iters_per_step < 0 || c.batch < 1 || !(c.lr > 0.0) ||
      !(c.ess_fraction >= 0.0 && c.ess_fraction <= 1.0))
    return h->fail(SGDLM_ERR_BAD_ARG, "invalid proposal configuration");
  cudaStreamSynchronize(h->stream);
  h->prop.release();
  h->prop.cfg = c;
  if (c.mode == SGDLM_PROPOSAL_LEARNED && h->mem_init) return proposal_ensure(h);
  return SGDLM_OK;
}

int sgdlm_get_proposal(sgdlm_handle h, sgdlm_proposal_config *cfg) {
  HCHECK(h);
  if (!cfg) return SGDLM_ERR_BAD_ARG;
  *cfg = h->prop.cfg;
  return SGDLM_OK;
}

int sgdlm_get_proposal_info(sgdlm_handle h, sgdlm_proposal_info *info) {
  HCHECK(h);
  if (!info) return SGDLM_ERR_BAD_ARG;
  *info = h->prop.info;
  return SGDLM_OK;
}

int sgdlm_proposal_sizes(sgdlm_handle h, size_t *n_params, int *n_features, int *n_outputs) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  const int F = proposal_features((int)h->P), O = proposal_outputs((int)h->P);
  if (n_params) *n_params = (size_t)mlp_layout(F, O).total;
  if (n_features) *n_features = F;
  if (n_outputs) *n_outputs = O;
  return SGDLM_OK;
}

int sgdlm_proposal_get_params(sgdlm_handle h, float *params) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!params) return h->fail(SGDLM_ERR_BAD_ARG, "null parameter array");
  int st = proposal_ensure(h);
  if (st) return st;
  if ((st = d2h(h, params, h->prop.w.ptr, h->prop.L.total * sizeof(float)))) return st;
  return sync(h);
}

int sgdlm_proposal_set_params(sgdlm_handle h, const float *params) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!params) return h->fail(SGDLM_ERR_BAD_ARG, "null parameter array");
  int st = proposal_ensure(h);
  if (st) return st;
  ProposalState &q = h->prop;
  if ((st = h2d(h, q.w.ptr, params, q.L.total * sizeof(float)))) return st;
  mlp_refresh_bf16(h->stream, q.L, q.w.ptr, q.w16.ptr);
  h->launches += 1;
  return sync(h);
}

int sgdlm_proposal_loss_and_gradient(sgdlm_handle h, size_t batch, const float *X, const float *Y,
                                     const float *mask, double *loss, float *grad) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!X || !Y || !mask || batch < 1 || batch > (1u << 24))
    return h->fail(SGDLM_ERR_BAD_ARG, "invalid batch");
  int st = proposal_ensure(h);
  if (st) return st;
  ProposalState &q = h->prop;
  const MlpLayout &L = q.L;
  const size_t B = batch;
  DevBuf<float> x, y, mk, g, z1, a1, z2, a2, out, dout, da, da2;
  DevBuf<double> l;
  CK(x.alloc(B * L.F));
  CK(y.alloc(B * L.O));
  CK(mk.alloc(B * L.O));
  CK(g.alloc(L.total));
  for (auto *b : {&z1, &a1, &z2, &a2, &da, &da2}) CK(b->alloc(B * L.H));
  CK(out.alloc(B * L.O));
  CK(dout.alloc(B * L.O));
  CK(l.alloc(1));
  if ((st = h2d(h, x.ptr, X, B * L.F * sizeof(float)))) return st;
  if ((st = h2d(h, y.ptr, Y, B * L.O * sizeof(float)))) return st;
  if ((st = h2d(h, mk.ptr, mask, B * L.O * sizeof(float)))) return st;
  const MlpActs a{z1.ptr, a1.ptr, z2.ptr, a2.ptr, out.ptr, dout.ptr, da.ptr, da2.ptr};
  mlp_forward(h->stream, L, (int)B, x.ptr, q.w.ptr, q.w16.ptr, a);
  mlp_loss_backward(h->stream, L, (int)B, x.ptr, y.ptr, mk.ptr, q.w16.ptr, a, g.ptr, l.ptr);
  h->launches += 13;
  if (loss && (st = d2h(h, loss, l.ptr, sizeof(double)))) return st;
  if (grad && (st = d2h(h, grad, g.ptr, L.total * sizeof(float)))) return st;
  return sync(h);
}

int sgdlm_get_proposal_state(sgdlm_handle h, double *m_q, double *C_q, double *n_q, double *s_q,
                             double *log_weights) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  ProposalState &q = h->prop;
  if (!q.mq.ptr || !q.logw.ptr)
    return h->fail(SGDLM_ERR_WRONG_STATE, "no learned proposal has been drawn from");
  const size_t m = h->m, P = h->P;
  int st;
  std::vector<double> U(P * P * m);
  if (m_q && (st = d2h(h, m_q, q.mq.ptr, P * m * sizeof(double)))) return st;
  if (n_q && (st = d2h(h, n_q, q.nq.ptr, m * sizeof(double)))) return st;
  if (s_q && (st = d2h(h, s_q, q.sq.ptr, m * sizeof(double)))) return st;
  if (C_q && (st = d2h(h, U.data(), q.Uq64.ptr, U.size() * sizeof(double)))) return st;
  if (log_weights && (st = d2h(h, log_weights, q.logw.ptr, h->nsim * sizeof(double)))) return st;
  if ((st = sync(h))) return st;
  if (C_q)  // C~ = U~' U~ per series
    for (size_t j = 0; j < m; ++j)
      for (size_t c = 0; c < P; ++c)
        for (size_t r = 0; r < P; ++r) {
          double acc = 0.0;
          for (size_t l = 0; l < P; ++l) acc += U[j * P * P + l + P * r] * U[j * P * P + l + P * c];
          C_q[j * P * P + r + P * c] = acc;
        }
  return SGDLM_OK;
}

int sgdlm_filter_step_device(sgdlm_handle h, const double *d_y, const double *d_F,
                             const double *d_x, double ess_threshold, double *d_forecast,
                             double *d_is_weights, double *d_step_stats) {
  HCHECK(h);
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
  if (!h->check_prior(true)) return SGDLM_ERR_WRONG_STATE;
  if (!d_y || !d_F) return h->fail(SGDLM_ERR_BAD_ARG, "null input");
  int st = h->precision == SGDLM_PRECISION_FP64
               ? filter_step<double>(h, d_y, d_F, d_x, ess_threshold, d_forecast, d_is_weights,
                                     d_step_stats)
               : filter_step<float>(h, d_y, d_F, d_x, ess_threshold, d_forecast, d_is_weights,
                                    d_step_stats);
  if (st) return st;
  h->is_prior = true;
  return SGDLM_OK;
}

int sgdlm_set_lu_options(sgdlm_handle h, int allow_tensor_cores, int max_ctas) {
  HCHECK(h);
  if (max_ctas < 0) return h->fail(SGDLM_ERR_BAD_ARG, "max_ctas must not be negative");
  h->lu_opt.allow_tc = allow_tensor_cores ? 1 : 0;
  h->lu_opt.max_grid = max_ctas;
  if (!h->mem_init) return SGDLM_OK;
  cudaStreamSynchronize(h->stream);
  return replan_sim(h);
}

int sgdlm_set_warp_lu(sgdlm_handle h, int enable) {
  HCHECK(h);
  h->lu_opt.allow_warp = enable ? 1 : 0;
  return SGDLM_OK;
}
int sgdlm_get_warp_lu(sgdlm_handle h, int *enabled, int *in_use) {
  HCHECK(h);
  if (enabled) *enabled = h->lu_opt.allow_warp;
  if (in_use) *in_use = warp_lu(h) ? 1 : 0;
  return SGDLM_OK;
}

int sgdlm_set_forecast_solver(sgdlm_handle h, int iterative) {
  HCHECK(h);
  h->forecast_iterative = iterative ? 1 : 0;
  return SGDLM_OK;
}

int sgdlm_get_lu_options(sgdlm_handle h, int *allow_tensor_cores, int *max_ctas) {
  HCHECK(h);
  if (allow_tensor_cores) *allow_tensor_cores = h->lu_opt.allow_tc;
  if (max_ctas) *max_ctas = h->lu_opt.max_grid;
  return SGDLM_OK;
}

}  // extern "C"

namespace {
template <typename T> int tune_lu(sgdlm_engine *h, sgdlm_lu_tuning *out) {
  const int levels0 = h->elim_levels;
  const LuOptions opt0 = h->lu_opt;
  CK(cudaMemsetAsync(h->draw_flags.ptr, 0, h->nsim * sizeof(int), h->stream));
  sample_draws<T>(h, h->m_t.ptr, h->C_t.ptr, h->n_t.ptr, h->s_t.ptr, h->key((uint32_t)h->epoch));
  const int cand_levels[4] = {0, 2, 4, 6};
  double best = 1e300;
  int best_l = levels0, best_tc = opt0.allow_tc;
  for (int q = 0; q < 8; ++q) out->ms_candidates[q] = -1.0;
  for (int li = 0; li < 4; ++li)
    for (int tc = 1; tc >= 0; --tc) {
      if (tc == 0 && std::is_same<T, double>::value) continue;  // FP64 has no tensor-core path
      h->lu_opt.allow_tc = tc;
      int st = sgdlm_set_elimination_levels(h, cand_levels[li]);
      if (st) return st;
      if (tc == 1 && !h->plan.tc && !std::is_same<T, double>::value) {
        // no tensor-core plan for this core: the FFMA candidate covers it
        continue;
      }
      std::vector<float> ms;
      for (int rep = 0; rep < 4; ++rep) {
        CK(cudaEventRecord(h->ev[5], h->stream));
        if ((st = lu_draws<T>(h, nullptr, h->key((uint32_t)h->epoch), nullptr))) return st;
        CK(cudaEventRecord(h->ev[6], h->stream));
        if ((st = sync(h))) return st;
        if (rep > 0) ms.push_back(elapsed(h->ev[5], h->ev[6]));
      }
      std::sort(ms.begin(), ms.end());
      const double t = ms[ms.size() / 2];
      out->ms_candidates[2 * li + (1 - tc)] = t;
      if (t < best) {
        best = t;
        best_l = cand_levels[li];
        best_tc = h->plan.tc;
      }
    }
  h->lu_opt.allow_tc = best_tc;
  int st = sgdlm_set_elimination_levels(h, best_l);
  if (st) return st;
  out->levels = h->eplan.nlev;
  out->tensor_cores = h->plan.tc;
  out->core_n = h->eplan.core_n;
  out->ms = best;
  return SGDLM_OK;
}
}  // namespace

extern "C" {

int sgdlm_tune_lu(sgdlm_handle h, sgdlm_lu_tuning *out) {
  HCHECK(h);
  if (!out) return SGDLM_ERR_BAD_ARG;
  if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
  if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
  *out = sgdlm_lu_tuning{};
  return h->precision == SGDLM_PRECISION_FP64 ? tune_lu<double>(h, out) : tune_lu<float>(h, out);
}

}  // extern "C"

struct sgdlm_batch {
  std::vector<sgdlm_engine *> eng;
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<uint64_t> launches_per_step;
  // the recording's arguments (re-recorded by the autotuner)
  std::vector<const double *> y, F, x;
  std::vector<double *> fc, w, st;
  double ess = 0.0;
  bool recorded = false;
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    recorded = false;
  }
};

namespace {

// Captures every engine's fused step into b->graph: the origin stream forks to
// the engines' streams, each runs its step, and they join back.
int batch_capture(sgdlm_batch *b) {
  b->drop_graph();
  const size_t k = b->eng.size();
  cudaError_t e = cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return SGDLM_ERR_DEVICE;
  int status = SGDLM_OK;
  e = cudaEventRecord(b->fork, b->origin);
  for (size_t i = 0; i < k && e == cudaSuccess && status == SGDLM_OK; ++i) {
    sgdlm_engine *h = b->eng[i];
    e = cudaStreamWaitEvent(h->stream, b->fork, 0);
    if (e != cudaSuccess) break;
    const uint64_t l0 = h->launches, ep0 = h->epoch;
    status = h->precision == SGDLM_PRECISION_FP64
                 ? filter_step<double>(h, b->y[i], b->F[i], b->x[i], b->ess, b->fc[i], b->w[i],
                                       b->st[i])
                 : filter_step<float>(h, b->y[i], b->F[i], b->x[i], b->ess, b->fc[i], b->w[i],
                                      b->st[i]);
    b->launches_per_step[i] = h->launches - l0;
    h->launches = l0;   // counted when the graph runs
    h->epoch = ep0;     // advanced when the graph runs
    if (status == SGDLM_OK) e = cudaEventRecord(b->join[i], h->stream);
    if (e == cudaSuccess && status == SGDLM_OK) e = cudaStreamWaitEvent(b->origin, b->join[i], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(b->origin, &g);
  if (status != SGDLM_OK || e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    (void)cudaGetLastError();
    return status != SGDLM_OK ? status : SGDLM_ERR_DEVICE;
  }
  b->graph = g;
  if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) {
    b->drop_graph();
    return SGDLM_ERR_DEVICE;
  }
  b->recorded = true;
  return SGDLM_OK;
}

int batch_launch(sgdlm_batch *b) {
  for (size_t i = 0; i < b->eng.size(); ++i) {
    if (cudaEventRecord(b->join[i], b->eng[i]->stream) != cudaSuccess ||
        cudaStreamWaitEvent(b->origin, b->join[i], 0) != cudaSuccess)
      return SGDLM_ERR_DEVICE;
  }
  if (cudaGraphLaunch(b->exec, b->origin) != cudaSuccess) return SGDLM_ERR_DEVICE;
  if (cudaEventRecord(b->done, b->origin) != cudaSuccess) return SGDLM_ERR_DEVICE;
  for (size_t i = 0; i < b->eng.size(); ++i) {
    sgdlm_engine *h = b->eng[i];
    if (cudaStreamWaitEvent(h->stream, b->done, 0) != cudaSuccess) return SGDLM_ERR_DEVICE;
    h->epoch += 2;
    h->launches += b->launches_per_step[i];
    h->is_prior = true;
  }
  return SGDLM_OK;
}

// Parameters and RNG states of every engine, for the autotuner's trial steps.
struct BatchSnapshot {
  std::vector<std::vector<double>> m, C, n, s;
  std::vector<uint64_t> seed, epoch;
};
int batch_save(sgdlm_batch *b, BatchSnapshot &snap) {
  const size_t k = b->eng.size();
  snap.m.resize(k); snap.C.resize(k); snap.n.resize(k); snap.s.resize(k);
  snap.seed.resize(k); snap.epoch.resize(k);
  for (size_t i = 0; i < k; ++i) {
    sgdlm_engine *h = b->eng[i];
    snap.m[i].resize(h->P * h->m);
    snap.C[i].resize(h->P * h->P * h->m);
    snap.n[i].resize(h->m);
    snap.s[i].resize(h->m);
    int st = sgdlm_get_parameters(h, snap.m[i].data(), snap.C[i].data(), snap.n[i].data(),
                                  snap.s[i].data());
    if (st) return st;
    snap.seed[i] = h->seed;
    snap.epoch[i] = h->epoch;
  }
  return SGDLM_OK;
}
int batch_restore(sgdlm_batch *b, const BatchSnapshot &snap) {
  for (size_t i = 0; i < b->eng.size(); ++i) {
    sgdlm_engine *h = b->eng[i];
    int st = sgdlm_set_parameters(h, snap.m[i].data(), snap.C[i].data(), snap.n[i].data(),
                                  snap.s[i].data());
    if (!st) st = sgdlm_set_is_prior(h, 1);
    if (!st) st = sgdlm_set_rng_state(h, snap.seed[i], snap.epoch[i]);
    if (st) return st;
  }
  return SGDLM_OK;
}

}  // namespace

extern "C" {

int sgdlm_batch_create(const sgdlm_handle *handles, size_t count, sgdlm_batch_handle *out) {
  if (!out || !handles || count < 1) return SGDLM_ERR_BAD_ARG;
  *out = nullptr;
  std::unique_ptr<sgdlm_batch> b(new sgdlm_batch());
  for (size_t i = 0; i < count; ++i) {
    if (!handles[i]) return SGDLM_ERR_BAD_ARG;
    if (handles[i]->device != handles[0]->device)
      return handles[i]->fail(SGDLM_ERR_BAD_ARG, "the engines of a batch share one device");
    for (size_t q = 0; q < i; ++q)
      if (handles[q] == handles[i])
        return handles[i]->fail(SGDLM_ERR_BAD_ARG, "an engine appears twice in the batch");
    b->eng.push_back(handles[i]);
  }
  cudaSetDevice(handles[0]->device);
  if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess)
    return SGDLM_ERR_DEVICE;
  b->join.assign(count, nullptr);
  for (auto &e : b->join)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return SGDLM_ERR_DEVICE;
  b->launches_per_step.assign(count, 0);
  *out = b.release();
  return SGDLM_OK;
}

int sgdlm_batch_destroy(sgdlm_batch_handle b) {
  if (!b) return SGDLM_OK;
  if (b->origin) cudaStreamSynchronize(b->origin);
  b->drop_graph();
  for (auto e : b->join)
    if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->done) cudaEventDestroy(b->done);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
  return SGDLM_OK;
}

int sgdlm_batch_record(sgdlm_batch_handle b, const double *const *d_y, const double *const *d_F,
                       const double *const *d_x, double ess_threshold,
                       double *const *d_forecast, double *const *d_is_weights,
                       double *const *d_step_stats) {
  if (!b || !d_y || !d_F) return SGDLM_ERR_BAD_ARG;
  const size_t k = b->eng.size();
  for (size_t i = 0; i < k; ++i) {
    sgdlm_engine *h = b->eng[i];
    cudaSetDevice(h->device);
    if (!h->check_initialized()) return SGDLM_ERR_NOT_INIT;
    if (!h->check_sim_initialized()) return SGDLM_ERR_SIM_NOT_INIT;
    if (!h->check_prior(true)) return SGDLM_ERR_WRONG_STATE;
    if (!d_y[i] || !d_F[i]) return h->fail(SGDLM_ERR_BAD_ARG, "null input");
  }
  b->y.assign(d_y, d_y + k);
  b->F.assign(d_F, d_F + k);
  b->x.assign(k, nullptr);
  b->fc.assign(k, nullptr);
  b->w.assign(k, nullptr);
  b->st.assign(k, nullptr);
  for (size_t i = 0; i < k; ++i) {
    if (d_x) b->x[i] = d_x[i];
    if (d_forecast) b->fc[i] = d_forecast[i];
    if (d_is_weights) b->w[i] = d_is_weights[i];
    if (d_step_stats) b->st[i] = d_step_stats[i];
  }
  b->ess = ess_threshold;
  for (auto *h : b->eng) cudaStreamSynchronize(h->stream);
  return batch_capture(b);
}

int sgdlm_batch_step(sgdlm_batch_handle b) {
  if (!b) return SGDLM_ERR_BAD_ARG;
  if (!b->recorded) return SGDLM_ERR_WRONG_STATE;
  cudaSetDevice(b->eng[0]->device);
  return batch_launch(b);
}

}  // extern "C"

namespace {

// Time of one recorded batch step (mean over `replays` replays after one
// warm-up), with the engines' states restored afterwards.
int batch_time(sgdlm_batch *b, int replays, const BatchSnapshot &snap, double *ms_out) {
  int st = batch_capture(b);
  if (!st) st = batch_launch(b);  // warm-up
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  if (!st) {
    cudaEventRecord(e0, b->origin);
    for (int r = 0; r < replays && !st; ++r) st = batch_launch(b);
    cudaEventRecord(e1, b->origin);
    cudaEventSynchronize(e1);
  }
  for (auto *h : b->eng) cudaStreamSynchronize(h->stream);
  float ms = 0.f;
  if (!st) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  *ms_out = ms / replays;
  return batch_restore(b, snap);
}

int set_plans(sgdlm_batch *b, const std::vector<int> &levels, const std::vector<int> &tc, int c) {
  for (size_t i = 0; i < b->eng.size(); ++i) {
    sgdlm_engine *h = b->eng[i];
    h->lu_opt.allow_tc = tc[i];
    int st = sgdlm_set_elimination_levels(h, levels[i]);
    if (!st) st = sgdlm_set_lu_options(h, tc[i], c == 1 ? 0 : 2 * h->num_sms / c);
    if (st) return st;
  }
  return SGDLM_OK;
}

}  // namespace

extern "C" {

int sgdlm_batch_autotune(sgdlm_batch_handle b, int replays, sgdlm_batch_tuning *out) {
  if (!b || !out || replays < 1) return SGDLM_ERR_BAD_ARG;
  if (!b->recorded) return SGDLM_ERR_WRONG_STATE;
  cudaSetDevice(b->eng[0]->device);
  *out = sgdlm_batch_tuning{};
  for (auto *h : b->eng) cudaStreamSynchronize(h->stream);
  const size_t k = b->eng.size();
  BatchSnapshot snap;
  int st = batch_save(b, snap);
  if (st) return st;
  std::vector<int> lev0(k), tc0(k), lev1(k), tc1(k);
  for (size_t i = 0; i < k; ++i) {
    lev0[i] = b->eng[i]->elim_levels;
    tc0[i] = b->eng[i]->lu_opt.allow_tc;
  }
  double base = 0.0;
  if ((st = set_plans(b, lev0, tc0, 1)) || (st = batch_time(b, replays, snap, &base))) return st;
  // (1) per m bucket (m rounded up to 32): tune the LU on one engine, apply to the rest
  std::vector<int> bucket_done;
  lev1 = lev0;
  tc1 = tc0;
  for (size_t i = 0; i < k; ++i) {
    sgdlm_engine *h = b->eng[i];
    const int bucket = (int)((h->m + 31) / 32);
    bool seen = false;
    for (int q : bucket_done) seen |= (q == bucket);
    if (seen) continue;
    bucket_done.push_back(bucket);
    sgdlm_lu_tuning t{};
    if ((st = sgdlm_tune_lu(h, &t))) return st;
    for (size_t j = 0; j < k; ++j)
      if ((int)((b->eng[j]->m + 31) / 32) == bucket) {
        lev1[j] = h->elim_levels;
        tc1[j] = h->lu_opt.allow_tc;
      }
  }
  out->buckets = (int)bucket_done.size();
  if ((st = batch_restore(b, snap))) return st;  // the LU tuner drew with the current state
  // keep the tuned plans only if the whole batch step is faster with them
  double tuned = 0.0;
  if ((st = set_plans(b, lev1, tc1, 1)) || (st = batch_time(b, replays, snap, &tuned))) return st;
  const bool keep = tuned < base;
  const std::vector<int> &lev = keep ? lev1 : lev0, &tc = keep ? tc1 : tc0;
  // (2) concurrency: each engine's LU grid capped at 2 x SMs / c
  const int cs[4] = {1, 2, 4, 8};
  double best = keep ? tuned : base;
  int best_c = 1;
  out->ms_candidates[0] = best;
  for (int ci = 1; ci < 4; ++ci) {
    double ms = 0.0;
    if ((st = set_plans(b, lev, tc, cs[ci])) || (st = batch_time(b, replays, snap, &ms))) return st;
    out->ms_candidates[ci] = ms;
    if (ms < best) {
      best = ms;
      best_c = cs[ci];
    }
  }
  if ((st = set_plans(b, lev, tc, best_c))) return st;
  if ((st = batch_restore(b, snap))) return st;
  out->concurrency = best_c;
  out->ms_per_step = best;
  out->lu_plans_kept = keep ? 1 : 0;
  out->ms_untuned = base;
  return batch_capture(b);
}

int sgdlm_get_stream(sgdlm_handle h, void **stream) {
  HCHECK(h);
  if (!stream) return SGDLM_ERR_BAD_ARG;
  *stream = (void *)h->stream;
  return SGDLM_OK;
}
int sgdlm_synchronize(sgdlm_handle h) {
  HCHECK(h);
  return sync(h);
}
int sgdlm_get_launch_count(sgdlm_handle h, uint64_t *count) {
  HCHECK(h);
  if (!count) return SGDLM_ERR_BAD_ARG;
  *count = h->launches;
  return SGDLM_OK;
}

}  // extern "C"

// C-ABI entry points (include/glagpu.h): plans, workspace, launch sequence.
//
// A plan fixes the matrix orders of a batch, so all host-side planning
// (offsets, size buckets, chase lane order, workspace carving) happens once
// in gla_plan_create and gla_plan_execute only enqueues kernels.
//
// Launch sequence for jobz 'V' (eigen!):
//   k_tridiag  per size bucket   symtri! + Array(Q)      (one CTA per matrix)
//   repeat per pass (normally one):
//     k_chase                     eigQL!/eigQR! scalars   (one lane per matrix)
//     k_apply  per size bucket    rotations on Q, sorteig!
//   [F32_REFINED] refinement kernels (refine.cu)
// jobz 'N' (eigvals!): k_tridiag (no Q), k_chase<PWK>, k_sort_values.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <map>
#include <mutex>
#include <new>
#include <numeric>
#include <tuple>
#include <vector>

#include "../../include/glagpu.h"
#include "gla_launch.h"
#include "gla_adjoint.h"
#include "gla_large.h"
#include "gla_refine.h"

using namespace gla;

namespace gla {
cudaError_t tridiag_kernels_init();
cudaError_t chase_kernels_init();
cudaError_t apply_kernels_init();
void release_eigenq_cache();
void release_complex_cache();
void release_quaternion_cache();
}  // namespace gla

namespace {

constexpr int kRotPerN2 = 2;    // rotation-log capacity per pass, in units of n^2
constexpr int kHdrPerN = 3;     // header-log capacity per pass, in units of n
constexpr int kAsyncPasses = 2;     // chase passes enqueued without a host check
constexpr int kGraphPasses = 4;     // chase passes of a capture-safe (GLA_FLAG_GRAPH) execute
constexpr int kMaxBuckets = 8;      // size buckets of width 16 over (0, 128]
constexpr int kMaxChunks = 4;       // host-execute pipeline: chunks of the batch

#define GLA_CUDA(x)                                  \
  do {                                               \
    cudaError_t e_ = (x);                            \
    if (e_ != cudaSuccess) return -1000 - (int)e_;   \
  } while (0)

// A lazily allocated cache buffer: *slot is set only on success, so a failed
// allocation leaves it empty and a later call retries.
template <class P>
cudaError_t cache_alloc(P** slot, size_t bytes) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e == cudaSuccess) *slot = static_cast<P*>(q);
  return e;
}

struct Bucket {
  int nmax;   // largest order in the bucket
  int nt;     // threads per CTA (apply)
  int nt_tri; // threads per CTA (tridiagonalisation)
  int lpw = 0;  // chase: matrices per warp (0: the launcher's default)
  int start;  // first index into perm_bucket (orders descending inside the bucket)
  int count;
  cudaStream_t stream = nullptr;  // the bucket's pipeline runs on its own stream
  cudaEvent_t join = nullptr;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

std::once_flag g_init_flag;
cudaError_t g_init_err = cudaSuccess;

cudaError_t ensure_init() {
  std::call_once(g_init_flag, [] {
    cudaError_t e;
    if ((e = tridiag_kernels_init()) != cudaSuccess) g_init_err = e;
    if ((e = chase_kernels_init()) != cudaSuccess) g_init_err = e;
    if ((e = apply_kernels_init()) != cudaSuccess) g_init_err = e;
    if ((e = refine_kernels_init()) != cudaSuccess) g_init_err = e;
    if ((e = adjoint_kernels_init()) != cudaSuccess) g_init_err = e;
  });
  return g_init_err;
}

}  // namespace

struct gla_plan_s {
  int prec = GLA_PREC_F64;
  char jobz = 'V', uplo = 'L';
  int algo = kAlgoQL;
  int64_t batch = 0;
  double tol = 0;
  std::vector<int64_t> n;
  int64_t a_elems = 0, w_elems = 0;
  int nwork = 0;  // matrices with n >= 1
  std::vector<Bucket> buckets;
  int nmax = 0;
  // device workspace
  char* ws = nullptr;
  size_t ws_bytes = 0;
  SmallDesc* d_desc = nullptr;
  int* d_perm_bucket = nullptr;
  void* d_d = nullptr;
  void* d_e = nullptr;
  void* d_rot = nullptr;
  unsigned* d_hdr = nullptr;
  ChaseState* d_cst = nullptr;
  int* d_pending = nullptr;
  unsigned long long* d_stats = nullptr;
  int* d_scale = nullptr;
  void* d_x32 = nullptr;  // FP32 eigenvectors (refined runs, or 'N' refined)
  void* d_w32 = nullptr;
  RefineWork rw;          // refinement scratch
  bool refine_tc = true;  // the refinement's double-float products on the tensor cores
  void* d_vtmp = nullptr; // V target when the caller passes none
  void* d_qtmp = nullptr; // stein: Q of every matrix (float arena) while its tridiagonal is solved
  // host-execute buffers
  void* h_A = nullptr;
  void* h_w = nullptr;
  void* h_V = nullptr;
  int* h_info = nullptr;
  int* pin_pending = nullptr;
  df64* d_adj = nullptr;  // adjoint workspace (allocated by the first gla_plan_adjoint)
  double* h_adj = nullptr;  // device staging of gla_plan_adjoint_host
  LargeAdjoint* adj_large = nullptr;  // adjoint context of the orders above GLA_MAX_SMALL_N
  // orders above GLA_MAX_SMALL_N: solved one at a time by the large path
  std::vector<int> large_idx;           // batch indices, in batch order
  std::map<int, LargeCtx*> large_ctx;   // one context per distinct order
  std::map<int, RefineLarge*> large_ref;  // F32_REFINED: refinement per distinct order
  int large_iters = 0;                  // refinement iterations of the last execute (max)
  double large_refine_n3 = 0;           // sum over large matrices of iterations * n^3
  float large_refine_ms = 0.f;          // host-timed refinement of the last execute
  int* h_large_info = nullptr;          // pinned, one word per large matrix
  cudaStream_t last_stream = nullptr;
  int last_passes = 0;
  cudaEvent_t fork = nullptr;
  // phase timing (GLA_FLAG_TIMING): begin/end events per bucket and phase;
  // a phase's time is the sum over buckets of its kernels' stream time
  bool timing = false;
  bool graph = false;  // capture-safe execute (no host synchronisation)
  bool stein = false;  // FP32 stage by bisection + twisted factorisation (small_stein.cuh)
  // F32_REFINED with that solver: the orders <= 128 are solved and refined by
  // one persistent launch (k_solve_refine) instead of per-bucket pipelines
  bool persistent = false;
  int persist_grid = 0;
  int* d_next = nullptr;  // its work counters (one per chunk of the host-execute pipeline)
  // gla_plan_execute_host of a persistent plan on pinned host buffers: the
  // batch as contiguous runs of matrices ("chunks"), so that the copy of
  // chunk c + 1's A and of chunk c - 1's w and V overlap the solve of chunk
  // c; consecutive chunks are solved on two alternating streams, so that the
  // next chunk's CTAs take the SMs the last matrices of a chunk leave idle
  int nchunks = 0;                        // 0: no pipeline
  int64_t chunk_b[kMaxChunks + 1] = {};   // chunk c: batch indices chunk_b[c] .. chunk_b[c + 1] - 1
  int64_t chunk_a[kMaxChunks + 1] = {};   // its A / V elements from chunk_a[c]
  int64_t chunk_w[kMaxChunks + 1] = {};   // its w elements from chunk_w[c]
  int chunk_start[kMaxChunks + 1] = {};   // its work items: d_chunk_order[chunk_start[c] ..]
  int* d_chunk_order = nullptr;           // each chunk's work items, orders descending
  cudaStream_t s_in = nullptr, s_out = nullptr, s_odd = nullptr;  // s_odd: the odd chunks' solves
  cudaEvent_t ev_in[kMaxChunks] = {}, ev_solved[kMaxChunks] = {}, ev_out = nullptr;
  ChaseState* h_cst = nullptr;            // pinned: the chase states after the persistent launches
  bool last_pipelined = false;            // the last gla_plan_execute_host used the pipeline
  cudaEvent_t tev[kMaxBuckets][GLA_NUM_PHASES][2] = {};
  bool tused[kMaxBuckets][GLA_NUM_PHASES] = {};
  void mark(int b, int phase, int end, cudaStream_t st) {
    if (!timing || b >= kMaxBuckets) return;
    cudaEventRecord(tev[b][phase][end], st);
    if (end) tused[b][phase] = true;
  }
  int tcode() const { return prec == GLA_PREC_F64 ? kF64 : (prec == GLA_PREC_F32 ? kF32 : kF32FromF64); }
  size_t elem() const { return prec == GLA_PREC_F64 ? 8 : 4; }          // working element size
  size_t io_elem() const { return prec == GLA_PREC_F32 ? 4 : 8; }       // caller element size
};

namespace {
int autotune_plan(gla_plan_t p, int base_flags);
}

extern "C" {

int gla_version(void) { return GLA_VERSION; }

const char* gla_status_string(int status) {
  if (status == 0) return "success";
  if (status > 0) return "some matrices did not converge or held non-finite values (see info)";
  if (status == GLA_ERR_STATIC_TOO_LARGE) return "order exceeds GLA_STATIC_MAX_N (128) for gla_dsyev_static";
  if (status == GLA_ERR_UNSUPPORTED) return "operation not supported for this plan (see glagpu.h)";
  if (status <= -1000) return cudaGetErrorString((cudaError_t)(-1000 - status));
  switch (status) {
    case -1: return "invalid argument 1";
    case -2: return "invalid argument 2";
    case -3: return "invalid argument 3";
    case -4: return "invalid argument 4";
    case -5: return "invalid argument 5";
    case -6: return "invalid argument 6";
    case -7: return "invalid argument 7";
    case -8: return "invalid argument 8";
    case -9: return "invalid argument 9";
    case -10: return "invalid argument 10";
    default: return "invalid argument";
  }
}

int gla_plan_create(gla_plan_t* plan_out, int precision, char jobz, char uplo, int64_t batch, const int64_t* n,
                    double tol, int flags) {
  if (!plan_out) return -1;
  *plan_out = nullptr;
  if (precision != GLA_PREC_F64 && precision != GLA_PREC_F32 && precision != GLA_PREC_F32_REFINED) return -2;
  if (jobz != 'V' && jobz != 'N') return -3;
  if (uplo != 'L' && uplo != 'U') return -4;
  if (batch < 0) return -5;
  if (batch > 0 && !n) return -6;
  for (int64_t b = 0; b < batch; b++)
    if (n[b] < 0 || n[b] > GLA_MAX_N) return -6;
  if (!(tol == tol)) return -7;
  {
    bool any_large = false;
    for (int64_t b = 0; b < batch; b++) any_large |= n[b] > GLA_MAX_SMALL_N;
    // large orders: no capture-safe mode (their solves synchronise)
    if (any_large && (flags & GLA_FLAG_GRAPH)) return -8;
  }
  if ((flags & ~(3 | GLA_FLAG_SMALL_LOG | GLA_FLAG_TIMING | GLA_FLAG_GRAPH | GLA_FLAG_AUTOTUNE |
                 GLA_FLAG_REFINE_QL | GLA_FLAG_F32_BISECT | GLA_FLAG_REFINE_SIMT)) != 0 ||
      (flags & 3) > GLA_ALG_QR)
    return -8;
  GLA_CUDA(ensure_init());

  gla_plan_s* p = new (std::nothrow) gla_plan_s();
  if (!p) return -1;
  p->prec = precision;
  p->jobz = jobz;
  p->uplo = uplo;
  p->algo = (flags & 3) == GLA_ALG_QR ? kAlgoQR : kAlgoQL;
  p->batch = batch;
  p->tol = tol > 0 ? tol : (precision == GLA_PREC_F64 ? kTolF64 : kTolF32);
  p->timing = (flags & GLA_FLAG_TIMING) != 0;
  p->graph = (flags & GLA_FLAG_GRAPH) != 0;
  p->stein = (precision == GLA_PREC_F32_REFINED && !(flags & GLA_FLAG_REFINE_QL)) ||
             (precision == GLA_PREC_F32 && (flags & GLA_FLAG_F32_BISECT));
  p->persistent = p->stein && precision == GLA_PREC_F32_REFINED;
  p->refine_tc = !(flags & GLA_FLAG_REFINE_SIMT);
  p->n.assign(n, n + batch);

  // ---- descriptors and offsets
  std::vector<SmallDesc> desc(batch);
  int64_t aoff = 0, woff = 0, roff = 0, hoff = 0;
  for (int64_t b = 0; b < batch; b++) {
    const int nb = (int)n[b];
    SmallDesc& d = desc[b];
    d.n = nb;
    d.pad = 0;
    d.a_off = aoff;
    d.w_off = woff;
    d.rot_off = roff;
    d.hdr_off = hoff;
    const bool large = nb > GLA_MAX_SMALL_N;
    d.rot_cap = large ? 0 : (flags & GLA_FLAG_SMALL_LOG) ? nb * nb / 8 + nb : kRotPerN2 * nb * nb + 4;
    d.hdr_cap = large ? 0 : (flags & GLA_FLAG_SMALL_LOG) ? nb / 4 + 2 : kHdrPerN * nb + 4;
    aoff += (int64_t)nb * nb;
    woff += nb;
    roff += d.rot_cap;
    hoff += d.hdr_cap;
    if (large)
      p->large_idx.push_back((int)b);
    else
      p->nmax = std::max(p->nmax, nb);
  }
  p->a_elems = aoff;
  p->w_elems = woff;

  // ---- size buckets (descending order inside each bucket), chase order
  std::vector<int> idx;
  for (int64_t b = 0; b < batch; b++)
    if (n[b] >= 1 && n[b] <= GLA_MAX_SMALL_N) idx.push_back((int)b);
  p->nwork = (int)idx.size();
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return n[a] > n[b]; });
  std::vector<int> perm_bucket;
  for (int ei = kMaxBuckets - 1; ei >= 0; ei--) {  // largest orders first: longest pipelines start first
    const int lo = 16 * ei, hi = 16 * (ei + 1);
    Bucket bk;
    bk.nmax = 0;
    bk.start = (int)perm_bucket.size();
    bk.count = 0;
    for (int b : idx) {
      if (n[b] > lo && n[b] <= hi) {
        perm_bucket.push_back(b);
        bk.count++;
        bk.nmax = std::max(bk.nmax, (int)n[b]);
      }
    }
    bk.nt = std::max(32, (bk.nmax + 31) / 32 * 32);
    // FP32 reductions are latency bound: two threads per row halve the
    // per-thread loops of the tridiagonalisation (FP64 keeps one: its cost
    // is the FP64 pipe, not latency)
    bk.nt_tri = precision == GLA_PREC_F64 ? bk.nt : std::min(256, 2 * bk.nt);
    if (bk.count) p->buckets.push_back(bk);
  }

  // ---- workspace carve-up
  const size_t el = p->elem();
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + std::max<size_t>(bytes, 1), 256);
    return o;
  };
  const size_t o_desc = carve(sizeof(SmallDesc) * batch);
  const size_t o_pb = carve(sizeof(int) * perm_bucket.size());
  const size_t o_d = carve(el * woff);
  const size_t o_e = carve(el * woff);
  const bool wantvec = jobz == 'V' || precision == GLA_PREC_F32_REFINED;
  const size_t o_rot = carve(wantvec ? 2 * el * roff : 0);
  const size_t o_hdr = carve(wantvec ? sizeof(unsigned) * hoff : 0);
  const size_t o_cst = carve(sizeof(ChaseState) * batch);
  const size_t o_pend = carve(sizeof(int) * kMaxBuckets);
  const size_t o_stats = carve(sizeof(unsigned long long) * 4);
  const size_t o_scale = carve(sizeof(int) * batch);
  const bool refined = precision == GLA_PREC_F32_REFINED;
  const size_t o_x32 = carve(refined ? 4 * aoff : 0);
  const size_t o_w32 = carve(refined ? 4 * woff : 0);
  const size_t o_vtmp = carve((jobz == 'N' && refined) ? 8 * aoff : 0);
  const size_t o_qtmp = carve(p->stein ? 4 * aoff : 0);
  const size_t o_next = carve(sizeof(int) * kMaxChunks);
  size_t refine_bytes = refined ? refine_workspace_bytes(aoff, woff, batch) : 0;
  const size_t o_ref = carve(refine_bytes);
  cudaError_t err = cudaSuccess;
  if (p->persistent) {  // two CTAs per SM (registers and shared memory allow two)
    int dev = 0, nsm = 0;
    err = cudaGetDevice(&dev);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (err != cudaSuccess) {
      delete p;
      return -1000 - (int)err;
    }
    p->persist_grid = std::max(1, std::min(2 * nsm, p->nwork));
  }
  // host-execute pipeline: one chunk per matrix of every persistent CTA
  // (two chunks at least, kMaxChunks at most), split at equal A bytes
  std::vector<int> chunk_order;
  if (p->persistent && p->large_idx.empty() && !p->graph && !p->timing) {
    const int nc = std::min(kMaxChunks, p->nwork / std::max(1, p->persist_grid));
    if (nc >= 2) {
      p->nchunks = nc;
      int64_t b = 0, a = 0, wo = 0;
      for (int c = 1; c <= nc; c++) {
        const int64_t target = aoff * c / nc;
        while (b < batch && (c == nc || a < target)) {
          a += n[b] * n[b];
          wo += n[b];
          b++;
        }
        p->chunk_b[c] = b;
        p->chunk_a[c] = a;
        p->chunk_w[c] = wo;
      }
      for (int c = 0; c < nc; c++) {
        p->chunk_start[c] = (int)chunk_order.size();
        for (int64_t i = p->chunk_b[c]; i < p->chunk_b[c + 1]; i++)
          if (n[i] >= 1) chunk_order.push_back((int)i);
        std::stable_sort(chunk_order.begin() + p->chunk_start[c], chunk_order.end(),
                         [&](int x, int y) { return n[x] > n[y]; });
      }
      p->chunk_start[nc] = (int)chunk_order.size();
    }
  }
  const size_t o_corder = carve(sizeof(int) * chunk_order.size());
  // the tensor-core products' slice scratch, one per persistent CTA (orders
  // above 32 only); a second set for the pipeline's odd chunks, whose CTAs
  // run beside the even chunks' with the same block indices
  const bool pcache = p->persistent && p->refine_tc && p->nmax > 32;
  const size_t pcache_set = pcache ? (size_t)p->persist_grid * refine_pcache_bytes() : 0;
  const size_t o_pcache = carve((p->nchunks ? 2 : 1) * pcache_set);
  p->ws_bytes = off;
  err = cudaMalloc((void**)&p->ws, p->ws_bytes);
  if (err != cudaSuccess) {
    delete p;
    return -1000 - (int)err;
  }
  char* w = p->ws;
  p->d_desc = (SmallDesc*)(w + o_desc);
  p->d_perm_bucket = (int*)(w + o_pb);
  p->d_d = w + o_d;
  p->d_e = w + o_e;
  p->d_rot = w + o_rot;
  p->d_hdr = (unsigned*)(w + o_hdr);
  p->d_cst = (ChaseState*)(w + o_cst);
  p->d_pending = (int*)(w + o_pend);
  p->d_stats = (unsigned long long*)(w + o_stats);
  p->d_scale = (int*)(w + o_scale);
  p->d_x32 = refined ? (void*)(w + o_x32) : nullptr;
  p->d_w32 = refined ? (void*)(w + o_w32) : nullptr;
  p->d_vtmp = (jobz == 'N' && refined) ? (void*)(w + o_vtmp) : nullptr;
  p->d_qtmp = p->stein ? (void*)(w + o_qtmp) : nullptr;
  p->d_next = (int*)(w + o_next);
  p->d_chunk_order = (int*)(w + o_corder);
  if (refined) refine_carve(&p->rw, w + o_ref, aoff, woff, batch);
  if (refined) p->rw.pcache = pcache ? (unsigned char*)(w + o_pcache) : nullptr;
  if (batch) err = cudaMemcpy(p->d_desc, desc.data(), sizeof(SmallDesc) * batch, cudaMemcpyHostToDevice);
  if (err == cudaSuccess && !perm_bucket.empty())
    err = cudaMemcpy(p->d_perm_bucket, perm_bucket.data(), sizeof(int) * perm_bucket.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess && !chunk_order.empty())
    err = cudaMemcpy(p->d_chunk_order, chunk_order.data(), sizeof(int) * chunk_order.size(), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(p->d_scale, 0, sizeof(int) * std::max<int64_t>(batch, 1));
  if (err == cudaSuccess) err = cudaMallocHost((void**)&p->pin_pending, sizeof(int) * kMaxBuckets);
  if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
  for (Bucket& bk : p->buckets) {
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&bk.stream, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&bk.join, cudaEventDisableTiming);
  }
  if (p->nchunks) {
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&p->s_in, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&p->s_out, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&p->s_odd, cudaStreamNonBlocking);
    for (int c = 0; c < p->nchunks; c++) {
      if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->ev_in[c], cudaEventDisableTiming);
      if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->ev_solved[c], cudaEventDisableTiming);
    }
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming);
    if (err == cudaSuccess) err = cudaMallocHost((void**)&p->h_cst, sizeof(ChaseState) * batch);
  }
  if (err == cudaSuccess && !p->large_idx.empty())
    err = cudaMallocHost((void**)&p->h_large_info, sizeof(int) * p->large_idx.size());
  for (int b : p->large_idx) {
    if (err != cudaSuccess) break;
    const int nb = (int)n[b];
    if (p->large_ctx.count(nb)) continue;
    LargeCtx* c = nullptr;
    int rc = large_create(&c, nb, precision == GLA_PREC_F64, precision == GLA_PREC_F32_REFINED);
    if (rc) {
      gla_plan_destroy(p);
      return rc;
    }
    p->large_ctx[nb] = c;
    if (precision == GLA_PREC_F32_REFINED) {
      RefineLarge* r = nullptr;
      rc = refine_large_create(&r, nb);
      if (rc) {
        gla_plan_destroy(p);
        return rc;
      }
      p->large_ref[nb] = r;
    }
  }
  if (p->timing)
    for (int b = 0; b < kMaxBuckets && err == cudaSuccess; b++)
      for (int ph = 0; ph < GLA_NUM_PHASES && err == cudaSuccess; ph++)
        for (int k = 0; k < 2 && err == cudaSuccess; k++) err = cudaEventCreate(&p->tev[b][ph][k]);
  if (err != cudaSuccess) {
    gla_plan_destroy(p);
    return -1000 - (int)err;
  }
  if (flags & GLA_FLAG_AUTOTUNE) {
    int rc = autotune_plan(p, flags & (3 | GLA_FLAG_SMALL_LOG | GLA_FLAG_REFINE_QL | GLA_FLAG_REFINE_SIMT));
    if (rc) {
      gla_plan_destroy(p);
      return rc;
    }
  }
  *plan_out = p;
  return 0;
}

int gla_plan_destroy(gla_plan_t p) {
  if (!p) return -1;
  for (Bucket& bk : p->buckets) {
    if (bk.stream) cudaStreamDestroy(bk.stream);
    if (bk.join) cudaEventDestroy(bk.join);
  }
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->s_in) cudaStreamDestroy(p->s_in);
  if (p->s_out) cudaStreamDestroy(p->s_out);
  if (p->s_odd) cudaStreamDestroy(p->s_odd);
  for (int c = 0; c < kMaxChunks; c++) {
    if (p->ev_in[c]) cudaEventDestroy(p->ev_in[c]);
    if (p->ev_solved[c]) cudaEventDestroy(p->ev_solved[c]);
  }
  if (p->ev_out) cudaEventDestroy(p->ev_out);
  cudaFreeHost(p->h_cst);
  for (int b = 0; b < kMaxBuckets; b++)
    for (int ph = 0; ph < GLA_NUM_PHASES; ph++)
      for (int k = 0; k < 2; k++)
        if (p->tev[b][ph][k]) cudaEventDestroy(p->tev[b][ph][k]);
  cudaFree(p->ws);
  cudaFree(p->h_A);
  cudaFree(p->h_w);
  cudaFree(p->h_V);
  cudaFree(p->h_info);
  cudaFreeHost(p->pin_pending);
  cudaFree(p->d_adj);
  cudaFree(p->h_adj);
  large_adjoint_destroy(p->adj_large);
  for (auto& kv : p->large_ctx) large_destroy(kv.second);
  for (auto& kv : p->large_ref) refine_large_destroy(kv.second);
  cudaFreeHost(p->h_large_info);
  delete p;
  return 0;
}

int gla_plan_workspace_size(gla_plan_t p, size_t* bytes) {
  if (!p) return -1;
  if (!bytes) return -2;
  *bytes = p->ws_bytes;
  return 0;
}

int gla_plan_arena_sizes(gla_plan_t p, int64_t* a_elems, int64_t* w_elems) {
  if (!p) return -1;
  if (a_elems) *a_elems = p->a_elems;
  if (w_elems) *w_elems = p->w_elems;
  return 0;
}

}  // extern "C"

namespace {

// One chase pass (+ rotation replay, and the sort once a matrix is done) of
// bucket b on stream st. V holds Q (or the previous pass's rotated Q).
int enqueue_pass(gla_plan_t p, int b, int tcode, void* V, void* wout, int* info, const int* scale,
                 cudaStream_t st, bool timed = false, bool rows2 = false) {
  const Bucket& bk = p->buckets[b];
  const int work_t = tcode == kF64 ? kF64 : kF32;
  const int el = tcode == kF64 ? 8 : 4;
  GLA_CUDA(cudaMemsetAsync(p->d_pending + b, 0, sizeof(int), st));
  if (timed) p->mark(b, GLA_PHASE_CHASE, 0, st);
  GLA_CUDA(launch_chase(work_t, p->algo, bk.count, chase_smem_bytes(bk.nmax, el), st, p->d_desc,
                        p->d_perm_bucket + bk.start, p->d_d, p->d_e, p->d_cst, p->d_rot, p->d_hdr, info, p->tol,
                        kMaxSweepsPerN, p->d_pending + b, p->d_stats, bk.lpw));
  if (timed) {
    p->mark(b, GLA_PHASE_CHASE, 1, st);
    p->mark(b, GLA_PHASE_APPLY, 0, st);
  }
  GLA_CUDA(launch_apply(work_t, bk.count, bk.nt, apply_smem_bytes(bk.nmax, el), st, p->d_desc,
                        p->d_perm_bucket + bk.start, V, p->d_d, wout, p->d_cst, p->d_rot, p->d_hdr, info, scale,
                        rows2));
  if (timed) p->mark(b, GLA_PHASE_APPLY, 1, st);
  return 0;
}

// Chase passes until bucket b has no matrix left with a full rotation log
// (host-checked; used by the single-matrix drivers and as the fallback).
int run_passes_sync(gla_plan_t p, int b, int tcode, void* V, void* wout, int* info, const int* scale,
                    cudaStream_t st, int done_passes, bool rows2 = false) {
  int passes = done_passes;
  for (;;) {
    if (passes > 0) {
      GLA_CUDA(cudaMemcpyAsync(p->pin_pending + b, p->d_pending + b, sizeof(int), cudaMemcpyDeviceToHost, st));
      GLA_CUDA(cudaStreamSynchronize(st));
      if (p->pin_pending[b] == 0 || passes >= kMaxPasses) break;
    }
    int rc = enqueue_pass(p, b, tcode, V, wout, info, scale, st, false, rows2);
    if (rc) return rc;
    passes++;
  }
  p->last_passes = std::max(p->last_passes, passes);
  return 0;
}

}  // namespace

namespace gla {

// Batched SymTridiagonal solve over a plan's buckets: (din, ein) in the
// plan's arena layout (entry i of matrix b at w_off + i), eigenvectors into
// Q, ascending eigenvalues into w. Synchronises st.
int plan_stev_batched(gla_plan_s* p, int tcode, const void* din, const void* ein, void* Q, void* w, int* info,
                      cudaStream_t st) {
  const int work_t = tcode == kF64 ? kF64 : kF32;
  GLA_CUDA(cudaMemsetAsync(p->d_stats, 0, sizeof(unsigned long long) * 4, st));
  p->last_stream = st;
  p->last_passes = 0;
  for (size_t b = 0; b < p->buckets.size(); b++) {
    const Bucket& bk = p->buckets[b];
    GLA_CUDA(launch_init_tridiagonal(work_t, bk.count, st, p->d_desc, p->d_perm_bucket + bk.start, din, ein, p->d_d,
                                     p->d_e, Q, info, p->d_cst, true));
    if (p->stein && work_t == kF32)  // the chase passes below then finish only the matrices it leaves
      GLA_CUDA(launch_stein_tri(bk.count, bk.nmax, st, p->d_desc, p->d_perm_bucket + bk.start, p->d_d, p->d_e, Q, w,
                                p->d_cst, info));
  }
  for (size_t b = 0; b < p->buckets.size(); b++) {
    int rc = run_passes_sync(p, (int)b, work_t, Q, w, info, nullptr, st, 0);
    if (rc) return rc;
  }
  return 0;
}

}  // namespace gla

namespace {

int enqueue_refine(gla_plan_t p, int b, const void* A, int lower, void* Vout, void* w, int* info, cudaStream_t st) {
  const Bucket& bk = p->buckets[b];
  GLA_CUDA(launch_refine(&p->rw, bk.count, bk.nmax, st, p->d_desc, p->d_perm_bucket + bk.start, (const double*)A,
                         lower, (const float*)p->d_x32, (double*)Vout, (double*)w, info, p->d_scale, p->d_stats,
                         p->d_cst, p->refine_tc));
  return 0;
}

// Matrices above the small-matrix limit, one at a time on the caller's
// stream (each large solve uses the whole GPU).
int execute_large(gla_plan_t p, const void* A, void* w, void* V, int* info, cudaStream_t st) {
  const size_t ioe = p->io_elem();
  p->large_iters = 0;
  p->large_refine_n3 = 0;
  p->large_refine_ms = 0.f;
  for (size_t k = 0; k < p->large_idx.size(); k++) {
    const int b = p->large_idx[k];
    const int nb = (int)p->n[b];
    // offsets of matrix b in the packed arenas
    int64_t aoff = 0, woff = 0;
    for (int q = 0; q < b; q++) {
      aoff += p->n[q] * p->n[q];
      woff += p->n[q];
    }
    const void* Ab = (const char*)A + ioe * aoff;
    void* wb = (char*)w + ioe * woff;
    void* Vb = (p->jobz == 'V' && V) ? (char*)V + ioe * aoff : nullptr;
    int inf = 0;
    int rc;
    if (p->prec == GLA_PREC_F32_REFINED) {
      // FP32 solve of the rounded matrix straight into the refinement's
      // buffers, then refinement against the FP64 input
      RefineLarge* r = p->large_ref[nb];
      rc = large_syev(p->large_ctx[nb], kF32FromF64, true, p->uplo == 'L', Ab, nb, refine_large_wbuf(r),
                      refine_large_xbuf(r), nb, &inf, st);
      if (rc) return rc;
      if (inf == 0) {
        const auto t0 = std::chrono::steady_clock::now();
        rc = refine_large_run(r, (const double*)Ab, nb, p->uplo == 'L', refine_large_xbuf(r), nb,
                              refine_large_wbuf(r), (double*)wb, (double*)Vb, nb, st);
        p->large_refine_ms +=
            std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
        p->large_refine_n3 += (double)refine_large_iters(r) * nb * (double)nb * nb;
        if (rc == -1)
          inf = -1;
        else if (rc)
          return rc;
        p->large_iters = std::max(p->large_iters, refine_large_iters(r));
      }
    } else {
      const int tc = p->prec == GLA_PREC_F64 ? kF64 : kF32;
      rc = large_syev(p->large_ctx[nb], tc, p->jobz == 'V', p->uplo == 'L', Ab, nb, wb, Vb, nb, &inf, st);
      if (rc) return rc;
    }
    p->h_large_info[k] = inf;
    GLA_CUDA(cudaMemcpyAsync(info + b, p->h_large_info + k, sizeof(int), cudaMemcpyHostToDevice, st));
  }
  return 0;
}

// The persistent launch over `count` matrices of the work list `order`
// (orders descending), with work counter `next` and the refinement
// scratch `rw` (its slice scratch is per block index).
int persistent_solve(gla_plan_t p, const void* A, void* w, void* Vout, int* info, cudaStream_t st, const int* order,
                     int count, int* next, const RefineWork* rw) {
  GLA_CUDA(cudaMemsetAsync(next, 0, sizeof(int), st));
  GLA_CUDA(launch_solve_refine(rw, count, p->nmax, std::min(p->persist_grid, count), st, p->d_desc, order, next,
                               (const double*)A, p->uplo == 'L', (float*)p->d_d, (float*)p->d_e,
                               (float*)p->d_x32, info, p->d_cst, p->d_scale, (float*)p->d_w32, (float*)p->d_qtmp,
                               (double*)Vout, (double*)w, p->d_stats, p->refine_tc));
  return 0;
}

int persistent_finish(gla_plan_t p, const void* A, void* w, void* Vout, int* info, cudaStream_t st);

// The orders <= 128 of an FP32 + refinement plan with the in-kernel FP32
// solver: one persistent launch solves and refines every matrix it can
// (largest first, from a work counter); the QL chase, rotation replay and
// refinement kernels, launched once over all those matrices, finish the
// few it leaves (they skip the rest). With no host check in capture-safe
// plans; otherwise a full rotation log is finished by further host-checked
// passes.
int execute_persistent(gla_plan_t p, const void* A, void* w, void* Vout, int* info, cudaStream_t st) {
  p->mark(0, GLA_PHASE_TRIDIAG, 0, st);
  if (int rc = persistent_solve(p, A, w, Vout, info, st, p->d_perm_bucket, p->nwork, p->d_next, &p->rw)) return rc;
  p->mark(0, GLA_PHASE_TRIDIAG, 1, st);
  return persistent_finish(p, A, w, Vout, info, st);
}

// The chase, rotation-replay and refinement launches over the whole work
// list that finish the matrices the persistent launches left (they return
// at once for the others).
int persistent_finish(gla_plan_t p, const void* A, void* w, void* Vout, int* info, cudaStream_t st) {
  const int lower = p->uplo == 'L';
  const int n = p->nwork;
  const int npass = p->graph ? kGraphPasses : kAsyncPasses;
  auto pass = [&]() -> int {
    GLA_CUDA(cudaMemsetAsync(p->d_pending, 0, sizeof(int), st));
    GLA_CUDA(launch_chase(kF32, p->algo, n, chase_smem_bytes(p->nmax, 4), st, p->d_desc, p->d_perm_bucket, p->d_d,
                          p->d_e, p->d_cst, p->d_rot, p->d_hdr, info, p->tol, kMaxSweepsPerN, p->d_pending,
                          p->d_stats));
    GLA_CUDA(launch_apply(kF32, n, kSmallMaxN, apply_smem_bytes(p->nmax, 4), st, p->d_desc, p->d_perm_bucket,
                          p->d_x32, p->d_d, p->d_w32, p->d_cst, p->d_rot, p->d_hdr, info, p->d_scale));
    return 0;
  };
  p->mark(0, GLA_PHASE_CHASE, 0, st);
  for (int k = 0; k < npass; k++) {
    int rc = pass();
    if (rc) return rc;
  }
  p->mark(0, GLA_PHASE_CHASE, 1, st);
  int passes = npass;
  if (p->graph) {
    GLA_CUDA(launch_mark_unfinished(n, st, p->d_desc, p->d_perm_bucket, p->d_cst, info));
  } else {
    for (;;) {  // a rotation log that filled up in every pass so far
      GLA_CUDA(cudaMemcpyAsync(p->pin_pending, p->d_pending, sizeof(int), cudaMemcpyDeviceToHost, st));
      GLA_CUDA(cudaStreamSynchronize(st));
      if (p->pin_pending[0] == 0 || passes >= kMaxPasses) break;
      int rc = pass();
      if (rc) return rc;
      passes++;
    }
  }
  p->last_passes = passes;
  p->mark(0, GLA_PHASE_REFINE, 0, st);
  GLA_CUDA(launch_refine(&p->rw, n, p->nmax, st, p->d_desc, p->d_perm_bucket, (const double*)A, lower,
                         (const float*)p->d_x32, (double*)Vout, (double*)w, info, p->d_scale, p->d_stats, p->d_cst,
                         p->refine_tc));
  p->mark(0, GLA_PHASE_REFINE, 1, st);
  return 0;
}

// Every size bucket runs its whole pipeline on its own stream (buckets are
// independent), forked from and joined back into the caller's stream, so
// the long chases of the largest matrices overlap with the other buckets.
int plan_execute(gla_plan_t p, const void* A, void* w, void* V, int* info, cudaStream_t st) {
  p->last_stream = st;
  p->last_passes = 0;
  for (int b = 0; b < kMaxBuckets; b++)
    for (int ph = 0; ph < GLA_NUM_PHASES; ph++) p->tused[b][ph] = false;
  GLA_CUDA(cudaMemsetAsync(p->d_stats, 0, sizeof(unsigned long long) * 4, st));
  if (p->batch) GLA_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * p->batch, st));
  int rc_large = execute_large(p, A, w, V, info, st);
  if (rc_large) return rc_large;
  if (p->nwork == 0) return 0;
  const int lower = p->uplo == 'L';
  const bool refined = p->prec == GLA_PREC_F32_REFINED;
  const bool wantq = p->jobz == 'V' || refined;
  const int tc = p->tcode();
  const int work_t = tc == kF64 ? kF64 : kF32;
  const int el = (int)p->elem();
  void* Q = refined ? p->d_x32 : V;
  void* wq = refined ? p->d_w32 : w;
  const int* scale = refined ? p->d_scale : nullptr;
  void* Vout = p->jobz == 'V' ? V : p->d_vtmp;
  if (refined) GLA_CUDA(cudaMemsetAsync(p->rw.err, 0, sizeof(int), st));
  if (p->persistent) return execute_persistent(p, A, w, Vout, info, st);
  const int nb = (int)p->buckets.size();
  GLA_CUDA(cudaEventRecord(p->fork, st));
  for (int b = 0; b < nb; b++) {
    const Bucket& bk = p->buckets[b];
    cudaStream_t s = bk.stream;
    GLA_CUDA(cudaStreamWaitEvent(s, p->fork, 0));
    p->mark(b, GLA_PHASE_TRIDIAG, 0, s);
    GLA_CUDA(launch_tridiag(tc, wantq, bk.count, bk.nt_tri, tridiag_smem_bytes(bk.nmax, bk.nt_tri, el, p->stein), s,
                            p->d_desc, p->d_perm_bucket + bk.start, A, lower, p->d_d, p->d_e, Q, info, p->d_cst,
                            p->d_scale, p->stein, wq, p->d_qtmp));
    p->mark(b, GLA_PHASE_TRIDIAG, 1, s);
    if (wantq) {
      const int npass = p->graph ? kGraphPasses : kAsyncPasses;
      for (int k = 0; k < npass; k++) {  // passes after the first only finish overflowed logs
        int rc = enqueue_pass(p, b, tc, Q, wq, info, scale, s, k == 0);
        if (rc) return rc;
      }
      if (p->graph)
        GLA_CUDA(launch_mark_unfinished(bk.count, s, p->d_desc, p->d_perm_bucket + bk.start, p->d_cst, info));
      if (refined) {
        p->mark(b, GLA_PHASE_REFINE, 0, s);
        int rc = enqueue_refine(p, b, A, lower, Vout, w, info, s);
        if (rc) return rc;
        p->mark(b, GLA_PHASE_REFINE, 1, s);
      }
      if (!p->graph)
        GLA_CUDA(cudaMemcpyAsync(p->pin_pending + b, p->d_pending + b, sizeof(int), cudaMemcpyDeviceToHost, s));
    } else {
      p->mark(b, GLA_PHASE_CHASE, 0, s);
      GLA_CUDA(launch_chase(work_t, kAlgoPWK, bk.count, chase_smem_bytes(bk.nmax, el), s, p->d_desc,
                            p->d_perm_bucket + bk.start, p->d_d, p->d_e, p->d_cst, nullptr, nullptr, info, p->tol,
                            kMaxSweepsPerN, p->d_pending + b, p->d_stats, bk.lpw));
      GLA_CUDA(launch_sort_values(work_t, bk.count, s, p->d_desc, p->d_perm_bucket + bk.start, p->d_d, w, info,
                                  nullptr));
      p->mark(b, GLA_PHASE_CHASE, 1, s);
    }
    GLA_CUDA(cudaEventRecord(bk.join, s));
    GLA_CUDA(cudaStreamWaitEvent(st, bk.join, 0));
  }
  if (!wantq) {
    p->last_passes = 1;
    return 0;
  }
  if (p->graph) {
    p->last_passes = kGraphPasses;
    return 0;
  }
  // A matrix whose rotation log filled up in both asynchronous passes (never
  // seen on random spectra with the 2 n^2 capacity) is finished here.
  GLA_CUDA(cudaStreamSynchronize(st));
  p->last_passes = kAsyncPasses;
  for (int b = 0; b < nb; b++) {
    if (p->pin_pending[b] == 0) continue;
    int rc = run_passes_sync(p, b, tc, Q, wq, info, scale, st, kAsyncPasses);
    if (rc) return rc;
    if (refined) {
      rc = enqueue_refine(p, b, A, lower, Vout, w, info, st);
      if (rc) return rc;
    }
  }
  return 0;
}

}  // namespace

extern "C" {

int gla_plan_execute(gla_plan_t p, const void* A, void* w, void* V, int* info, void* stream) {
  if (!p) return -1;
  if (!A && p->a_elems) return -2;
  if (!w && p->w_elems) return -3;
  if (p->jobz == 'V' && !V && p->a_elems) return -4;
  if (!info && p->batch) return -5;
  return plan_execute(p, A, w, V, info, (cudaStream_t)stream);
}

}  // extern "C"

namespace {
// Device staging of the _host entry points: all four buffers, or none (a
// later call retries). V also holds the 2 x n row blocks of eigen2.
int ensure_staging(gla_plan_t p) {
  if (p->h_info) return 0;
  const size_t ioe = p->io_elem();
  const size_t abytes = ioe * std::max<int64_t>(p->a_elems, 1), wbytes = ioe * std::max<int64_t>(p->w_elems, 1);
  cudaError_t e = cudaMalloc(&p->h_A, abytes);
  if (e == cudaSuccess) e = cudaMalloc(&p->h_w, wbytes);
  if (e == cudaSuccess) e = cudaMalloc(&p->h_V, p->jobz == 'V' ? std::max(abytes, 2 * wbytes) : 16);
  if (e == cudaSuccess) e = cudaMalloc((void**)&p->h_info, sizeof(int) * std::max<int64_t>(p->batch, 1));
  if (e != cudaSuccess) {
    cudaFree(p->h_A);
    cudaFree(p->h_w);
    cudaFree(p->h_V);
    p->h_A = p->h_w = p->h_V = nullptr;
    p->h_info = nullptr;
    return -1000 - (int)e;
  }
  return 0;
}

// Page-locked host memory (registered or allocated by CUDA): copies from
// and to it run asynchronously.
bool host_pinned(const void* ptr) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// gla_plan_execute_host of a persistent plan, pipelined over its chunks:
// chunk c's A goes in on s_in; its persistent launch waits for it, on the
// caller's stream for even c and on s_odd for odd c, with its own work
// counter (and, for odd c, the second set of slice scratch), so that it
// starts on the SMs the previous chunk's last matrices leave idle; its w
// and V come out on s_out while later chunks are solved. The launches that
// finish the matrices the persistent kernel left (the QL chase and its
// replay, refinement) run once at the end over the whole batch, as in
// execute_persistent; those matrices, known from the chase states copied
// after the last persistent launch, are copied out again afterwards.
// Results are those of gla_plan_execute.
int pipelined_body(gla_plan_t p, const void* A_host, void* w_host, void* V_host, int* info_host, cudaStream_t st) {
  const size_t ioe = p->io_elem();
  const bool wantv = p->jobz == 'V';
  void* Vout = wantv ? p->h_V : p->d_vtmp;
  char* dA = static_cast<char*>(p->h_A);
  char* dW = static_cast<char*>(p->h_w);
  char* dV = static_cast<char*>(p->h_V);
  const char* hA = static_cast<const char*>(A_host);
  char* hW = static_cast<char*>(w_host);
  char* hV = static_cast<char*>(V_host);
  p->last_stream = st;
  p->last_passes = 0;
  for (int b = 0; b < kMaxBuckets; b++)
    for (int ph = 0; ph < GLA_NUM_PHASES; ph++) p->tused[b][ph] = false;
  GLA_CUDA(cudaEventRecord(p->fork, st));
  GLA_CUDA(cudaStreamWaitEvent(p->s_in, p->fork, 0));
  GLA_CUDA(cudaStreamWaitEvent(p->s_out, p->fork, 0));
  RefineWork rw_odd = p->rw;
  if (rw_odd.pcache) rw_odd.pcache += (size_t)p->persist_grid * refine_pcache_bytes();
  for (int c = 0; c < p->nchunks; c++) {
    const size_t a0 = ioe * p->chunk_a[c], ab = ioe * (p->chunk_a[c + 1] - p->chunk_a[c]);
    if (ab) GLA_CUDA(cudaMemcpyAsync(dA + a0, hA + a0, ab, cudaMemcpyHostToDevice, p->s_in));
    GLA_CUDA(cudaEventRecord(p->ev_in[c], p->s_in));
  }
  GLA_CUDA(cudaMemsetAsync(p->d_stats, 0, sizeof(unsigned long long) * 4, st));
  GLA_CUDA(cudaMemsetAsync(p->h_info, 0, sizeof(int) * p->batch, st));
  GLA_CUDA(cudaMemsetAsync(p->rw.err, 0, sizeof(int), st));
  // the memsets above come before every chunk's launch
  GLA_CUDA(cudaEventRecord(p->fork, st));
  GLA_CUDA(cudaStreamWaitEvent(p->s_odd, p->fork, 0));
  for (int c = 0; c < p->nchunks; c++) {
    cudaStream_t cs = (c & 1) ? p->s_odd : st;
    GLA_CUDA(cudaStreamWaitEvent(cs, p->ev_in[c], 0));
    if (int rc = persistent_solve(p, p->h_A, p->h_w, Vout, p->h_info, cs, p->d_chunk_order + p->chunk_start[c],
                                  p->chunk_start[c + 1] - p->chunk_start[c], p->d_next + c,
                                  (c & 1) ? &rw_odd : &p->rw))
      return rc;
    GLA_CUDA(cudaEventRecord(p->ev_solved[c], cs));
    GLA_CUDA(cudaStreamWaitEvent(p->s_out, p->ev_solved[c], 0));
    const size_t w0 = ioe * p->chunk_w[c], wb = ioe * (p->chunk_w[c + 1] - p->chunk_w[c]);
    const size_t a0 = ioe * p->chunk_a[c], ab = ioe * (p->chunk_a[c + 1] - p->chunk_a[c]);
    if (wb) GLA_CUDA(cudaMemcpyAsync(hW + w0, dW + w0, wb, cudaMemcpyDeviceToHost, p->s_out));
    if (wantv && ab) GLA_CUDA(cudaMemcpyAsync(hV + a0, dV + a0, ab, cudaMemcpyDeviceToHost, p->s_out));
  }
  for (int c = 1; c < p->nchunks; c += 2) GLA_CUDA(cudaStreamWaitEvent(st, p->ev_solved[c], 0));
  GLA_CUDA(cudaMemcpyAsync(p->h_cst, p->d_cst, sizeof(ChaseState) * p->batch, cudaMemcpyDeviceToHost, st));
  if (int rc = persistent_finish(p, p->h_A, p->h_w, Vout, p->h_info, st)) return rc;
  GLA_CUDA(cudaMemcpyAsync(info_host, p->h_info, sizeof(int) * p->batch, cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaEventRecord(p->ev_out, p->s_out));
  GLA_CUDA(cudaStreamWaitEvent(st, p->ev_out, 0));
  GLA_CUDA(cudaStreamSynchronize(st));
  // the matrices finished after their chunk's copy
  std::vector<int64_t> late;
  for (int64_t b = 0; b < p->batch; b++)
    if (p->n[b] >= 1 && p->h_cst[b].applied != kRefinedInKernel) late.push_back(b);
  if (late.size() > 64) {
    GLA_CUDA(cudaMemcpyAsync(hW, dW, ioe * p->w_elems, cudaMemcpyDeviceToHost, st));
    if (wantv) GLA_CUDA(cudaMemcpyAsync(hV, dV, ioe * p->a_elems, cudaMemcpyDeviceToHost, st));
  } else if (!late.empty()) {
    size_t k = 0;
    int64_t aoff = 0, woff = 0;
    for (int64_t b = 0; b < p->batch && k < late.size(); b++) {
      const int64_t nb = p->n[b];
      if (b == late[k]) {
        GLA_CUDA(cudaMemcpyAsync(hW + ioe * woff, dW + ioe * woff, ioe * nb, cudaMemcpyDeviceToHost, st));
        if (wantv)
          GLA_CUDA(cudaMemcpyAsync(hV + ioe * aoff, dV + ioe * aoff, ioe * nb * nb, cudaMemcpyDeviceToHost, st));
        k++;
      }
      aoff += nb * nb;
      woff += nb;
    }
  }
  if (!late.empty()) GLA_CUDA(cudaStreamSynchronize(st));
  int bad = 0;
  for (int64_t b = 0; b < p->batch; b++) bad += info_host[b] != 0;
  return bad;
}

int execute_host_pipelined(gla_plan_t p, const void* A_host, void* w_host, void* V_host, int* info_host,
                           cudaStream_t st) {
  const int rc = pipelined_body(p, A_host, w_host, V_host, info_host, st);
  if (rc < 0) {  // an error: none of this call's copies or solves stays in flight
    cudaStreamSynchronize(p->s_in);
    cudaStreamSynchronize(p->s_odd);
    cudaStreamSynchronize(p->s_out);
    cudaStreamSynchronize(st);
  }
  return rc;
}
}  // namespace

extern "C" {

int gla_plan_execute_host(gla_plan_t p, const void* A_host, void* w_host, void* V_host, int* info_host,
                          void* stream) {
  if (!p) return -1;
  if (!A_host && p->a_elems) return -2;
  if (!w_host && p->w_elems) return -3;
  if (p->jobz == 'V' && !V_host && p->a_elems) return -4;
  if (!info_host && p->batch) return -5;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t ioe = p->io_elem();
  if (int rs = ensure_staging(p)) return rs;
  p->last_pipelined =
      p->nchunks && host_pinned(A_host) && host_pinned(w_host) && (p->jobz != 'V' || host_pinned(V_host));
  if (p->last_pipelined) return execute_host_pipelined(p, A_host, w_host, V_host, info_host, st);
  GLA_CUDA(cudaMemcpyAsync(p->h_A, A_host, ioe * p->a_elems, cudaMemcpyHostToDevice, st));
  int rc = plan_execute(p, p->h_A, p->h_w, p->h_V, p->h_info, st);
  if (rc) return rc;
  GLA_CUDA(cudaMemcpyAsync(w_host, p->h_w, ioe * p->w_elems, cudaMemcpyDeviceToHost, st));
  if (p->jobz == 'V') GLA_CUDA(cudaMemcpyAsync(V_host, p->h_V, ioe * p->a_elems, cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaMemcpyAsync(info_host, p->h_info, sizeof(int) * p->batch, cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaStreamSynchronize(st));
  int bad = 0;
  for (int64_t b = 0; b < p->batch; b++) bad += info_host[b] != 0;
  return bad;
}

int gla_plan_execute_eigen2(gla_plan_t p, const void* A, void* w, void* V2, int* info, void* stream) {
  if (!p) return -1;
  if (!A && p->a_elems) return -2;
  if (!w && p->w_elems) return -3;
  if (!V2 && p->w_elems) return -4;
  if (!info && p->batch) return -5;
  if (p->jobz != 'V' || p->prec == GLA_PREC_F32_REFINED || !p->large_idx.empty()) return GLA_ERR_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  p->last_stream = st;
  p->last_passes = 0;
  for (int b = 0; b < kMaxBuckets; b++)
    for (int ph = 0; ph < GLA_NUM_PHASES; ph++) p->tused[b][ph] = false;
  GLA_CUDA(cudaMemsetAsync(p->d_stats, 0, sizeof(unsigned long long) * 4, st));
  if (p->batch) GLA_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * p->batch, st));
  if (p->nwork == 0) return 0;
  const int tc = p->tcode(), el = (int)p->elem();
  const int nb = (int)p->buckets.size();
  GLA_CUDA(cudaEventRecord(p->fork, st));
  for (int b = 0; b < nb; b++) {
    const Bucket& bk = p->buckets[b];
    cudaStream_t s = bk.stream;
    GLA_CUDA(cudaStreamWaitEvent(s, p->fork, 0));
    p->mark(b, GLA_PHASE_TRIDIAG, 0, s);
    GLA_CUDA(launch_tridiag(tc, false, bk.count, bk.nt_tri, tridiag_smem_bytes(bk.nmax, bk.nt_tri, el), s, p->d_desc,
                            p->d_perm_bucket + bk.start, A, p->uplo == 'L', p->d_d, p->d_e, nullptr, info, p->d_cst,
                            p->d_scale, false, nullptr, nullptr, V2));
    p->mark(b, GLA_PHASE_TRIDIAG, 1, s);
    const int npass = p->graph ? kGraphPasses : kAsyncPasses;
    for (int k = 0; k < npass; k++) {
      int rc = enqueue_pass(p, b, tc, V2, w, info, nullptr, s, k == 0, true);
      if (rc) return rc;
    }
    if (p->graph)
      GLA_CUDA(launch_mark_unfinished(bk.count, s, p->d_desc, p->d_perm_bucket + bk.start, p->d_cst, info));
    else
      GLA_CUDA(cudaMemcpyAsync(p->pin_pending + b, p->d_pending + b, sizeof(int), cudaMemcpyDeviceToHost, s));
    GLA_CUDA(cudaEventRecord(bk.join, s));
    GLA_CUDA(cudaStreamWaitEvent(st, bk.join, 0));
  }
  if (p->graph) {
    p->last_passes = kGraphPasses;
    return 0;
  }
  GLA_CUDA(cudaStreamSynchronize(st));
  p->last_passes = kAsyncPasses;
  for (int b = 0; b < nb; b++) {
    if (p->pin_pending[b] == 0) continue;
    int rc = run_passes_sync(p, b, tc, V2, w, info, nullptr, st, kAsyncPasses, true);
    if (rc) return rc;
  }
  return 0;
}

int gla_plan_execute_eigen2_host(gla_plan_t p, const void* A_host, void* w_host, void* V2_host, int* info_host,
                                 void* stream) {
  if (!p) return -1;
  if (!A_host && p->a_elems) return -2;
  if (!w_host && p->w_elems) return -3;
  if (!V2_host && p->w_elems) return -4;
  if (!info_host && p->batch) return -5;
  if (p->jobz != 'V' || p->prec == GLA_PREC_F32_REFINED || !p->large_idx.empty()) return GLA_ERR_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t ioe = p->io_elem();
  if (int rs = ensure_staging(p)) return rs;
  GLA_CUDA(cudaMemcpyAsync(p->h_A, A_host, ioe * p->a_elems, cudaMemcpyHostToDevice, st));
  int rc = gla_plan_execute_eigen2(p, p->h_A, p->h_w, p->h_V, p->h_info, st);
  if (rc) return rc;
  GLA_CUDA(cudaMemcpyAsync(w_host, p->h_w, ioe * p->w_elems, cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaMemcpyAsync(V2_host, p->h_V, 2 * ioe * p->w_elems, cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaMemcpyAsync(info_host, p->h_info, sizeof(int) * p->batch, cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaStreamSynchronize(st));
  int bad = 0;
  for (int64_t b = 0; b < p->batch; b++) bad += info_host[b] != 0;
  return bad;
}

int gla_plan_adjoint(gla_plan_t p, const double* w, const double* V, const double* wbar, const double* Vbar,
                     double* Abar, double gap_rel, void* stream) {
  if (!p) return -1;
  if (p->prec == GLA_PREC_F32) return -1;  // the adjoint works on FP64 eigenpairs
  if (!w && p->w_elems) return -2;
  if (!V && p->a_elems) return -3;
  if (!wbar && p->w_elems) return -4;
  if (!Vbar && p->a_elems) return -5;
  if (!Abar && p->a_elems) return -6;
  if (!(gap_rel == gap_rel)) return -7;
  const double gr = gap_rel > 0 ? gap_rel : 1e-10;
  cudaStream_t st = (cudaStream_t)stream;
  if (p->nwork > 0) {  // orders <= GLA_MAX_SMALL_N: one CTA per matrix
    if (!p->d_adj) GLA_CUDA(cache_alloc(&p->d_adj, adjoint_workspace_bytes(p->a_elems)));
    GLA_CUDA(launch_adjoint(p->nwork, st, p->d_desc, p->d_perm_bucket, w, V, wbar, Vbar, Abar, p->d_adj, p->a_elems,
                            gr));
  }
  if (!p->large_idx.empty()) {  // larger orders: three FP64 GEMMs each, one shared workspace
    int nl = 0;
    for (int b : p->large_idx) nl = std::max(nl, (int)p->n[b]);
    if (!p->adj_large) {
      int rc = large_adjoint_create(&p->adj_large, nl);
      if (rc) return rc;
    }
    for (int b : p->large_idx) {
      const int nb = (int)p->n[b];
      int64_t aoff = 0, woff = 0;
      for (int q = 0; q < b; q++) {
        aoff += p->n[q] * p->n[q];
        woff += p->n[q];
      }
      GLA_CUDA(large_adjoint(p->adj_large, nb, w + woff, V + aoff, nb, wbar + woff, Vbar + aoff, nb, Abar + aoff, nb,
                             gr, st));
    }
  }
  return 0;
}

int gla_plan_adjoint_host(gla_plan_t p, const double* w, const double* V, const double* wbar, const double* Vbar,
                          double* Abar, double gap_rel, void* stream) {
  if (!p) return -1;
  if (p->prec == GLA_PREC_F32) return -1;
  if (!w && p->w_elems) return -2;
  if (!V && p->a_elems) return -3;
  if (!wbar && p->w_elems) return -4;
  if (!Vbar && p->a_elems) return -5;
  if (!Abar && p->a_elems) return -6;
  if (!(gap_rel == gap_rel)) return -7;
  if (p->a_elems == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t ab = sizeof(double) * p->a_elems, wb = sizeof(double) * p->w_elems;
  if (!p->h_adj) GLA_CUDA(cache_alloc(&p->h_adj, 3 * ab + 2 * wb));
  double* dV = p->h_adj;
  double* dVbar = dV + p->a_elems;
  double* dAbar = dVbar + p->a_elems;
  double* dw = dAbar + p->a_elems;
  double* dwbar = dw + p->w_elems;
  GLA_CUDA(cudaMemcpyAsync(dV, V, ab, cudaMemcpyHostToDevice, st));
  GLA_CUDA(cudaMemcpyAsync(dVbar, Vbar, ab, cudaMemcpyHostToDevice, st));
  GLA_CUDA(cudaMemcpyAsync(dw, w, wb, cudaMemcpyHostToDevice, st));
  GLA_CUDA(cudaMemcpyAsync(dwbar, wbar, wb, cudaMemcpyHostToDevice, st));
  int rc = gla_plan_adjoint(p, dw, dV, dwbar, dVbar, dAbar, gap_rel, stream);
  if (rc) return rc;
  GLA_CUDA(cudaMemcpyAsync(Abar, dAbar, ab, cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int gla_plan_phase_times(gla_plan_t p, float* ms) {
  if (!p) return -1;
  if (!ms) return -2;
  for (int ph = 0; ph < GLA_NUM_PHASES; ph++) ms[ph] = 0.f;
  if (!p->timing) return 0;
  GLA_CUDA(cudaStreamSynchronize(p->last_stream));
  for (int b = 0; b < kMaxBuckets; b++)
    for (int ph = 0; ph < GLA_NUM_PHASES; ph++) {
      if (!p->tused[b][ph]) continue;
      float t = 0.f;
      GLA_CUDA(cudaEventElapsedTime(&t, p->tev[b][ph][0], p->tev[b][ph][1]));
      ms[ph] += t;
    }
  // large matrices: tridiagonalisation, divide and conquer (reported as the
  // chase phase), back-transformation (reported as apply)
  for (int b : p->large_idx) {
    float st[3];
    large_stage_ms(p->large_ctx[(int)p->n[b]], st);
    ms[GLA_PHASE_TRIDIAG] += st[0];
    ms[GLA_PHASE_CHASE] += st[1];
    ms[GLA_PHASE_APPLY] += st[2];
  }
  ms[GLA_PHASE_REFINE] += p->large_refine_ms;
  return 0;
}

int gla_plan_stats(gla_plan_t p, int64_t* rotations, int64_t* sweeps, int* passes) {
  int64_t c[GLA_NUM_COUNTERS] = {};
  int rc = gla_plan_counters(p, c);
  if (rc) return rc;
  if (rotations) *rotations = c[GLA_COUNTER_ROTATIONS];
  if (sweeps) *sweeps = c[GLA_COUNTER_SWEEPS];
  if (passes) *passes = (int)c[GLA_COUNTER_PASSES];
  return 0;
}

int gla_plan_host_pipeline(gla_plan_t p, int* chunks, int* last_pipelined) {
  if (!p) return -1;
  if (!chunks) return -2;
  if (!last_pipelined) return -3;
  *chunks = p->nchunks;
  *last_pipelined = p->last_pipelined ? 1 : 0;
  return 0;
}

int gla_plan_counters(gla_plan_t p, int64_t* c) {
  if (!p) return -1;
  if (!c) return -2;
  unsigned long long h[4] = {0, 0, 0, 0};
  GLA_CUDA(cudaStreamSynchronize(p->last_stream));
  GLA_CUDA(cudaMemcpy(h, p->d_stats, sizeof(h), cudaMemcpyDeviceToHost));
  c[GLA_COUNTER_ROTATIONS] = (int64_t)h[0];
  c[GLA_COUNTER_SWEEPS] = (int64_t)h[1];
  c[GLA_COUNTER_ROW_ROTATIONS] = (int64_t)h[2];
  c[GLA_COUNTER_REFINE_N3] = (int64_t)h[3] + (int64_t)p->large_refine_n3;
  c[GLA_COUNTER_PASSES] = p->last_passes;
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- single-matrix drivers
namespace {

struct SingleKey {
  int prec;
  char jobz, uplo;
  int64_t n;
  int flags;
  bool operator<(const SingleKey& o) const {
    return std::tie(prec, jobz, uplo, n, flags) < std::tie(o.prec, o.jobz, o.uplo, o.n, o.flags);
  }
};
struct SingleEntry {
  gla_plan_t plan = nullptr;
  void* buf = nullptr;  // packed n*n matrix + n values
  int* dinfo = nullptr;
};
std::mutex g_single_mu;
std::map<SingleKey, SingleEntry> g_single;
std::mutex g_gemm_mu;
OzWork* g_gemm_w = nullptr;  // slice buffers of gla_gemm_df
cudaEvent_t g_gemm_ev[3] = {nullptr, nullptr, nullptr};  // slicing start, GEMM start, GEMM end
bool g_gemm_timed = false;
std::map<int, LargeCtx*> g_stev_large;  // gla_dstev above GLA_MAX_SMALL_N

int single_entry(int prec, char jobz, char uplo, int64_t n, int flags, SingleEntry** out) {
  SingleKey k{prec, jobz, uplo, n, flags};
  auto it = g_single.find(k);
  if (it != g_single.end()) {
    *out = &it->second;
    return 0;
  }
  SingleEntry e;
  int rc = gla_plan_create(&e.plan, prec, jobz, uplo, 1, &n, 0.0, flags);
  if (rc) return rc;
  const size_t el = prec == GLA_PREC_F32 ? 4 : 8;
  cudaError_t ce = cudaMalloc(&e.buf, el * (size_t)(n * n + 2 * n + 2));
  if (ce == cudaSuccess) ce = cudaMalloc((void**)&e.dinfo, sizeof(int));
  if (ce != cudaSuccess) {  // nothing is cached on failure
    cudaFree(e.buf);
    gla_plan_destroy(e.plan);
    return -1000 - (int)ce;
  }
  auto r = g_single.emplace(k, e);
  *out = &r.first->second;
  return 0;
}

template <class T>
int syev_single(int prec, char jobz, char uplo, int64_t n, T* A, int64_t lda, T* w, int* info, void* stream) {
  if (jobz != 'V' && jobz != 'N') return -1;
  if (uplo != 'L' && uplo != 'U') return -2;
  if (n < 0 || n > GLA_MAX_N) return -3;
  if (!A && n) return -4;
  if (lda < std::max<int64_t>(1, n)) return -5;
  if (!w && n) return -6;
  if (!info) return -7;
  *info = 0;
  if (n == 0) return 0;
  std::lock_guard<std::mutex> lk(g_single_mu);
  SingleEntry* e;
  int rc = single_entry(prec, jobz, uplo, n, 0, &e);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  T* buf = (T*)e->buf;
  GLA_CUDA(cudaMemcpy2DAsync(buf, sizeof(T) * n, A, sizeof(T) * lda, sizeof(T) * n, n, cudaMemcpyDeviceToDevice, st));
  rc = gla_plan_execute(e->plan, buf, w, buf, e->dinfo, stream);
  if (rc) return rc;
  if (jobz == 'V')
    GLA_CUDA(cudaMemcpy2DAsync(A, sizeof(T) * lda, buf, sizeof(T) * n, sizeof(T) * n, n, cudaMemcpyDeviceToDevice, st));
  GLA_CUDA(cudaMemcpyAsync(info, e->dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaStreamSynchronize(st));
  return *info != 0;
}

}  // namespace

extern "C" {

int gla_dsyev(char jobz, char uplo, int64_t n, double* A, int64_t lda, double* w, int* info, void* stream) {
  return syev_single<double>(GLA_PREC_F64, jobz, uplo, n, A, lda, w, info, stream);
}

int gla_ssyev(char jobz, char uplo, int64_t n, float* A, int64_t lda, float* w, int* info, void* stream) {
  return syev_single<float>(GLA_PREC_F32, jobz, uplo, n, A, lda, w, info, stream);
}

int gla_gemm_df(int64_t m, int64_t n, int64_t k, const float* Ahi, const float* Alo, int64_t lda, const float* Bhi,
                const float* Blo, int64_t ldb, float* Chi, float* Clo, int64_t ldc, void* stream) {
  if (m < 0 || m > (1 << 24)) return -1;
  if (n < 0 || n > (1 << 24)) return -2;
  if (k < 0 || k > (1 << 24)) return -3;
  if (!Ahi && m && k) return -4;
  if (lda < std::max<int64_t>(1, m)) return -6;
  if (!Bhi && n && k) return -7;
  if (ldb < std::max<int64_t>(1, k)) return -9;
  if ((!Chi || !Clo) && m && n) return -10;
  if (ldc < std::max<int64_t>(1, m)) return -12;
  if (m == 0 || n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  if (k == 0) {
    GLA_CUDA(cudaMemset2DAsync(Chi, sizeof(float) * ldc, 0, sizeof(float) * m, n, st));
    GLA_CUDA(cudaMemset2DAsync(Clo, sizeof(float) * ldc, 0, sizeof(float) * m, n, st));
    return 0;
  }
  std::lock_guard<std::mutex> lk(g_gemm_mu);
  if (g_gemm_w) {
    int h = 0;
    GLA_CUDA(cudaMemcpy(&h, oz_error_word(g_gemm_w), sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
      GLA_CUDA(cudaMemset(oz_error_word(g_gemm_w), 0, sizeof(int)));
      return -1000 - (int)cudaErrorLaunchTimeout;
    }
  }
  if (!g_gemm_w || !oz_fits(g_gemm_w, (int)m, (int)n, (int)k)) {
    if (g_gemm_w) {
      GLA_CUDA(cudaDeviceSynchronize());
      oz_destroy(g_gemm_w);
      g_gemm_w = nullptr;
    }
    int rc = oz_create(&g_gemm_w, (int)m, (int)n, (int)k);
    if (rc) return rc;
  }
  if (!g_gemm_ev[0])
    for (auto& ev : g_gemm_ev) GLA_CUDA(cudaEventCreate(&ev));
  GLA_CUDA(cudaEventRecord(g_gemm_ev[0], st));
  GLA_CUDA(oz_slice_rows(g_gemm_w, Ahi, Alo, lda, (int)m, (int)k, 7, st));
  GLA_CUDA(oz_slice(g_gemm_w, false, Bhi, Blo, ldb, (int)n, (int)k, 7, st));
  GLA_CUDA(cudaEventRecord(g_gemm_ev[1], st));
  GLA_CUDA(oz_gemm(g_gemm_w, (int)m, (int)n, (int)k, Chi, Clo, ldc, false, st));
  GLA_CUDA(cudaEventRecord(g_gemm_ev[2], st));
  g_gemm_timed = true;
  return 0;
}

int gla_gemm_df_last_ms(float* slice_ms, float* gemm_ms) {
  if (!slice_ms) return -1;
  if (!gemm_ms) return -2;
  std::lock_guard<std::mutex> lk(g_gemm_mu);
  *slice_ms = *gemm_ms = 0.f;
  if (!g_gemm_timed) return 0;
  GLA_CUDA(cudaEventSynchronize(g_gemm_ev[2]));
  GLA_CUDA(cudaEventElapsedTime(slice_ms, g_gemm_ev[0], g_gemm_ev[1]));
  GLA_CUDA(cudaEventElapsedTime(gemm_ms, g_gemm_ev[1], g_gemm_ev[2]));
  return 0;
}

int gla_release_workspaces(void) {
  // every cached buffer may still be in use by queued work on any stream
  GLA_CUDA(cudaDeviceSynchronize());
  {
    std::lock_guard<std::mutex> lk(g_single_mu);
    for (auto& kv : g_single) {
      gla_plan_destroy(kv.second.plan);
      cudaFree(kv.second.buf);
      cudaFree(kv.second.dinfo);
    }
    g_single.clear();
    for (auto& kv : g_stev_large) large_destroy(kv.second);
    g_stev_large.clear();
  }
  {
    std::lock_guard<std::mutex> lk(g_gemm_mu);
    if (g_gemm_w) oz_destroy(g_gemm_w);
    g_gemm_w = nullptr;
    g_gemm_timed = false;
  }
  release_eigenq_cache();
  release_complex_cache();
  release_quaternion_cache();
  GLA_CUDA(cudaGetLastError());
  return 0;
}

int gla_dstev(char jobz, int64_t n, double* d, double* e, double* Z, int64_t ldz, int flags, int* info,
              void* stream) {
  if (jobz != 'V' && jobz != 'N') return -1;
  if (n < 0 || n > GLA_MAX_N) return -2;
  if (n > GLA_MAX_SMALL_N) {  // divide and conquer
    if (!d) return -3;
    if (!e) return -4;
    if (jobz == 'V' && !Z) return -5;
    if (jobz == 'V' && ldz < n) return -6;
    if ((flags & ~3) != 0 || (flags & 3) > GLA_ALG_QR) return -7;
    if (!info) return -8;
    std::lock_guard<std::mutex> lk(g_single_mu);
    auto it = g_stev_large.find((int)n);
    if (it == g_stev_large.end()) {
      LargeCtx* c = nullptr;
      int rc = large_create(&c, (int)n, true);
      if (rc) return rc;
      it = g_stev_large.emplace((int)n, c).first;
    }
    int inf = 0;
    cudaStream_t st = (cudaStream_t)stream;
    // eigenvalues are written over d (LAPACK dstev convention, like the small path)
    int rc = large_stev(it->second, d, e, d, jobz == 'V' ? Z : nullptr, ldz, &inf, st);
    if (rc) return rc;
    *info = inf;
    return inf != 0;
  }
  if (!d && n) return -3;
  if (!e && n > 1) return -4;
  if (jobz == 'V' && !Z && n) return -5;
  if (jobz == 'V' && ldz < std::max<int64_t>(1, n)) return -6;
  if ((flags & ~3) != 0 || (flags & 3) > GLA_ALG_QR) return -7;
  if (!info) return -8;
  *info = 0;
  if (n == 0) return 0;
  std::lock_guard<std::mutex> lk(g_single_mu);
  SingleEntry* ent;
  int rc = single_entry(GLA_PREC_F64, jobz, 'L', n, flags, &ent);
  if (rc) return rc;
  gla_plan_t p = ent->plan;
  cudaStream_t st = (cudaStream_t)stream;
  double* buf = (double*)ent->buf;   // Q (n*n) | e padded (n)
  double* epad = buf + n * n;
  GLA_CUDA(cudaMemsetAsync(epad, 0, sizeof(double) * n, st));
  if (n > 1) GLA_CUDA(cudaMemcpyAsync(epad, e, sizeof(double) * (n - 1), cudaMemcpyDeviceToDevice, st));
  GLA_CUDA(cudaMemsetAsync(p->d_stats, 0, sizeof(unsigned long long) * 4, st));
  p->last_stream = st;
  GLA_CUDA(launch_init_tridiagonal(kF64, 1, st, p->d_desc, p->d_perm_bucket, d, epad, p->d_d, p->d_e, buf,
                                   ent->dinfo, p->d_cst, jobz == 'V'));
  if (jobz == 'V') {
    p->last_passes = 0;
    rc = run_passes_sync(p, 0, kF64, buf, d, ent->dinfo, nullptr, st, 0);
    if (rc) return rc;
    GLA_CUDA(cudaMemcpy2DAsync(Z, sizeof(double) * ldz, buf, sizeof(double) * n, sizeof(double) * n, n,
                               cudaMemcpyDeviceToDevice, st));
  } else {
    GLA_CUDA(launch_chase(kF64, kAlgoPWK, 1, chase_smem_bytes((int)n, 8), st, p->d_desc, p->d_perm_bucket, p->d_d,
                          p->d_e, p->d_cst, nullptr, nullptr, ent->dinfo, p->tol, kMaxSweepsPerN, p->d_pending,
                          p->d_stats));
    GLA_CUDA(launch_sort_values(kF64, 1, st, p->d_desc, p->d_perm_bucket, p->d_d, d, ent->dinfo, nullptr));
  }
  if (n > 1) GLA_CUDA(cudaMemcpyAsync(e, p->d_e, sizeof(double) * (n - 1), cudaMemcpyDeviceToDevice, st));
  GLA_CUDA(cudaMemcpyAsync(info, ent->dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  GLA_CUDA(cudaStreamSynchronize(st));
  return *info != 0;
}

}  // extern "C"

// ---------------------------------------------------------------- autotuner
//
// The launch shapes of the two batched kernels whose best shape depends on
// the order and on how many matrices share a bucket: threads per CTA of the
// tridiagonalisation (1, 2 or 4 per row of the bucket's largest order, at
// most 256) and matrices per warp of the chase (4, 8, 16 or 32 lanes).
// Plans created with GLA_FLAG_AUTOTUNE look each bucket up in a process-wide
// table keyed by (precision family, jobz, 16-wide order range, log2 of the
// bucket's matrix count); a missing entry is measured on the spot: probe
// plans of the range's largest order and the bucket's count run on
// synthetic symmetric matrices (deterministic, generated on the device),
// first one per tridiagonalisation shape, then one per chase shape with
// the best of those, each timed by its phase events (best of two after a
// warm-up). The table can be saved to and loaded from a text file.
namespace {

template <class T>
__global__ void k_tune_fill(T* A, int n, long long total) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long nn = (long long)n * n;
    const unsigned m = (unsigned)(t / nn);
    const int r = (int)(t % nn), i = r % n, j = r / n;
    const unsigned a = (unsigned)max(i, j), b = (unsigned)min(i, j);
    unsigned h = (m * 0x9E3779B1u) ^ (a * 0x85EBCA77u) ^ (b * 0xC2B2AE3Du + 0x27D4EB2Fu);
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    A[t] = (T)((double)h * (2.0 / 4294967296.0) - 1.0);
  }
}

struct TuneKey {
  int fam;  // 0: FP64 kernels, 1: FP32 kernels, 2: FP32 + refinement with the in-kernel tridiagonal solver
  char jobz;
  int range;   // orders 16 range + 1 .. 16 (range + 1)
  int cclass;  // floor(log2(matrices in the bucket))
  bool operator<(const TuneKey& o) const {
    if (fam != o.fam) return fam < o.fam;
    if (jobz != o.jobz) return jobz < o.jobz;
    if (range != o.range) return range < o.range;
    return cclass < o.cclass;
  }
};
struct TuneVal {
  int tri_mult;
  int lpw;
  float tri_ms, chase_ms;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;

constexpr int kTuneMaxCount = 2048;

// One probe configuration: best-of-two phase times after a warm-up run.
int tune_probe(int prec, char jobz, int n, int count, int base_flags, int tri_mult, int lpw, const void* A,
               void* w, void* V, int* info, float* tri_ms, float* chase_ms) {
  std::vector<int64_t> ns((size_t)count, n);
  gla_plan_t q = nullptr;
  int rc = gla_plan_create(&q, prec, jobz, 'L', count, ns.data(), 0.0, base_flags | GLA_FLAG_TIMING);
  if (rc) return rc;
  Bucket& bk = q->buckets[0];
  bk.nt_tri = std::min(256, bk.nt * tri_mult);
  bk.lpw = lpw;
  float bt = 1e30f, bc = 1e30f;
  for (int rep = 0; rep < 3 && rc >= 0; rep++) {
    rc = gla_plan_execute(q, A, w, jobz == 'V' ? V : nullptr, info, nullptr);
    if (rc < 0) break;
    float ms[GLA_NUM_PHASES];
    rc = gla_plan_phase_times(q, ms);
    if (rep > 0) {
      bt = std::min(bt, ms[GLA_PHASE_TRIDIAG]);
      bc = std::min(bc, ms[GLA_PHASE_CHASE]);
    }
  }
  gla_plan_destroy(q);
  if (rc < 0) return rc;
  *tri_ms = bt;
  *chase_ms = bc;
  return 0;
}

int tune_measure(const TuneKey& k, int count, int base_flags, TuneVal* out) {
  const int n = 16 * (k.range + 1);
  count = std::max(1, std::min(count, kTuneMaxCount));
  // family 2: FP32 + refinement with the in-kernel tridiagonal solver (its
  // tridiagonalisation kernel does the FP32 solve; FP64 input)
  const int prec = k.fam == 0 ? GLA_PREC_F64 : (k.fam == 1 ? GLA_PREC_F32 : GLA_PREC_F32_REFINED);
  const size_t el = k.fam == 1 ? 4 : 8;
  void *A = nullptr, *w = nullptr, *V = nullptr;
  int* info = nullptr;
  const long long total = (long long)count * n * n;
  cudaError_t e = cudaMalloc(&A, el * total);
  if (e == cudaSuccess) e = cudaMalloc(&V, el * total);
  if (e == cudaSuccess) e = cudaMalloc(&w, el * (size_t)count * n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&info, sizeof(int) * count);
  if (e == cudaSuccess) {
    if (k.fam != 1)
      k_tune_fill<double><<<1024, 256>>>((double*)A, n, total);
    else
      k_tune_fill<float><<<1024, 256>>>((float*)A, n, total);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int rc = e == cudaSuccess ? 0 : -1000 - (int)e;
  const int nt = std::max(32, (n + 31) / 32 * 32);
  TuneVal best{1, k.fam == 0 ? 16 : 8, 1e30f, 1e30f};
  for (int mult = 1; mult <= 4 && rc == 0; mult *= 2) {
    if (mult > 1 && nt * mult / 2 >= 256) break;  // the shape would repeat the previous one
    float t = 0, c = 0;
    rc = tune_probe(prec, k.jobz, n, count, base_flags, mult, best.lpw, A, w, V, info, &t, &c);
    if (rc == 0 && t < best.tri_ms) {
      best.tri_ms = t;
      best.tri_mult = mult;
    }
  }
  // 1 or 2 matrices per warp win a bucket's probe run alone but lose in a
  // plan, where all buckets share the SMs: a warp pays its FP64 (and most
  // FP32) issue slots for 32 lanes whatever the number active
  for (int lpw : {4, 8, 16, 32}) {
    if (rc || k.fam == 2) break;  // family 2 chases only the rare matrices its solver leaves
    float t = 0, c = 0;
    rc = tune_probe(prec, k.jobz, n, count, base_flags, best.tri_mult, lpw, A, w, V, info, &t, &c);
    if (rc == 0 && c < best.chase_ms) {
      best.chase_ms = c;
      best.lpw = lpw;
    }
  }
  cudaFree(A);
  cudaFree(V);
  cudaFree(w);
  cudaFree(info);
  if (rc) return rc;
  *out = best;
  return 0;
}

int autotune_plan(gla_plan_t p, int base_flags) {
  const int fam = p->prec == GLA_PREC_F64 ? 0 : (p->prec == GLA_PREC_F32_REFINED && p->stein ? 2 : 1);
  const char jz = p->prec == GLA_PREC_F32_REFINED ? 'V' : p->jobz;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (Bucket& bk : p->buckets) {
    int cc = 0;
    while ((2 << cc) <= bk.count && cc < 30) cc++;
    const TuneKey key{fam, jz, (bk.nmax - 1) / 16, cc};
    auto it = g_tune.find(key);
    if (it == g_tune.end()) {
      TuneVal v{};
      int rc = tune_measure(key, bk.count, base_flags, &v);
      if (rc) return rc;
      it = g_tune.emplace(key, v).first;
    }
    bk.nt_tri = std::min(256, bk.nt * it->second.tri_mult);
    bk.lpw = it->second.lpw;
  }
  return 0;
}

}  // namespace

extern "C" {

int gla_autotune_clear(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
  return 0;
}

int gla_autotune_save(const char* path) {
  if (!path) return -1;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  FILE* f = std::fopen(path, "w");
  if (!f) return -1;
  std::fprintf(f, "# glagpu autotune v1: family jobz range count_class tri_mult lanes_per_warp tri_ms chase_ms\n");
  for (const auto& kv : g_tune)
    std::fprintf(f, "%d %c %d %d %d %d %.6g %.6g\n", kv.first.fam, kv.first.jobz, kv.first.range, kv.first.cclass,
                 kv.second.tri_mult, kv.second.lpw, kv.second.tri_ms, kv.second.chase_ms);
  return std::fclose(f) == 0 ? 0 : -1;
}

int gla_autotune_load(const char* path) {
  if (!path) return -1;
  FILE* f = std::fopen(path, "r");
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  char line[256];
  int loaded = 0;
  while (std::fgets(line, sizeof line, f)) {
    if (line[0] == '#') continue;
    TuneKey k{};
    TuneVal v{};
    char jz = 0;
    if (std::sscanf(line, "%d %c %d %d %d %d %g %g", &k.fam, &jz, &k.range, &k.cclass, &v.tri_mult, &v.lpw,
                    &v.tri_ms, &v.chase_ms) != 8)
      continue;
    k.jobz = jz;
    const bool ok = (k.fam == 0 || k.fam == 1) && (jz == 'V' || jz == 'N') && k.range >= 0 &&
                    k.range < kMaxBuckets && k.cclass >= 0 && (v.tri_mult == 1 || v.tri_mult == 2 ||
                    v.tri_mult == 4) && v.lpw >= 1 && v.lpw <= 32;
    if (!ok) continue;
    g_tune[k] = v;
    loaded++;
  }
  std::fclose(f);
  return loaded;
}

int gla_plan_buckets(gla_plan_t p, int* count) {
  if (!p) return -1;
  if (!count) return -2;
  *count = (int)p->buckets.size();
  return 0;
}

int gla_plan_bucket_config(gla_plan_t p, int b, int* nmax, int* matrices, int* nt_tri, int* lanes_per_warp) {
  if (!p) return -1;
  if (b < 0 || b >= (int)p->buckets.size()) return -2;
  if (!nmax) return -3;
  if (!matrices) return -4;
  if (!nt_tri) return -5;
  if (!lanes_per_warp) return -6;
  const Bucket& bk = p->buckets[b];
  *nmax = bk.nmax;
  *matrices = bk.count;
  *nt_tri = bk.nt_tri;
  *lanes_per_warp = bk.lpw > 0 ? bk.lpw : (p->prec == GLA_PREC_F64 ? 16 : 8);
  return 0;
}

}  // extern "C"

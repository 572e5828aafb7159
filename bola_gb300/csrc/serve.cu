// serve.cu — a continuous-batching solve server (no BOLA counterpart).
//
// Requests A X = B (general or SPD, 1 <= n <= 8192, 1 <= nrhs <= 32) are
// admitted while the device bytes held by admitted requests stay within a
// budget.  Two kinds of worker thread run concurrently on one device:
//   * slots: each owns a CUDA stream and a mixed-solver context and serves
//     one large request (n > small_n) at a time — bola_dgesv_mixed_ctx in
//     mixed mode, the plain FP64 getrf/getrs (potrf/potrs for SPD) path in
//     plain mode.  Slots run at once, so their kernels share the device.
//   * the batcher: takes every admitted small request (n <= small_n) that is
//     waiting when its previous launch ends, up to max_batch, and solves them
//     in one persistent batched launch (FP64 LU / Cholesky per system).
// Every result's backward error is measured in FP64 on the device against
// the request's original A and B: by the mixed solver itself (its exact
// FP64 residual) on the mixed path, by berr_rows below on the others.  No
// request's arithmetic depends on the other requests in flight.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace bola {
namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
  int64_t id = 0, n = 0, nrhs = 0;
  int32_t kind = 0;
  const double *a = nullptr, *b = nullptr;  // caller's host buffers (column-major, ld n)
  std::vector<double> x;
  bola_request_info info{};
  int64_t bytes = 0;
  bool small = false, done = false;
};

// ---- backward error of many systems ---------------------------------------
// berr = max_c ||b_c - A x_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf).
// One CTA per 32 rows of one system: lanes are rows, the 8 warps split the
// columns of A; the per-system maxima are combined with atomicMax on the bit
// patterns of non-negative doubles (which order like the values; a NaN
// orders above +inf).
struct BerrSys {
  const double *A, *B, *X;
  int32_t n, nrhs;
};
constexpr int BERR_STRIDE = 128;  // acc per system: [0] ||A||, [1+c] r, [33+c] x, [65+c] b

__device__ __forceinline__ void max_bits(unsigned long long *p, double v) {
  atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

__global__ void __launch_bounds__(256) berr_rows(const BerrSys *__restrict__ sys, const int2 *__restrict__ jobs,
                                                 unsigned long long *__restrict__ acc) {
  __shared__ double red[8][32][9];
  const int2 job = jobs[blockIdx.x];
  const BerrSys S = sys[job.x];
  const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int64_t n = S.n, i = job.y + lane;
  const bool valid = i < n;
  unsigned long long *out = acc + (size_t)job.x * BERR_STRIDE;
  double rowsum = 0.0;
  for (int c0 = 0; c0 < S.nrhs; c0 += 8) {
    double s8[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) s8[c] = 0.0;
    for (int64_t j = g; j < n; j += 8) {
      const double a = valid ? S.A[i + j * n] : 0.0;
      if (c0 == 0) rowsum += fabs(a);
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (c0 + c < S.nrhs) s8[c] = fma(a, S.X[j + (int64_t)(c0 + c) * n], s8[c]);
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) red[g][lane][c] = s8[c];
    red[g][lane][8] = rowsum;
    __syncthreads();
    if (g == 0) {
      for (int c = 0; c < 8 && c0 + c < S.nrhs; ++c) {
        double ax = 0.0;
        for (int q = 0; q < 8; ++q) ax += red[q][lane][c];
        const int64_t k = i + (int64_t)(c0 + c) * n;
        const double res = valid ? S.B[k] - ax : 0.0;
        double r = fabs(res), xv = valid ? fabs(S.X[k]) : 0.0, bv = valid ? fabs(S.B[k]) : 0.0;
        // fmax drops a NaN operand: carry a NaN residual explicitly
        const bool bad = __any_sync(0xffffffffu, isnan(res) || isnan(xv));
        for (int off = 16; off > 0; off >>= 1) {
          r = fmax(r, __shfl_xor_sync(0xffffffffu, r, off));
          xv = fmax(xv, __shfl_xor_sync(0xffffffffu, xv, off));
          bv = fmax(bv, __shfl_xor_sync(0xffffffffu, bv, off));
        }
        if (lane == 0) {
          max_bits(out + 1 + c0 + c, bad ? __longlong_as_double(0x7ff8000000000000ll) : r);
          max_bits(out + 33 + c0 + c, xv);
          max_bits(out + 65 + c0 + c, bv);
        }
      }
      if (c0 == 0) {
        double rs = 0.0;
        for (int q = 0; q < 8; ++q) rs += red[q][lane][8];
        for (int off = 16; off > 0; off >>= 1) rs = fmax(rs, __shfl_xor_sync(0xffffffffu, rs, off));
        if (lane == 0) max_bits(out, rs);
      }
    }
    __syncthreads();
  }
}

__global__ void berr_finish(const BerrSys *__restrict__ sys, int32_t count, const unsigned long long *__restrict__ acc,
                            double *__restrict__ berr) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= count) return;
  const double *v = reinterpret_cast<const double *>(acc + (size_t)s * BERR_STRIDE);
  double e = 0.0;
  for (int c = 0; c < sys[s].nrhs; ++c) {
    const double r = v[1 + c], den = v[0] * v[33 + c] + v[65 + c];
    const double q = den > 0.0 ? r / den : (r > 0.0 ? INFINITY : 0.0);
    e = isnan(q) ? INFINITY : fmax(e, q);
  }
  berr[s] = e;
}

// Grow-only device buffer owned by one worker stream.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes, cudaStream_t s) {
    if (bytes <= cap) return 0;
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    cap = 0;
    bytes = std::max(bytes, (size_t)4096);
    BOLA_TRY_CUDA(cudaMallocAsync(&p, bytes, s));
    cap = bytes;
    return 0;
  }
  void release(cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    cap = 0;
  }
};

// Grow-only pinned host staging buffer.
struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return 0;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    bytes = std::max(bytes * 3 / 2, (size_t)1 << 20);
    BOLA_TRY_CUDA(cudaHostAlloc(&p, bytes, cudaHostAllocDefault));
    cap = bytes;
    return 0;
  }
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
};

// Backward errors of `count` systems already on the device (descriptors in
// sys_h, host) into berr_d (device); buffers from the caller's worker.
// Synchronises s (the host vectors must outlive the uploads).
int launch_berr(cudaStream_t s, const std::vector<BerrSys> &sys_h, DevBuf &dsys, DevBuf &djobs, DevBuf &dacc,
                double *berr_d) {
  const int count = (int)sys_h.size();
  std::vector<int2> jobs;
  for (int q = 0; q < count; ++q)
    for (int r = 0; r < sys_h[q].n; r += 32) jobs.push_back(make_int2(q, r));
  BOLA_TRY(dsys.ensure(sizeof(BerrSys) * count, s));
  BOLA_TRY(djobs.ensure(sizeof(int2) * jobs.size(), s));
  BOLA_TRY(dacc.ensure(sizeof(unsigned long long) * BERR_STRIDE * count, s));
  BOLA_TRY_CUDA(cudaMemcpyAsync(dsys.p, sys_h.data(), sizeof(BerrSys) * count, cudaMemcpyHostToDevice, s));
  BOLA_TRY_CUDA(cudaMemcpyAsync(djobs.p, jobs.data(), sizeof(int2) * jobs.size(), cudaMemcpyHostToDevice, s));
  BOLA_TRY_CUDA(cudaMemsetAsync(dacc.p, 0, sizeof(unsigned long long) * BERR_STRIDE * count, s));
  berr_rows<<<(unsigned)jobs.size(), 256, 0, s>>>((const BerrSys *)dsys.p, (const int2 *)djobs.p,
                                                  (unsigned long long *)dacc.p);
  berr_finish<<<(unsigned)cdiv(count, 128), 128, 0, s>>>((const BerrSys *)dsys.p, count,
                                                         (const unsigned long long *)dacc.p, berr_d);
  BOLA_CHECK_LAUNCH();
  BOLA_TRY_CUDA(cudaStreamSynchronize(s));
  return 0;
}

struct Server {
  bola_server_opts o{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req *> q_large, q_small;
  std::unordered_map<int64_t, Req *> reqs;
  int64_t bytes_in_use = 0, next_id = 1;
  int32_t running = 0;
  bool stop = false;
  double t0 = 0.0;
  std::vector<std::thread> threads;

  // Device bytes a request holds while admitted.
  int64_t footprint(const Req &r) const {
    const int64_t n = r.n, nr = r.nrhs;
    if (r.small) return 16 * n * n + 16 * n * nr + 1024;
    if (o.mode == 1) return 16 * n * n + 16 * n * nr + 64 * n + 1024;
    // A, B, X; the FP32 working matrix, tensor-core operands, GMRES basis
    // (2 x 25 vectors per right-hand side) and the FP64 fallback copy
    return 8 * n * n + 24 * n * nr + 4 * n * n + 2 * 4 * 64 * n + 8 * 64 * n + 400 * n * nr + 8 * n * n + 4096;
  }

  bool fits(const Req *r) const { return bytes_in_use + r->bytes <= o.hbm_budget_bytes; }

  void finish(Req *r) {
    std::lock_guard<std::mutex> lk(mu);
    bytes_in_use -= r->bytes;
    running -= 1;
    r->info.t_done = now_s() - t0;
    if (r->info.status >= 0) r->info.status = 2;
    r->done = true;
    cv_done.notify_all();
    cv_work.notify_all();
  }

  void slot_loop() {
    cudaSetDevice(device);
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    bola_mixed_ctx ctx = nullptr;
    bola_mixed_ctx_create(&ctx);
    DevBuf dsys, djobs, dacc, dberr;
    for (;;) {
      Req *r = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return (stop && q_large.empty()) || (!q_large.empty() && fits(q_large.front())); });
        if (q_large.empty()) break;
        r = q_large.front();
        q_large.pop_front();
        bytes_in_use += r->bytes;
        running += 1;
        r->info.status = 1;
        r->info.t_admit = now_s() - t0;
      }
      const int st = serve_large(r, s, ctx, dsys, djobs, dacc, dberr);
      if (st != 0) r->info.status = st;
      finish(r);
    }
    for (DevBuf *b : {&dsys, &djobs, &dacc, &dberr}) b->release(s);
    cudaStreamSynchronize(s);
    bola_mixed_ctx_destroy(ctx);
    cudaStreamDestroy(s);
  }

  int serve_large(Req *r, cudaStream_t s, bola_mixed_ctx ctx, DevBuf &dsys, DevBuf &djobs, DevBuf &dacc,
                  DevBuf &dberr) {
    double *A = nullptr, *B = nullptr, *X = nullptr, *W = nullptr;
    int32_t *ipiv = nullptr, *dinfo = nullptr;
    r->x.resize((size_t)r->n * r->nrhs);
    int st = solve_large(r, s, ctx, dsys, djobs, dacc, dberr, A, B, X, W, ipiv, dinfo);
    for (void *p : {(void *)A, (void *)B, (void *)X, (void *)W, (void *)ipiv, (void *)dinfo})
      if (p) cudaFreeAsync(p, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (st == 0 && e != cudaSuccess) st = cuda_fail(e, "bola_server");
    return st;
  }

  // The solve proper; the buffers it allocates are returned through the
  // references so that serve_large frees them on every exit.
  int solve_large(Req *r, cudaStream_t s, bola_mixed_ctx ctx, DevBuf &dsys, DevBuf &djobs, DevBuf &dacc,
                  DevBuf &dberr, double *&A, double *&B, double *&X, double *&W, int32_t *&ipiv, int32_t *&dinfo) {
    const int64_t n = r->n, nr = r->nrhs;
    const size_t an = sizeof(double) * n * n, bn = sizeof(double) * n * nr;
    BOLA_TRY_CUDA(cudaMallocAsync(&A, an, s));
    BOLA_TRY_CUDA(cudaMallocAsync(&B, bn, s));
    BOLA_TRY_CUDA(cudaMallocAsync(&X, bn, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(A, r->a, an, cudaMemcpyHostToDevice, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(B, r->b, bn, cudaMemcpyHostToDevice, s));
    if (o.mode == 0) {
      // SPD requests (kind 1) take the mixed Cholesky, the others the mixed LU
      bola_mixed_opts mo = {o.factor_kind, 30, 1e-14, 1, 1, 1};
      bola_mixed_info mi{};
      if (r->kind == 1)
        BOLA_TRY(bola_dposv_mixed_ctx(ctx, n, nr, A, n, B, n, X, n, &mo, &mi, (bola_stream_t)s));
      else
        BOLA_TRY(bola_dgesv_mixed_ctx(ctx, n, nr, A, n, B, n, X, n, &mo, &mi, (bola_stream_t)s));
      r->info.factorization = mi.factorization;
      r->info.path = mi.path == 3 ? 4 : mi.path;  // (3 is the batched path here)
      r->info.iterations = mi.iterations;
      r->info.info = mi.factor_info;
      r->info.backward_error = mi.backward_error;
      BOLA_TRY_CUDA(cudaMemcpyAsync(r->x.data(), X, bn, cudaMemcpyDeviceToHost, s));
      return 0;
    }
    // the plain FP64 per-request path: BOLA-exact factorisation and solve
    BOLA_TRY_CUDA(cudaMallocAsync(&W, an, s));
    BOLA_TRY_CUDA(cudaMallocAsync(&ipiv, sizeof(int32_t) * n, s));
    BOLA_TRY_CUDA(cudaMallocAsync(&dinfo, sizeof(int32_t), s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(W, A, an, cudaMemcpyDeviceToDevice, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(X, B, bn, cudaMemcpyDeviceToDevice, s));
    if (r->kind == 1) {
      BOLA_TRY(bola_dpotrf('L', n, W, n, dinfo, (bola_stream_t)s));
      BOLA_TRY(bola_dpotrs('L', n, nr, W, n, X, n, (bola_stream_t)s));
    } else {
      BOLA_TRY(bola_dgetrf(n, n, W, n, ipiv, dinfo, (bola_stream_t)s));
      BOLA_TRY(bola_dgetrs(n, nr, W, n, ipiv, X, n, (bola_stream_t)s));
    }
    std::vector<BerrSys> one = {BerrSys{A, B, X, (int32_t)n, (int32_t)nr}};
    BOLA_TRY(dberr.ensure(sizeof(double), s));
    BOLA_TRY(launch_berr(s, one, dsys, djobs, dacc, (double *)dberr.p));
    int32_t hinfo = 0;
    BOLA_TRY_CUDA(cudaMemcpyAsync(&hinfo, dinfo, sizeof hinfo, cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(&r->info.backward_error, dberr.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(r->x.data(), X, bn, cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaStreamSynchronize(s));
    r->info.info = hinfo;
    r->info.path = 2;
    r->info.factorization = r->kind == 1 ? 1 : 0;
    return 0;
  }

  void batch_loop() {
    cudaSetDevice(device);
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    DevBuf data, desc, items, counter, info, berr, dsys, djobs, dacc;
    HostBuf stage;
    for (;;) {
      std::vector<Req *> take;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return (stop && q_small.empty()) || (!q_small.empty() && fits(q_small.front())); });
        if (q_small.empty()) break;
        while (!q_small.empty() && (int)take.size() < o.max_batch && fits(q_small.front())) {
          Req *r = q_small.front();
          q_small.pop_front();
          bytes_in_use += r->bytes;
          running += 1;
          r->info.status = 1;
          r->info.t_admit = now_s() - t0;
          take.push_back(r);
        }
      }
      const int st = serve_batch(take, s, data, desc, items, counter, info, berr, dsys, djobs, dacc, stage);
      for (Req *r : take) {
        if (st != 0) r->info.status = st;
        finish(r);
      }
    }
    for (DevBuf *b : {&data, &desc, &items, &counter, &info, &berr, &dsys, &djobs, &dacc}) b->release(s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }

  // Layout of one batch in `data`: A0 (originals) | A (factored) | B0 | X.
  int serve_batch(std::vector<Req *> &take, cudaStream_t s, DevBuf &data, DevBuf &desc, DevBuf &items,
                  DevBuf &counter, DevBuf &info, DevBuf &berr, DevBuf &dsys, DevBuf &djobs, DevBuf &dacc,
                  HostBuf &stage) {
    const int cnt = (int)take.size();
    std::vector<int64_t> aoff(cnt + 1, 0), boff(cnt + 1, 0);
    std::vector<int32_t> ns(cnt), kinds(cnt);
    for (int i = 0; i < cnt; ++i) {
      aoff[i + 1] = aoff[i] + take[i]->n * take[i]->n;
      boff[i + 1] = boff[i] + take[i]->n * take[i]->nrhs;
      ns[i] = (int32_t)take[i]->n;
      kinds[i] = take[i]->kind;
    }
    const int64_t na = aoff[cnt], nb = boff[cnt];
    std::vector<int32_t> flat;
    int32_t nitems = 0;
    int group[8];
    BOLA_TRY(batch_items(cnt, ns.data(), kinds.data(), o.group_size[0] ? o.group_size : nullptr, flat, &nitems, group,
                         nullptr, o.panel_width[0] ? o.panel_width : nullptr));
    BOLA_TRY(data.ensure(sizeof(double) * (2 * na + 2 * nb), s));
    BOLA_TRY(desc.ensure(sizeof(bola_system) * cnt, s));
    BOLA_TRY(items.ensure(sizeof(int32_t) * flat.size(), s));
    BOLA_TRY(counter.ensure(sizeof(int32_t), s));
    BOLA_TRY(info.ensure(sizeof(int32_t) * cnt, s));
    BOLA_TRY(berr.ensure(sizeof(double) * cnt, s));
    double *A0 = (double *)data.p, *A = A0 + na, *B0 = A + na, *X = B0 + nb;
    // gather the inputs, descriptors and work items into one pinned buffer
    const size_t desc_bytes = sizeof(bola_system) * cnt;
    BOLA_TRY(stage.ensure(sizeof(double) * (na + nb) + desc_bytes + sizeof(int32_t) * flat.size()));
    double *h = (double *)stage.p;
    std::vector<BerrSys> bs(cnt);
    bola_system *hd = (bola_system *)(h + na + nb);
    for (int i = 0; i < cnt; ++i) {
      const Req *r = take[i];
      std::memcpy(h + aoff[i], r->a, sizeof(double) * r->n * r->n);
      std::memcpy(h + na + boff[i], r->b, sizeof(double) * r->n * r->nrhs);
      hd[i] = bola_system{(int32_t)r->n, (int32_t)r->nrhs, r->kind, (int32_t)r->n, (int32_t)r->n, 0, A + aoff[i],
                          X + boff[i]};
      bs[i] = BerrSys{A0 + aoff[i], B0 + boff[i], X + boff[i], (int32_t)r->n, (int32_t)r->nrhs};
    }
    std::memcpy((char *)hd + desc_bytes, flat.data(), sizeof(int32_t) * flat.size());
    BOLA_TRY_CUDA(cudaMemcpyAsync(A0, h, sizeof(double) * na, cudaMemcpyHostToDevice, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(B0, h + na, sizeof(double) * nb, cudaMemcpyHostToDevice, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(desc.p, hd, desc_bytes, cudaMemcpyHostToDevice, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(items.p, (char *)hd + desc_bytes, sizeof(int32_t) * flat.size(),
                                  cudaMemcpyHostToDevice, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(A, A0, sizeof(double) * na, cudaMemcpyDeviceToDevice, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(X, B0, sizeof(double) * nb, cudaMemcpyDeviceToDevice, s));
    BOLA_TRY(batch_launch(s, (const bola_system *)desc.p, (const int32_t *)items.p, nitems, (int32_t *)counter.p,
                          (int32_t *)info.p, o.tile_rows == 2 ? 2 : 4));
    BOLA_TRY(launch_berr(s, bs, dsys, djobs, dacc, (double *)berr.p));  // synchronises s
    // results back through the same staging buffer
    std::vector<double> hb(cnt);
    std::vector<int32_t> hi(cnt);
    BOLA_TRY_CUDA(cudaMemcpyAsync(h, X, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(hb.data(), berr.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaMemcpyAsync(hi.data(), info.p, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, s));
    BOLA_TRY_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < cnt; ++i) {
      Req *r = take[i];
      r->x.assign(h + boff[i], h + boff[i + 1]);
      r->info.backward_error = hb[i];
      r->info.info = hi[i];
      r->info.path = 3;
      r->info.factorization = r->kind;
    }
    return 0;
  }
};

}  // namespace
}  // namespace bola

using namespace bola;

extern "C" {

int bola_server_create(const bola_server_opts *opts, bola_server *out) {
  if (!opts || !out) return fail(-1, "bola_server_create: null argument");
  if (opts->hbm_budget_bytes <= 0) return fail(-1, "bola_server_create: hbm_budget_bytes must be positive");
  if (opts->mode != 0 && opts->mode != 1) return fail(-1, "bola_server_create: mode must be 0 or 1");
  Server *S = new Server();
  S->o = *opts;
  if (S->o.slots < 1) S->o.slots = 1;
  if (S->o.max_batch < 1) S->o.max_batch = 256;
  S->o.small_n = std::max(0, std::min(256, S->o.small_n));
  if (cudaGetDevice(&S->device) != cudaSuccess) {
    delete S;
    return fail(BOLA_ERR_CUDA, "bola_server_create: no CUDA device");
  }
  // keep freed stream-ordered memory in the device's pool between requests
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  S->t0 = now_s();
  for (int i = 0; i < S->o.slots; ++i) S->threads.emplace_back([S] { S->slot_loop(); });
  S->threads.emplace_back([S] { S->batch_loop(); });
  *out = reinterpret_cast<bola_server>(S);
  return 0;
}

int bola_server_submit(bola_server srv, int64_t n, int64_t nrhs, int32_t kind, const double *a, const double *b,
                       int64_t *id) {
  Server *S = reinterpret_cast<Server *>(srv);
  if (!S || !a || !b || !id) return fail(-1, "bola_server_submit: null argument");
  if (n < 1 || n > 8192) return fail(-2, "bola_server_submit: n = %lld (supported 1..8192)", (long long)n);
  if (nrhs < 1 || nrhs > 32) return fail(-3, "bola_server_submit: nrhs = %lld (supported 1..32)", (long long)nrhs);
  if (kind != 0 && kind != 1) return fail(-4, "bola_server_submit: kind must be 0 or 1");
  Req *r = new Req();
  r->n = n;
  r->nrhs = nrhs;
  r->kind = kind;
  r->a = a;
  r->b = b;
  r->small = n <= S->o.small_n;
  r->bytes = S->footprint(*r);
  if (r->bytes > S->o.hbm_budget_bytes) {
    const long long need = (long long)r->bytes;
    delete r;
    return fail(-5, "bola_server_submit: request needs %lld device bytes, over the budget", need);
  }
  std::lock_guard<std::mutex> lk(S->mu);
  r->id = S->next_id++;
  r->info.t_submit = now_s() - S->t0;
  S->reqs[r->id] = r;
  (r->small ? S->q_small : S->q_large).push_back(r);
  S->cv_work.notify_all();
  *id = r->id;
  return 0;
}

int bola_server_wait(bola_server srv, int64_t id, double *x, bola_request_info *info) {
  Server *S = reinterpret_cast<Server *>(srv);
  if (!S) return fail(-1, "bola_server_wait: null server");
  Req *r = nullptr;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return fail(-2, "bola_server_wait: unknown request %lld", (long long)id);
    r = it->second;
    S->cv_done.wait(lk, [&] { return r->done; });
    S->reqs.erase(it);
  }
  if (x && !r->x.empty()) std::memcpy(x, r->x.data(), sizeof(double) * r->x.size());
  if (info) *info = r->info;
  const int st = r->info.status < 0 ? r->info.status : 0;
  delete r;
  return st;
}

int bola_server_stats(bola_server srv, int64_t *bytes_in_use, int32_t *pending, int32_t *running) {
  Server *S = reinterpret_cast<Server *>(srv);
  if (!S) return fail(-1, "bola_server_stats: null server");
  std::lock_guard<std::mutex> lk(S->mu);
  if (bytes_in_use) *bytes_in_use = S->bytes_in_use;
  if (pending) *pending = (int32_t)(S->q_large.size() + S->q_small.size());
  if (running) *running = S->running;
  return 0;
}

int bola_server_destroy(bola_server srv) {
  Server *S = reinterpret_cast<Server *>(srv);
  if (!S) return 0;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv_work.notify_all();
  }
  for (auto &t : S->threads) t.join();
  for (auto &kv : S->reqs) delete kv.second;
  delete S;
  return 0;
}

}  // extern "C"

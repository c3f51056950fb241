// The reference's estimator formulas on the device, each as ONE batch (as
// several for a job larger than one batch holds).
//
// The reference's estimator mains loop over columns / pairs, call
// combined_densities() once per density (each a separate device allocation,
// upload and download, densities_cuda.cu:16-105) and reduce on the host:
//   Mi::main        mi.cpp:37-59        sum_k p_ij log(p_ij / p_i / p_j)
//   Transs::main    transs.cpp:39-115   TE weights h_i h_i h_j (and the mirrored
//                                       h_i h_j h_i), skipped non-finite terms
//   AutoEnt::main   autoent.cpp:39-58   sum_k p_i_itau h h log(p_itau / (p_i_itau h))
//   Negs::main      negs.cpp:36-47      -sum_k p~ log p~, p~ = sum1_normalized(p)
//   KLDiv::main     kldiv.cpp:36-54     sum_k p~_i log(p~_i / p~_j)
//   Dens            dens.cpp:19-106     sum1_normalized densities of every
//                                       column, pair or triple
// Here every density of an estimator is one instance of a single engine batch
// (one persistent pair-kernel launch per dimension) writing its per-point
// FP64 densities into HBM; marginals are computed once, not once per pair
// (mi.cpp:43-46 recomputes p_j for every i). The sums run on the device in
// FP64, one block per output in a fixed order (deterministic). Each term
// keeps the reference's arithmetic: densities normalised by the original
// n_rows (densities_cuda.cu:98-103), the float log returning 0 at 0
// (tools.cpp:18-37), Tools::inv (tools.hxx:45-53), the double products in
// the reference's order; only the accumulators differ (FP64 here, float in
// mi.cpp and negs.cpp), so results agree with the reference to its float
// precision.
#include <algorithm>
#include <cmath>
#include <map>
#include <utility>
#include <vector>

#include "../../include/entropical_gb300.h"
#include "api_internal.h"
#include "engine.h"

using namespace ent;

namespace {

enum : uint32_t { RT_MI = 1, RT_TE = 2, RT_AUTOENT = 3, RT_NEGS = 4, RT_KL = 5 };

// One output sum over k < n of a term of up to four per-point densities.
struct RefTerm {
  const double* a;
  const double* b;
  const double* c;
  const double* e;
  uint32_t sa, sb;  // index of the sum1 divisor of a / b in `sums` (~0u: none)
  double w1, w2, w3;
  uint32_t n;
  uint32_t kind;
  uint32_t slot;
  uint32_t pad;
};

__device__ __forceinline__ float flog(float x) { return x == 0.f ? 0.f : logf(x); }
__device__ __forceinline__ double dinv(double x) { return x == 0.0 ? x : 1.0 / x; }

template <int NT>
__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < NT / 32; ++i) t += sh[i];
  __syncthreads();
  return t;
}

// Per-array FP64 sums (the divisors of sum1_normalized, tools.hxx:33-43).
__global__ void __launch_bounds__(256)
    k_array_sums(const double* const* __restrict__ arrays, const uint32_t* __restrict__ lens,
                 double* __restrict__ sums) {
  __shared__ double sh[8];
  const double* x = arrays[blockIdx.x];
  const uint32_t n = lens[blockIdx.x];
  double a = 0.0;
  for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) a += x[k];
  const double t = block_sum<256>(a, sh);
  if (threadIdx.x == 0) sums[blockIdx.x] = t;
}

// x[k] /= sum, for every array (rows of one contiguous matrix).
__global__ void k_divide_rows(double* __restrict__ x, uint32_t n, const double* __restrict__ sums) {
  const uint32_t row = blockIdx.y;
  const double s = sums[row];
  if (s == 0.0) return;
  double* r = x + (size_t)row * n;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    r[k] /= s;
}

__global__ void __launch_bounds__(256)
    k_ref_terms(const RefTerm* __restrict__ terms, const double* __restrict__ sums,
                double* __restrict__ out) {
  __shared__ double sh[8];
  const RefTerm t = terms[blockIdx.x];
  const double da = t.sa != ~0u ? sums[t.sa] : 1.0;
  const double db = t.sb != ~0u ? sums[t.sb] : 1.0;
  double acc = 0.0;
  for (uint32_t k = threadIdx.x; k < t.n; k += blockDim.x) {
    switch (t.kind) {
      case RT_MI: {  // mi.cpp:54
        const double pij = t.a[k];
        acc += pij * (double)flog((float)(pij / t.b[k] / t.c[k]));
        break;
      }
      case RT_TE: {  // transs.cpp:76-104
        const double p3 = t.a[k];
        if (p3 > 0) {
          const double arg = p3 * t.b[k] * dinv(t.c[k]) * dinv(t.e[k]);
          const double te = p3 * t.w1 * t.w2 * t.w3 * (double)flog((float)arg);
          if (isfinite(te) && p3 <= 1.0) acc += te;
        }
        break;
      }
      case RT_AUTOENT: {  // autoent.cpp:51-55
        const double p2 = t.a[k];
        if (p2 > 0) acc += p2 * t.w1 * t.w1 * (double)flog((float)(t.b[k] * dinv(p2 * t.w1)));
        break;
      }
      case RT_NEGS: {  // negs.cpp:43-44, p already sum1-normalised by da
        const double p = da != 0.0 ? t.a[k] / da : t.a[k];
        acc += (double)flog((float)p) * p;
        break;
      }
      case RT_KL: {  // kldiv.cpp:49-50
        const double pi = da != 0.0 ? t.a[k] / da : t.a[k];
        const double pj = db != 0.0 ? t.b[k] / db : t.b[k];
        acc += pi * (double)flog((float)(pi / pj));
        break;
      }
    }
  }
  const double s = block_sum<256>(acc, sh);
  if (threadIdx.x == 0) out[t.slot] = s;
}

// Views of the coordinate columns, deduplicated by (column, lag, length).
struct ViewTable {
  const float* dc;
  size_t n_rows;
  std::vector<ViewSpec> views;
  std::map<std::pair<uint64_t, uint32_t>, uint32_t> index;
  uint32_t get(size_t col, uint32_t lag, uint32_t n) {
    const uint64_t key = (uint64_t)col * n_rows + lag;
    auto it = index.find({key, n});
    if (it != index.end()) return it->second;
    const uint32_t v = (uint32_t)views.size();
    views.push_back({dc + col * n_rows + lag, n});
    index[{key, n}] = v;
    return v;
  }
};

struct Batch {
  Ctx& c;
  ViewTable vt;
  std::vector<InstSpec> insts;
  std::vector<size_t> out_off;  // element offset of each instance's densities
  size_t total = 0;
  double* dens = nullptr;  // device, all instances back to back
  Batch(Ctx& cc, const float* dc, size_t n_rows) : c(cc) {
    vt.dc = dc;
    vt.n_rows = n_rows;
  }
  // density of d lagged columns, normalised by n_rows; returns its index
  // s3: d = 3 cells per bandwidth along dimensions 1 and 2 (0: the context's)
  uint32_t add(uint32_t d, const size_t* cols, const uint32_t* lags, const float* h,
               uint32_t s3a = 0, uint32_t s3b = 0) {
    uint32_t mx = 0;
    for (uint32_t j = 0; j < d; ++j) mx = std::max(mx, lags[j]);
    const uint32_t n = (uint32_t)(vt.n_rows - mx);
    InstSpec I;
    I.d = d;
    I.n = n;
    for (uint32_t j = 0; j < d; ++j) {
      I.view[j] = vt.get(cols[j], lags[j], n);
      I.h[j] = h[j];
    }
    I.norm = (double)vt.n_rows;
    I.S = c.strip_subdiv;
    I.S3[0] = s3a;
    I.S3[1] = s3b;
    insts.push_back(I);
    out_off.push_back(total);
    total += n;
    return (uint32_t)insts.size() - 1;
  }
  const double* ptr(uint32_t i) const { return dens + out_off[i]; }
  int run() {
    dens = static_cast<double*>(c.arena.alloc(sizeof(double) * std::max<size_t>(total, 1)));
    if (!dens) return c.fail(ENT_ERR_CUDA, "out of device memory");
    for (size_t i = 0; i < insts.size(); ++i) insts[i].out = dens + out_off[i];
    return run_engine_batches(c, vt.views, insts, DM_WRITE_F64, nullptr, nullptr);
  }
};

template <class T>
T* upload(Ctx& c, const std::vector<T>& v, int* status) {
  T* p = static_cast<T*>(c.arena.alloc(sizeof(T) * std::max<size_t>(v.size(), 1)));
  if (!p) {
    *status = c.fail(ENT_ERR_CUDA, "out of device memory");
    return nullptr;
  }
  cudaError_t e = cudaMemcpyAsync(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice,
                                  c.stream);
  if (e != cudaSuccess) {
    *status = c.cuda_fail(e, "upload");
    return nullptr;
  }
  return p;
}

// FP64 sums of the given instances' densities (device array, one per entry).
int instance_sums(Batch& B, const std::vector<uint32_t>& which, double** d_sums) {
  Ctx& c = B.c;
  int s = ENT_OK;
  std::vector<const double*> arrs;
  std::vector<uint32_t> lens;
  for (uint32_t i : which) {
    arrs.push_back(B.ptr(i));
    lens.push_back(B.insts[i].n);
  }
  const double* const* da = upload(c, arrs, &s);
  if (!da) return s;
  const uint32_t* dl = upload(c, lens, &s);
  if (!dl) return s;
  *d_sums = static_cast<double*>(c.arena.alloc(sizeof(double) * std::max<size_t>(which.size(), 1)));
  if (!*d_sums) return c.fail(ENT_ERR_CUDA, "out of device memory");
  if (!which.empty()) {
    k_array_sums<<<(unsigned)which.size(), 256, 0, c.stream>>>(da, dl, *d_sums);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c.cuda_fail(e, "array sums");
    c.stats.kernel_launches += 1;
  }
  return ENT_OK;
}

int run_terms(Ctx& c, const std::vector<RefTerm>& terms, const double* d_sums, size_t n_slots,
              std::vector<double>* out) {
  int s = ENT_OK;
  out->assign(n_slots, 0.0);
  if (terms.empty()) return ENT_OK;
  const RefTerm* dt = upload(c, terms, &s);
  if (!dt) return s;
  double* dout = static_cast<double*>(c.arena.alloc(sizeof(double) * n_slots));
  if (!dout) return c.fail(ENT_ERR_CUDA, "out of device memory");
  cudaError_t e = cudaMemsetAsync(dout, 0, sizeof(double) * n_slots, c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "memset");
  k_ref_terms<<<(unsigned)terms.size(), 256, 0, c.stream>>>(dt, d_sums, dout);
  e = cudaGetLastError();
  if (e != cudaSuccess) return c.cuda_fail(e, "estimator sums");
  c.stats.kernel_launches += 1;
  e = cudaMemcpyAsync(out->data(), dout, sizeof(double) * n_slots, cudaMemcpyDeviceToHost,
                      c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "read sums");
  return ENT_OK;
}

RefTerm term(uint32_t kind, uint32_t slot, uint32_t n, const double* a, const double* b = nullptr,
             const double* cc = nullptr, const double* e = nullptr) {
  RefTerm t{};
  t.a = a;
  t.b = b;
  t.c = cc;
  t.e = e;
  t.sa = t.sb = ~0u;
  t.w1 = t.w2 = t.w3 = 1.0;
  t.n = n;
  t.kind = kind;
  t.slot = slot;
  return t;
}

int common_checks(Ctx& c, const float* coords, size_t n_rows, size_t n_cols, const float* h,
                  void* out) {
  if (!coords || !h || !out) return c.fail(ENT_ERR_ARG, "null argument");
  if (n_cols < 1 || n_rows < 1) return c.fail(ENT_ERR_ARG, "empty input");
  if (n_rows > 0xffffff00ull) return c.fail(ENT_ERR_TOO_LARGE, "too many rows");
  for (size_t j = 0; j < n_cols; ++j)
    if (!(h[j] > 0.f) || !std::isfinite(h[j]))
      return c.fail(ENT_ERR_ARG, "bandwidth must be finite and positive");
  return ENT_OK;
}

const float* device_coords(Ctx& c, const float* coords, size_t n_rows, size_t n_cols,
                           uint32_t flags, int* s) {
  if (flags & ENT_BATCH_DEVICE_INPUT) return coords;
  float* p = static_cast<float*>(c.arena.alloc(4 * n_rows * n_cols));
  if (!p) {
    *s = c.fail(ENT_ERR_CUDA, "out of device memory");
    return nullptr;
  }
  cudaError_t e = cudaMemcpyAsync(p, coords, 4 * n_rows * n_cols, cudaMemcpyHostToDevice,
                                  c.stream);
  if (e != cudaSuccess) {
    *s = c.cuda_fail(e, "copy coordinates");
    return nullptr;
  }
  return p;
}

}  // namespace

extern "C" {

int ent_reference_estimator(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols,
                            const float* h, uint32_t estimator, uint32_t tau, uint32_t flags,
                            double* out) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if ((s = common_checks(c, coords, n_rows, n_cols, h, out))) return s;
  if (estimator < ENT_REF_MI || estimator > ENT_REF_KLDIV)
    return c.fail(ENT_ERR_ARG, "unknown estimator");
  const bool lagged = estimator == ENT_REF_TRANSS || estimator == ENT_REF_AUTOENT;
  if (lagged && (size_t)tau >= n_rows) return c.fail(ENT_ERR_ARG, "lag >= n_rows");
  const float* dc = device_coords(c, coords, n_rows, n_cols, flags, &s);
  if (!dc) return s;
  const size_t M = n_cols;
  const uint32_t m = lagged ? (uint32_t)(n_rows - tau) : (uint32_t)n_rows;
  Batch B(c, dc, n_rows);
  const uint32_t z[3] = {0, 0, 0};
  std::vector<uint32_t> p1(M), p2(M);
  std::vector<uint32_t> pij(M * M, 0), p3a(M * M, 0), p3b(M * M, 0);
  // densities, as the reference's mains request them (marginals once)
  for (size_t i = 0; i < M; ++i) {
    if (estimator == ENT_REF_AUTOENT) {
      const uint32_t lt[1] = {tau};
      p1[i] = B.add(1, &i, lt, &h[i]);  // p_itau: x_i[t + tau]
      const size_t cc[2] = {i, i};
      const uint32_t lg[2] = {0, tau};
      const float hh[2] = {h[i], h[i]};
      p2[i] = B.add(2, cc, lg, hh);  // p_i_itau
    } else {
      p1[i] = B.add(1, &i, z, &h[i]);
      if (estimator == ENT_REF_TRANSS) {
        const size_t cc[2] = {i, i};
        const uint32_t lg[2] = {0, tau};
        const float hh[2] = {h[i], h[i]};
        p2[i] = B.add(2, cc, lg, hh);  // p_tau[i]
      }
    }
  }
  if (estimator == ENT_REF_MI || estimator == ENT_REF_TRANSS)
    for (size_t i = 0; i < M; ++i)
      for (size_t j = i + 1; j < M; ++j) {
        const size_t cc[2] = {i, j};
        const float hh[2] = {h[i], h[j]};
        pij[i * M + j] = B.add(2, cc, z, hh);
        if (estimator == ENT_REF_TRANSS) {
          // the density of (x_i, x_i+tau, x_j) as (x_j, x_i, x_i+tau): the
          // independent coordinate sorted, cells of h and h/2 in the two
          // that follow each other (the order the TE batch measured fastest)
          const size_t ca[3] = {j, i, i};
          const uint32_t la[3] = {0, 0, tau};
          const float ha[3] = {h[j], h[i], h[i]};
          p3a[i * M + j] = B.add(3, ca, la, ha, 1, 2);  // p_ij_itau
          const size_t cb[3] = {i, j, j};
          const uint32_t lb[3] = {0, 0, tau};
          const float hb[3] = {h[i], h[j], h[j]};
          // (x_i, x_j, x_j+tau): dimension 2 follows dimension 1
          p3b[i * M + j] = B.add(3, cb, lb, hb, 2, 1);  // p_ij_jtau
        }
      }
  if ((s = B.run())) return s;

  double* d_sums = nullptr;
  if (estimator == ENT_REF_NEGS || estimator == ENT_REF_KLDIV) {
    if ((s = instance_sums(B, p1, &d_sums))) return s;
  }
  std::vector<RefTerm> terms;
  size_t n_slots = (estimator == ENT_REF_NEGS || estimator == ENT_REF_AUTOENT) ? M : M * M;
  for (size_t i = 0; i < M; ++i) {
    if (estimator == ENT_REF_NEGS) {
      RefTerm t = term(RT_NEGS, (uint32_t)i, (uint32_t)n_rows, B.ptr(p1[i]));
      t.sa = (uint32_t)i;
      terms.push_back(t);
    } else if (estimator == ENT_REF_AUTOENT) {
      RefTerm t = term(RT_AUTOENT, (uint32_t)i, m, B.ptr(p2[i]), B.ptr(p1[i]));
      t.w1 = (double)h[i];
      terms.push_back(t);
    }
    for (size_t j = i + 1; j < M; ++j) {
      const uint32_t ij = (uint32_t)(i * M + j), ji = (uint32_t)(j * M + i);
      if (estimator == ENT_REF_MI) {
        terms.push_back(term(RT_MI, ij, (uint32_t)n_rows, B.ptr(pij[ij]), B.ptr(p1[i]),
                             B.ptr(p1[j])));
      } else if (estimator == ENT_REF_KLDIV) {
        RefTerm t = term(RT_KL, ij, (uint32_t)n_rows, B.ptr(p1[i]), B.ptr(p1[j]));
        t.sa = (uint32_t)i;
        t.sb = (uint32_t)j;
        terms.push_back(t);
        RefTerm u = term(RT_KL, ji, (uint32_t)n_rows, B.ptr(p1[j]), B.ptr(p1[i]));
        u.sa = (uint32_t)j;
        u.sb = (uint32_t)i;
        terms.push_back(u);
      } else if (estimator == ENT_REF_TRANSS) {
        RefTerm t = term(RT_TE, ij, m, B.ptr(p3a[ij]), B.ptr(p1[i]), B.ptr(pij[ij]),
                         B.ptr(p2[i]));
        t.w1 = (double)h[i];
        t.w2 = (double)h[i];
        t.w3 = (double)h[j];
        terms.push_back(t);
        RefTerm u = term(RT_TE, ji, m, B.ptr(p3b[ij]), B.ptr(p1[j]), B.ptr(pij[ij]),
                         B.ptr(p2[j]));
        u.w1 = (double)h[i];
        u.w2 = (double)h[j];
        u.w3 = (double)h[i];
        terms.push_back(u);
      }
    }
  }
  std::vector<double> sums;
  if ((s = run_terms(c, terms, d_sums, n_slots, &sums))) return s;
  s = c.end_call();
  c.collect_kernel_stats();
  if (s) return s;
  if (estimator == ENT_REF_NEGS) {
    for (size_t i = 0; i < M; ++i) out[i] = -sums[i];
  } else if (estimator == ENT_REF_AUTOENT) {
    for (size_t i = 0; i < M; ++i) out[i] = sums[i];
  } else {
    for (size_t i = 0; i < M * M; ++i) out[i] = sums[i];
    if (estimator == ENT_REF_MI)
      for (size_t i = 0; i < M; ++i)
        for (size_t j = i + 1; j < M; ++j) out[j * M + i] = out[i * M + j];
  }
  return ENT_OK;
}

int ent_dens_all(ent_ctx* ctx, const float* coords, size_t n_rows, size_t n_cols,
                 const float* h, uint32_t dims, const uint32_t* taus, uint32_t flags,
                 double* out, size_t* n_inst_out, size_t* n_sel_out) {
  if (!ctx) return ENT_ERR_ARG;
  Ctx& c = *reinterpret_cast<Ctx*>(ctx);
  int s = c.begin_call();
  if (s) return s;
  if ((s = common_checks(c, coords, n_rows, n_cols, h, out))) return s;
  if (dims < 1 || dims > 3) return c.fail(ENT_ERR_DIM, "dims must be 1, 2 or 3");
  uint32_t lag[3] = {0, 0, 0}, mx = 0;
  if (taus && dims > 1)
    for (uint32_t j = 0; j < dims; ++j) {
      lag[j] = taus[j];
      mx = std::max(mx, lag[j]);
    }
  if ((size_t)mx >= n_rows) return c.fail(ENT_ERR_ARG, "lag >= n_rows");
  const size_t M = n_cols;
  size_t n_inst = dims == 1 ? M : (dims == 2 ? M * (M - 1) / 2 : M * (M - 1) * (M - 2) / 6);
  const size_t n_sel = n_rows - mx;
  if (n_inst_out) *n_inst_out = n_inst;
  if (n_sel_out) *n_sel_out = n_sel;
  if (n_inst == 0) return c.end_call();
  const float* dc = device_coords(c, coords, n_rows, n_cols, flags, &s);
  if (!dc) return s;
  Batch B(c, dc, n_rows);
  // dens.cpp:52-72 order: i < j (< k)
  for (size_t i = 0; i < M; ++i) {
    if (dims == 1) {
      const uint32_t z = 0;
      B.add(1, &i, &z, &h[i]);
      continue;
    }
    for (size_t j = i + 1; j < M; ++j) {
      if (dims == 2) {
        const size_t cc[2] = {i, j};
        const float hh[2] = {h[i], h[j]};
        B.add(2, cc, lag, hh);
        continue;
      }
      for (size_t k = j + 1; k < M; ++k) {
        const size_t cc[3] = {i, j, k};
        const float hh[3] = {h[i], h[j], h[k]};
        B.add(3, cc, lag, hh);
      }
    }
  }
  if ((s = B.run())) return s;
  std::vector<uint32_t> all(n_inst);
  for (size_t i = 0; i < n_inst; ++i) all[i] = (uint32_t)i;
  double* d_sums = nullptr;
  if ((s = instance_sums(B, all, &d_sums))) return s;
  cudaError_t e = cudaSuccess;
  for (size_t r0 = 0; r0 < n_inst && e == cudaSuccess; r0 += 65535) {  // grid y: 65535 rows
    const size_t nr = std::min<size_t>(65535, n_inst - r0);
    dim3 grid((unsigned)std::min<size_t>((n_sel + 255) / 256, 64), (unsigned)nr);
    k_divide_rows<<<grid, 256, 0, c.stream>>>(B.dens + r0 * n_sel, (uint32_t)n_sel, d_sums + r0);
    e = cudaGetLastError();
    c.stats.kernel_launches += 1;
  }
  if (e != cudaSuccess) return c.cuda_fail(e, "normalise");
  e = cudaMemcpyAsync(out, B.dens, sizeof(double) * n_inst * n_sel,
                      (flags & ENT_BATCH_DEVICE_OUTPUT) ? cudaMemcpyDeviceToDevice
                                                        : cudaMemcpyDeviceToHost,
                      c.stream);
  if (e != cudaSuccess) return c.cuda_fail(e, "read densities");
  s = c.end_call();
  c.collect_kernel_stats();
  return s;
}

}  // extern "C"

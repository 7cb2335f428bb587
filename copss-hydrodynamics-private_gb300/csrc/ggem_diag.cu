// ggem_diag.cu -- measurement hooks (include/ggem_diag.h): launch counts,
// per-kernel CUDA-event timing and the FP32 FMA throughput probe.
#include <cuda_runtime.h>

#include "ggem_diag.h"
#include "ggem_internal.cuh"

namespace ggem {

static cudaEvent_t take_event(ggem_ctx *c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

static bool kt_on(const ggem_ctx *c, int kind) {
  return c->timing && (c->timing_mask >> kind & 1u);
}

bool kt_enabled(const ggem_ctx *c, int kind) { return kt_on(c, kind); }

void kt_start(ggem_ctx *c, int kind) {
  if (!kt_on(c, kind) || c->span_kind == kind) return;
  auto &t = c->ktimer[kind];
  if (t.ev.size() % 2 == 1) {  // a start left open by an error return: restart it
    cudaEventRecord(t.ev.back(), c->stream);
    return;
  }
  cudaEvent_t e = take_event(c);
  if (!e) return;
  cudaEventRecord(e, c->stream);
  c->ktimer[kind].ev.push_back(e);
}

static void kt_stop_n(ggem_ctx *c, int kind, int launches) {
  auto &t = c->ktimer[kind];
  if (t.ev.size() % 2 == 0) return;  // unmatched start
  cudaEvent_t e = launches > 0 ? take_event(c) : nullptr;
  if (!e) {
    c->ev_pool.push_back(t.ev.back());
    t.ev.pop_back();
    return;
  }
  cudaEventRecord(e, c->stream);
  t.ev.push_back(e);
  t.n.push_back(launches);
}

void kt_stop(ggem_ctx *c, int kind) {
  if (!kt_on(c, kind)) return;
  if (c->span_kind == kind) {
    ++c->span_n;
    return;
  }
  kt_stop_n(c, kind, 1);
}

void kt_span_begin(ggem_ctx *c, int kind) {
  kt_span_end(c);
  if (!kt_on(c, kind)) return;
  kt_start(c, kind);
  c->span_kind = kind;
  c->span_n = 0;
}

void kt_span_end(ggem_ctx *c) {
  if (c->span_kind < 0) return;
  const int kind = c->span_kind;
  c->span_kind = -1;
  kt_stop_n(c, kind, c->span_n);
}

void trace_mark(ggem_ctx *c, const char *what) {
  if (c->trace_ev.size() >= 100000) return;
  cudaEvent_t e = take_event(c);
  if (!e) return;
  cudaEventRecord(e, c->stream);
  c->trace_ev.emplace_back(what, e);
}

static int drain(ggem_ctx *c) {
  cudaError_t err = cudaStreamSynchronize(c->stream);
  if (err) return cuda_fail(c, err, "timing sync");
  for (auto &t : c->ktimer) {
    for (size_t k = 0; k + 1 < t.ev.size(); k += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, t.ev[k], t.ev[k + 1]) == cudaSuccess) {
        t.total_ms += ms;
        t.count += k / 2 < t.n.size() ? t.n[k / 2] : 1;
      } else {
        cudaGetLastError();
      }
      c->ev_pool.push_back(t.ev[k]);
      c->ev_pool.push_back(t.ev[k + 1]);
    }
    // an open start (a span in progress) stays
    const bool open = t.ev.size() % 2 == 1;
    cudaEvent_t last = open ? t.ev.back() : nullptr;
    t.ev.clear();
    t.n.clear();
    if (open) t.ev.push_back(last);
  }
  return GGEM_OK;
}

namespace {
// eight independent FMA chains per thread; the store keeps the chains alive
__global__ void __launch_bounds__(256) k_fma_probe(int iters, float seed, float *sink) {
  float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
  float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
  const float m = 0.999999f, b = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fmaf(a0, m, b);
      a1 = fmaf(a1, m, b);
      a2 = fmaf(a2, m, b);
      a3 = fmaf(a3, m, b);
      a4 = fmaf(a4, m, b);
      a5 = fmaf(a5, m, b);
      a6 = fmaf(a6, m, b);
      a7 = fmaf(a7, m, b);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678f) sink[threadIdx.x] = s;  // never true for these inputs
}
}  // namespace

}  // namespace ggem

using namespace ggem;

extern "C" int ggem_get_launch_count(const ggem_ctx *ctx, int64_t *count) {
  if (!ctx || !count) return GGEM_ERR_BAD_ARG;
  *count = ctx->launches;
  return GGEM_OK;
}

extern "C" int ggem_get_pair_count(const ggem_ctx *ctx, int64_t *count) {
  if (!ctx || !count) return GGEM_ERR_BAD_ARG;
  // reading pending statistics of a deferred build updates only cached state
  if (int rc = settle_list(const_cast<ggem_ctx *>(ctx))) return rc;
  if (!ctx->list_built) return GGEM_ERR_BAD_ARG;
  *count = ctx->n_pairs;
  return GGEM_OK;
}

extern "C" int ggem_get_pair_storage(const ggem_ctx *ctx, int *row_width, int *tensors_stored) {
  if (!ctx || !row_width || !tensors_stored) return GGEM_ERR_BAD_ARG;
  if (int rc = settle_list(const_cast<ggem_ctx *>(ctx))) return rc;
  if (!ctx->list_built) return GGEM_ERR_BAD_ARG;
  *row_width = ctx->nb_w;
  *tensors_stored = ctx->pretensor_ok ? 1 : 0;
  return GGEM_OK;
}

extern "C" int ggem_set_fp64_pair_list(ggem_ctx *ctx, int enable) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  if (ctx->prm.precision != GGEM_FP64 || ctx->prm.nb_mode != GGEM_NB_CUTOFF)
    return ggem::fail(ctx, GGEM_ERR_BAD_ARG, "the FP64 pair list needs a GGEM_FP64 cutoff context");
  ctx->f64_list = enable != 0;
  ctx->cells_built = false;  // the next ggem_build_cells builds (or drops) the list
  ctx->list_built = false;
  return GGEM_OK;
}

extern "C" int ggem_set_pair_tensors(ggem_ctx *ctx, int enable) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  ctx->allow_pretensor = enable != 0;
  return GGEM_OK;
}

extern "C" int ggem_set_kernel_timing_kinds(ggem_ctx *ctx, int enable, unsigned mask) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  kt_span_end(ctx);
  if (int rc = drain(ctx)) return rc;
  for (auto &t : ctx->ktimer) {
    t.total_ms = 0.0;
    t.count = 0;
    for (cudaEvent_t e : t.ev) ctx->ev_pool.push_back(e);  // an unmatched start
    t.ev.clear();
    t.n.clear();
  }
  ctx->timing = enable != 0;
  ctx->timing_mask = mask & 0x1fu;
  return GGEM_OK;
}

extern "C" int ggem_set_series_graphs(ggem_ctx *ctx, int enable) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  ctx->series_graphs = enable != 0;
  if (!ctx->series_graphs) {
    cudaStreamSynchronize(ctx->stream);  // a replay in flight keeps using them
    for (cudaGraphExec_t &g : ctx->sg_exec)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    ctx->sg_key.clear();
  }
  return GGEM_OK;
}

extern "C" int ggem_get_series_graph_stats(const ggem_ctx *ctx, int64_t *captures,
                                           int64_t *replays) {
  if (!ctx || !captures || !replays) return GGEM_ERR_BAD_ARG;
  *captures = ctx->sg_captures;
  *replays = ctx->sg_replays;
  return GGEM_OK;
}

extern "C" int ggem_set_kernel_timing(ggem_ctx *ctx, int enable) {
  return ggem_set_kernel_timing_kinds(ctx, enable, 0x1fu);
}

extern "C" int ggem_get_kernel_timing(ggem_ctx *ctx, int kernel, double *total_ms,
                                      int64_t *launches) {
  if (!ctx || kernel < 0 || kernel > 4 || !total_ms || !launches) return GGEM_ERR_BAD_ARG;
  if (int rc = drain(ctx)) return rc;
  *total_ms = ctx->ktimer[kernel].total_ms;
  *launches = ctx->ktimer[kernel].count;
  return GGEM_OK;
}

extern "C" int ggem_probe_fp32_peak(ggem_ctx *ctx, double *tflops) {
  if (!ctx || !tflops) return GGEM_ERR_BAD_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  if (sms <= 0) sms = 1;
  DevBuf<float> sink;
  cudaError_t e = sink.ensure(256);
  if (e) return cuda_fail(ctx, e, "probe buffer");
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8, threads = 256, iters = 2048;
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(a, ctx->stream);
    k_fma_probe<<<blocks, threads, 0, ctx->stream>>>(iters, 1.0f + rep, sink.p);
    cudaEventRecord(b, ctx->stream);
    if (int rc = check_launch(ctx, "fma probe")) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return rc;
    }
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    if (rep > 0 && ms > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *tflops = best;
  return GGEM_OK;
}

extern "C" int ggem_set_launch_trace(ggem_ctx *ctx, int enable) {
  if (!ctx) return GGEM_ERR_BAD_ARG;
  cudaError_t err = cudaStreamSynchronize(ctx->stream);
  if (err) return cuda_fail(ctx, err, "trace sync");
  for (auto &t : ctx->trace_ev) ctx->ev_pool.push_back(t.second);
  ctx->trace_ev.clear();
  ctx->trace = enable != 0;
  if (ctx->trace) trace_mark(ctx, "trace start");
  return GGEM_OK;
}

extern "C" int ggem_get_launch_trace(ggem_ctx *ctx, int64_t max, double *t_ms,
                                     const char **names, int64_t *count) {
  if (!ctx || !count || (max > 0 && (!t_ms || !names))) return GGEM_ERR_BAD_ARG;
  cudaError_t err = cudaStreamSynchronize(ctx->stream);
  if (err) return cuda_fail(ctx, err, "trace sync");
  const int64_t n = (int64_t)ctx->trace_ev.size();
  *count = n;
  for (int64_t k = 0; k < n && k < max; ++k) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->trace_ev[0].second, ctx->trace_ev[k].second) != cudaSuccess) {
      cudaGetLastError();
      ms = -1.f;
    }
    t_ms[k] = ms;
    names[k] = ctx->trace_ev[k].first;
  }
  return GGEM_OK;
}

namespace ggem {
__global__ void k_convert_check(int64_t n, const double *__restrict__ in, float *__restrict__ out,
                                float *__restrict__ ref) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = d2f_bits(in[i]);
  ref[i] = __double2float_rn(in[i]);
}
}  // namespace ggem

extern "C" int ggem_diag_convert_f32(ggem_ctx *ctx, int64_t n, const double *d_in, float *d_out,
                                     float *d_ref) {
  if (!ctx || n < 0 || (n > 0 && (!d_in || !d_out || !d_ref))) return GGEM_ERR_BAD_ARG;
  if (n == 0) return GGEM_OK;
  k_convert_check<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(n, d_in, d_out, d_ref);
  if (int rc = check_launch(ctx, "convert check")) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_fail(ctx, e, "convert check");
  return GGEM_OK;
}

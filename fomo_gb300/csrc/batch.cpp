// Batched rendering captured in CUDA graphs, and the ray-tile autotuner.
//
// A planned batch (plan_batch) is one descriptor upload followed, per launch,
// by the view set-up kernels and one persistent march.  Everything that
// varies between batches of the same shape -- angles, tables, output
// pointers -- lives in the uploaded descriptors, so the captured graph is
// replayed as is after the host refills the pinned staging blob.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fomo_gpu.h"
#include "runtime_internal.h"

using namespace fomo;

namespace {

std::string plan_key(const Plan& p, const ScratchSet& scr) {
  std::ostringstream k;
  k << (const void*)scr.arena.base << "/" << (const void*)scr.staging.base << "/" << p.host_bytes << "/"
    << p.dev_bytes;
  for (const PlanGroup& G : p.groups)
    k << "|" << G.snapshot << "," << G.method << "," << G.imaging << "," << G.nv << "," << G.nl << "," << G.maxL
      << "," << G.maxnz << "," << G.maxnx << "," << G.maxny << "," << G.total_items << "," << G.tw << "," << G.th
      << "," << G.bps << "," << G.rscale << "," << G.any_nn << "," << (const void*)G.totpol;
  return k.str();
}

int order_after_ctx_stream(fomo_ctx* ctx, cudaStream_t s) {
  if (s == ctx->stream) return FOMO_OK;
  // payload kernels were queued on the context stream while planning
  cudaError_t e = cudaEventRecord(ctx->order_ev, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ctx->order_ev, 0);
  if (e != cudaSuccess) return cuda_err(ctx, e, "stream ordering");
  return FOMO_OK;
}

}  // namespace

namespace fomo {
int order_streams(fomo_ctx* ctx, cudaStream_t s) { return order_after_ctx_stream(ctx, s); }
}  // namespace fomo

extern "C" {

int fomo_render_batch_graph(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_outs, void* stream) {
  if (!ctx || !reqs || nreq <= 0 || !d_outs) return FOMO_EINVAL;
  NvtxRange range("fomo: render batch (graph)");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  Plan plan;
  int rc = plan_batch(ctx, reqs, nreq, d_outs, nullptr, &ctx->scratch, &plan);
  if (rc) return rc;
  rc = order_after_ctx_stream(ctx, s);
  if (rc) return rc;
  const std::string key = plan_key(plan, ctx->scratch);
  auto it = ctx->graphs.find(key);
  if (it == ctx->graphs.end()) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_err(ctx, e, "graph capture begin");
    rc = issue_plan(ctx, plan, &ctx->scratch, s);
    e = cudaStreamEndCapture(s, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_err(ctx, e, "graph capture end");
    GraphRec rec;
    e = cudaGraphInstantiate(&rec.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_err(ctx, e, "graph instantiate");
    if (ctx->graphs.size() > 64) {  // bound the cache
      for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
      ctx->graphs.clear();
    }
    it = ctx->graphs.emplace(key, rec).first;
  }
  cudaError_t e = cudaGraphLaunch(it->second.exec, s);
  if (e != cudaSuccess) return cuda_err(ctx, e, "graph launch");
  // the staging blob may be rewritten once this launch (and its upload) has run
  e = cudaEventRecord(ctx->scratch.staging.copy_done, s);
  if (e != cudaSuccess) return cuda_err(ctx, e, "graph launch");
  return FOMO_OK;
}

// Measure candidate march configurations on the given batch (device
// outputs), keep the fastest per workload class.  The axes: the ray tile
// (which rays a warp takes one after the other, i.e. the L1/L2 locality of
// consecutive work items), the CTAs-per-SM cap of the search pass (its
// occupancy against its shared-memory candidate lists), and the gather radius
// of the search in local point spacings (a wider gather resolves more samples
// in the first pass, at more candidates per segment; a narrower one leaves more
// to the deferred pass).  The segment length is fixed at 64 LOS samples (two
// per lane) by the deferred-record format.  Cache file lines:
// "<class> tile_w tile_h blocks_per_sm rscale ms".
int fomo_autotune(fomo_ctx* ctx, const fomo_request* reqs, int nreq, const char* cache_path) {
  if (!ctx || !reqs || nreq <= 0) return FOMO_EINVAL;
  NvtxRange range("fomo: autotune");
  cudaSetDevice(ctx->device);
  std::vector<size_t> off(nreq);
  size_t total = 0;
  for (int r = 0; r < nreq; ++r) {
    int rc = validate(ctx, reqs[r]);
    if (rc) return rc;
    off[r] = total;
    total += (cube_elems(reqs[r]) * sizeof(float) + 255) & ~size_t(255);
  }
  int rc = ctx->out_arena.reserve(ctx, total);
  if (rc) return rc;
  std::vector<float*> d(nreq);
  for (int r = 0; r < nreq; ++r) d[r] = reinterpret_cast<float*>(ctx->out_arena.base + off[r]);
  // classes covered by this batch
  Plan probe;
  rc = plan_batch(ctx, reqs, nreq, d.data(), nullptr, &ctx->scratch, &probe);
  if (rc) return rc;
  std::vector<std::string> classes;
  for (const PlanGroup& G : probe.groups) classes.push_back(workload_class(G, ctx->snaps[G.snapshot]));
  // cached answers
  if (cache_path) {
    std::ifstream f(cache_path);
    std::string line;
    bool all = true;
    std::map<std::string, TuneChoice> found;
    while (std::getline(f, line)) {
      std::string k;
      TuneChoice c;
      if (parse_tune_line(line, &k, &c)) found[k] = c;
    }
    for (auto& k : classes) {
      if (found.count(k))
        ctx->tuned[k] = found[k];
      else
        all = false;
    }
    if (all) return FOMO_OK;
  }
  const int saved_w = ctx->tile_w, saved_h = ctx->tile_h, saved_b = ctx->blocks_per_sm;
  const float saved_r = ctx->rscale;
  // {tile_w, tile_h, CTA cap of the search, gather radius x 10}: tiles at the
  // default search, then the search's occupancy and radius at the default tile
  const int cands[][4] = {{8, 4, 0, 9},  {16, 2, 0, 9}, {4, 8, 0, 9},  {32, 1, 0, 9},  {8, 8, 0, 9},
                          {8, 4, 6, 9},  {8, 4, 5, 9},  {8, 4, 0, 8},  {8, 4, 0, 10}, {8, 4, 0, 11}};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  TuneChoice bestc;
  for (auto& c : cands) {
    ctx->tile_w = c[0];
    ctx->tile_h = c[1];
    ctx->blocks_per_sm = c[2];
    ctx->rscale = 0.1f * (float)c[3];
    rc = enqueue_batch(ctx, reqs, nreq, d.data(), nullptr, ctx->stream, nullptr, nullptr);  // warm-up
    if (rc) break;
    cudaEventRecord(e0, ctx->stream);
    for (int rep = 0; rep < 2 && rc == 0; ++rep)
      rc = enqueue_batch(ctx, reqs, nreq, d.data(), nullptr, ctx->stream, nullptr, nullptr);
    cudaEventRecord(e1, ctx->stream);
    if (rc) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = cuda_err(ctx, cudaGetLastError(), "autotune");
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      bestc = TuneChoice{c[0], c[1], c[2], 0.1f * (float)c[3]};
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tile_w = saved_w;
  ctx->tile_h = saved_h;
  ctx->blocks_per_sm = saved_b;
  ctx->rscale = saved_r;
  if (rc) return rc;
  for (auto& k : classes) ctx->tuned[k] = bestc;
  if (cache_path) {
    std::ofstream f(cache_path, std::ios::app);
    for (auto& k : classes)
      f << k << " " << bestc.tile_w << " " << bestc.tile_h << " " << bestc.blocks_per_sm << " " << bestc.rscale << " "
        << best / 2 << "\n";
  }
  return FOMO_OK;
}

}  // extern "C"

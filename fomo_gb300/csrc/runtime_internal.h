// Host-side state of a libfomo_gpu context (opaque behind fomo_ctx* in the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <functional>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/fomo_gpu.h"
#include "fomo_internal.h"

namespace fomo {

// A named range of the host thread on the NVTX timeline (Nsight Systems, ncu
// --nvtx) around one stage of the library: snapshot upload and index build,
// emissivity, batch planning and launch, downloads, autotuning, a server
// batch.  Header-only NVTX 3: without a tool attached a range costs a few
// nanoseconds.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

struct TableHost {
  std::string ion, unit;
  double lambda0 = 0, atweight = 0;
  int nt = 0, nrho = 0;
  bool is_dn = false;
  std::vector<float> logT, logn, G;
};

struct TableRec {
  TableHost h;
  float* d = nullptr;  // logT | logn | G
};

struct SnapRec {
  int64_t n = 0;
  int64_t ncells = 0;
  GridParams g{};
  void* block = nullptr;  // one allocation for everything below
  size_t bytes = 0;
  float4* pts = nullptr;
  float4* vel = nullptr;
  float* ne = nullptr;
  float* T = nullptr;
  int* cell_start = nullptr;
  float* blk = nullptr;      // per-block bounding boxes (SnapDev::blk)
  int bdx = 0, bdy = 0, bdz = 0;
  float2* totpol = nullptr;  // Thomson payload, built on first use
  float vmax = 0.0f;         // largest |v| (bounds every Doppler shift)
};

// Grow-only device scratch; contents belong to the work last enqueued.
struct Arena {
  char* base = nullptr;
  size_t cap = 0;
  int reserve(fomo_ctx* ctx, size_t bytes);
};

// Pinned host staging for descriptor uploads; copy_done marks when the last
// upload from it has executed, before it may be rewritten.
struct Staging {
  char* base = nullptr;
  size_t cap = 0;
  cudaEvent_t copy_done = nullptr;
  int reserve(fomo_ctx* ctx, size_t bytes);
};

// Scratch for one in-flight batch: device arena, pinned descriptor staging and
// march timing events.  The context has one; the server one per slot.
struct ScratchSet {
  Arena arena;
  Staging staging;
  unsigned* stop = nullptr;  // a server slot's stop word (device), null for the context's own batches
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaError_t init() {
    cudaError_t e = cudaEventCreate(&ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ev1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&staging.copy_done, cudaEventDisableTiming);
    return e;
  }
  void release() {
    if (staging.copy_done) cudaEventSynchronize(staging.copy_done);
    if (staging.base) cudaFreeHost(staging.base);
    staging.base = nullptr;
    staging.cap = 0;
    if (staging.copy_done) cudaEventDestroy(staging.copy_done);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    staging.copy_done = ev0 = ev1 = nullptr;
  }
};

// One launch of a planned batch: requests sharing (snapshot, method, imaging).
struct PlanGroup {
  int snapshot = 0, method = 0, imaging = 0;
  std::vector<int> reqs;
  std::vector<std::vector<int>> vreqs;  // requests (lines) of each view
  int nv = 0, nl = 1, maxL = 1, maxnz = 1, maxnx = 2, maxny = 2;
  int max_nw = 1;  // largest number of 32-bin lambda windows of a line
  int tw = 8, th = 4, bps = 0;
  float rscale = 0.0f;
  std::vector<const float2*> ew;       // payload per request (NN)
  const float2* totpol = nullptr;      // Thomson payload
  bool any_nn = false;
  int64_t total_items = 0;
  int vbase = 0;
  size_t o_views = 0, o_lines = 0, o_off = 0, o_nnp = 0, o_lam = 0, o_ktab = 0, o_xy = 0, o_ctr = 0, o_s2 = 0;
  size_t o_def = 0;          // deferred-sample records
  size_t o_far = 0;          // slots of the records flagged for the far pass (with a neighbour buffer), or 0
  std::vector<std::pair<float*, size_t>> zero_outs;  // projection outputs to clear before the scatter
  int64_t deferred_cap = 0;  // records: one per segment of every work item
  size_t o_hard = 0;
  int64_t hard_cap = 0;      // hard-sample queue entries
  size_t o_npos = 0;         // a neighbour per (work item, sample) for the emission pass, or 0 (projection)
  int64_t npos_items = 0;    // work items the neighbour buffer holds (the launch marches in chunks of these)
  std::vector<int64_t> item_off;  // first work item of each view (nv + 1 entries)
  std::vector<double> vcost;      // LOS samples + output cells of each view
  size_t out_bytes = 0;           // cube bytes of all its requests
};

struct Plan {
  std::vector<PlanGroup> groups;
  std::vector<int> view_of_req;
  int nviews_total = 0;
  size_t host_bytes = 0, dev_bytes = 0;
  char* arena_base = nullptr;
};

struct ViewReadback {
  ViewDesc* dev;
  size_t base;
  int count;
};

struct GraphRec {
  cudaGraphExec_t exec = nullptr;
};

// One autotuned march configuration: ray tile, CTAs-per-SM cap of the search
// pass (0 = occupancy maximum), gather radius in local point spacings (0 = the
// default).
struct TuneChoice {
  int tile_w = 8, tile_h = 4, blocks_per_sm = 0;
  float rscale = 0.0f;
};

}  // namespace fomo

struct fomo_ctx {
  int device = 0;
  int sm_count = 152;
  cudaStream_t stream = nullptr;
  size_t budget = 0;
  size_t used = 0;
  std::map<void*, size_t> sizes;
  // freed blocks kept for an allocation of the same size (dev_free / dev_alloc)
  std::multimap<size_t, void*> free_blocks;
  size_t cached = 0;
  int next_id = 1;
  std::string err;
  std::map<int, fomo::SnapRec> snaps;
  std::map<int, fomo::TableRec> tables;
  std::map<std::tuple<int, int, int, double>, float2*> payloads;
  std::map<std::tuple<int, int, int, double>, float> payload_wmax;  // largest FWHM of emitting points
  void* stats_dev = nullptr;  // small device buffer for reductions read back by the host
  unsigned long long* march_stats = nullptr;  // search counters (profiling; FOMO_MARCH_STATS=1 prints them at destroy)
  bool print_stats = false;
  bool kernel_timing = false;  // per-kernel events around the march's kernels (direct launches)
  fomo::MarchTimer timer;
  fomo::ScratchSet scratch;  // descriptors, per-view tables, Thomson sin^2 chi
  fomo::Arena out_arena;     // device cubes of host-output renders
  std::vector<fomo::ViewReadback> view_readback;
  double cell_occupancy = 2.0;  // target points per grid cell (FOMO_CELL_OCCUPANCY)
  bool occupancy_set = false;   // set explicitly: no per-snapshot choice (see build_snapshot)
  int64_t npos_cap = int64_t(1) << 31;  // neighbour-buffer entries per launch (FOMO_NPOS_CAP): 8 GiB
  long fail_alloc_at = 0;  // FOMO_INJECT_ALLOC_FAILURE: this allocation (1-based) fails, for error-path tests
  long alloc_count = 0;
  int tile_w = 0, tile_h = 0, blocks_per_sm = 0;
  float rscale = 0.0f;  // forced gather radius (autotuner trials), 0 = tuned or default
  bool time_march = true;
  float last_ms = 0.0f;
  cudaEvent_t order_ev = nullptr;  // orders a caller stream after the context stream
  // host-output batches: the cube downloads of one range of views overlap the
  // march of the next (created on first use)
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> range_ev;
  std::map<std::string, fomo::GraphRec> graphs;
  std::map<std::string, fomo::TuneChoice> tuned;
};

namespace fomo {

int set_err(fomo_ctx* c, int code, const std::string& msg);
int cuda_err(fomo_ctx* c, cudaError_t e, const char* what);
int dev_alloc(fomo_ctx* ctx, void** p, size_t bytes);
void dev_free(fomo_ctx* ctx, void* p);
void release_free_blocks(fomo_ctx* ctx);  // cudaFree of the blocks dev_free kept
int validate(fomo_ctx* ctx, const fomo_request& q);
size_t cube_elems(const fomo_request& q);
// Called by issue_plan once the work of views [v0, v1) of launch G is on the
// stream: their cubes are complete when the stream reaches that point.  With
// it, a launch marches in view ranges: ranges of about `range_cost` LOS
// samples + output cells each when that is > 0, else up to 8 ranges, one per
// 256 MB of cubes.
using RangeDone = std::function<int(const PlanGroup& G, int v0, int v1)>;
int enqueue_batch(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_out, int32_t* const* d_nn,
                  cudaStream_t s, std::vector<ViewDesc>* views_out, std::vector<int>* view_of_req,
                  const RangeDone* done = nullptr);
int plan_batch(fomo_ctx* ctx, const fomo_request* reqs, int nreq, float* const* d_out, int32_t* const* d_nn,
               ScratchSet* scr, Plan* plan);
int issue_plan(fomo_ctx* ctx, const Plan& plan, ScratchSet* scr, cudaStream_t s, const RangeDone* done = nullptr,
               double range_cost = 0.0);
std::string workload_class(const PlanGroup& G, const SnapRec& snap);
int order_streams(fomo_ctx* ctx, cudaStream_t s);
SnapDev snap_dev(const SnapRec& r);
float payload_wmax(fomo_ctx* ctx, int snap, int table, int imaging, double abund);
void line_window(double lwa, int L, double lambda0, float vmax, float wmax, int* wstart, int* nw);
void fill_view_host(const fomo_request& q, double lambda0, int tw, int th, ViewDesc* V);
int finish_views(fomo_ctx* ctx, std::vector<ViewDesc>* views);
void view_info_from(const ViewDesc& V, const fomo_request& q, const TableHost* t, fomo_view_info* info);
int parse_table_text(const std::string& text, TableHost* t, std::string* err);
bool parse_tune_line(const std::string& line, std::string* key, TuneChoice* c);
// Upload n points (host or device arrays: x, y, z, n, T, vx, vy, vz; z may be
// null) and build the snapshot's spatial index.
int build_snapshot(fomo_ctx* ctx, int64_t n, const float* const host[8], SnapRec* out);
// Bounds-check build: read and clear the kernels' error words (FOMO_EDEVICE
// when one is set); FOMO_OK in the regular build.
int check_device_words(fomo_ctx* ctx);

}  // namespace fomo

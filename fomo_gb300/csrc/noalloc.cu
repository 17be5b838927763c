// fomo_render_noalloc: a nearest-neighbour render that allocates nothing.
//
// Some callers cannot allocate device memory while they render: a host
// application that runs its own device-memory pool and forbids allocation
// inside its frame loop, an embedding that has handed the whole device memory
// budget out in advance, or code on a real-time path where cudaMalloc /
// cudaFree would synchronise the device and stall it.  fomo_render (and its
// batched forms) keep their per-render working memory in a context arena that
// grows with cudaMalloc when a larger render comes along.  This entry point
// instead places that working memory -- the view and line descriptors, the
// lambda table, the per-sample derotation table, the per-ray position tables,
// the work counters and the deferred-sample queue -- in one file-scope static
// __device__ array of fixed size, so a call never allocates.  The descriptors
// reach the array as the parameter of a small kernel, not through a host
// copy.  The queue's fixed capacity (65,536 segment records) makes a large
// render march its rays in chunks; each chunk costs a counter clear and four
// launches (first pass, split, deferred and hard passes), so a render at the
// limits (4096 x 4096 rays at nz = 4096: chunks of 1,024 rays) issues about
// 16,000 chunks.
//
// The array costs every GPU that loads the library kNoAllocScratchBytes of
// device memory until the process exits.  Its device address is looked up
// with cudaGetSymbolAddress once per device, on the first call made on that
// device (that first call should therefore come before any stream capture).
// Every call on a device shares the same array and the array keeps the last
// call's contents: the work counters are cleared by each chunk, the per-view
// extents are initialised by a kernel of each call, everything else is fully
// rewritten.  Calls that overlap on the GPU (e.g. on two streams) race on the
// array; serialise them.
//
// The kernels are the ones every other render uses (view set-up and the ray
// march); only the place of their scratch differs.  With no room for a
// neighbour buffer, the march is the fused one: the first pass searches and
// bins, and the deferred samples' emission is added with atomics, so a cube
// matches the regular render's to FP32 summation order (not bit for bit).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/fomo_gpu.h"
#include "runtime_internal.h"

namespace fomo {
namespace {

constexpr int kNoAllocMaxNz = 4096;     // LOS samples
constexpr int kNoAllocMaxNxNy = 8192;   // x_pixel + y_pixel
constexpr int kNoAllocMaxL = 256;       // lambda bins
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }
// layout of the scratch array
constexpr size_t kOffView = 0;
constexpr size_t kOffLine = align_up(kOffView + sizeof(ViewDesc));
constexpr size_t kOffRayOff = align_up(kOffLine + sizeof(LineDesc));
constexpr size_t kOffLam = align_up(kOffRayOff + 2 * sizeof(int64_t));
constexpr size_t kHdrBytes = align_up(kOffLam + kNoAllocMaxL * sizeof(float));  // uploaded per call
constexpr size_t kOffCounter = kHdrBytes;
constexpr size_t kOffKtab = align_up(kOffCounter + kCtrCount * sizeof(unsigned long long));
constexpr size_t kOffXY = align_up(kOffKtab + (size_t)kNoAllocMaxNz * sizeof(double3));
constexpr size_t kOffDeferred = align_up(kOffXY + (size_t)kNoAllocMaxNxNy * sizeof(double));
// Deferred-sample queue: the rays are marched in chunks of at most
// kNoAllocDeferredCap segments (1024 rays at the largest nz).
constexpr int64_t kNoAllocDeferredCap = 65536;
constexpr size_t kNoAllocScratchBytes = align_up(kOffDeferred + (size_t)kNoAllocDeferredCap * sizeof(DeferredRec));

// The scratch of fomo_render_noalloc (about 1.2 MB per device).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The per-call descriptors (view, line, ray offsets, lambda table), built on
// the host.  They travel to the scratch array as a kernel parameter: a kernel
// argument is copied when the launch is issued, so the host buffer may go
// away at once and nothing goes through pageable memory.
struct HeaderBlob {
  uint4 w[kHdrBytes / sizeof(uint4)];
};
static_assert(kHdrBytes % sizeof(uint4) == 0, "header size");
static_assert(sizeof(HeaderBlob) <= 4000, "descriptors must fit the kernel parameter space");

__global__ void put_header(const HeaderBlob blob, uint4* dst) {
  for (int i = threadIdx.x; i < (int)(kHdrBytes / sizeof(uint4)); i += blockDim.x) dst[i] = blob.w[i];
}

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array on `device` (which must be current).
cudaError_t scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_addr[device]);
  return cudaSuccess;
}

}  // namespace
}  // namespace fomo

using namespace fomo;

extern "C" int fomo_render_noalloc(fomo_ctx* ctx, const fomo_request* req, float* d_out_cube, void* stream) {
  if (!ctx || !req || !d_out_cube) return FOMO_EINVAL;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return set_err(ctx, FOMO_EDEVICE, "cudaSetDevice failed");
  const fomo_request& q = *req;
  int rc = validate(ctx, q);
  if (rc) return rc;
  if (q.method != FOMO_METHOD_NN)
    return set_err(ctx, FOMO_EINVAL, "fomo_render_noalloc renders the NearestNeighbour method only");
  if (q.nz > kNoAllocMaxNz || q.nx + q.ny > kNoAllocMaxNxNy || q.nlambda > kNoAllocMaxL)
    return set_err(ctx, FOMO_EINVAL,
                   "fomo_render_noalloc limits: nz <= " + std::to_string(kNoAllocMaxNz) + ", nx + ny <= " +
                       std::to_string(kNoAllocMaxNxNy) + ", nlambda <= " + std::to_string(kNoAllocMaxL) +
                       " (its working memory is a fixed static device array)");
  const int imaging = q.nlambda <= 1 ? 1 : 0;
  auto pit = ctx->payloads.find(std::make_tuple(q.snapshot, q.table, imaging, q.abundratio));
  if (pit == ctx->payloads.end())
    return set_err(ctx, FOMO_EINVAL,
                   "emissivity of this snapshot and table is not resident yet: call fomo_emission or a regular "
                   "render for it once before fomo_render_noalloc (which allocates nothing)");
  unsigned char* base = nullptr;
  cudaError_t e = scratch_address(ctx->device, &base);
  if (e != cudaSuccess) return cuda_err(ctx, e, "cudaGetSymbolAddress (no-alloc scratch)");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;

  const SnapRec& snap = ctx->snaps[q.snapshot];
  const TableHost& t = ctx->tables[q.table].h;
  // descriptors, built on the host and written into the static array by a
  // kernel that receives them as its parameter
  HeaderBlob blob;
  unsigned char* hdr = reinterpret_cast<unsigned char*>(blob.w);
  std::memset(hdr, 0, sizeof(blob));
  ViewDesc* hv = reinterpret_cast<ViewDesc*>(hdr + kOffView);
  LineDesc* hl = reinterpret_cast<LineDesc*>(hdr + kOffLine);
  int64_t* hoff = reinterpret_cast<int64_t*>(hdr + kOffRayOff);
  float* hlam = reinterpret_cast<float*>(hdr + kOffLam);
  const int tw = 8, th = 4;
  fill_view_host(q, t.lambda0, tw, th, hv);
  double* dxy = reinterpret_cast<double*>(base + kOffXY);
  hv->xt = dxy;
  hv->yt = dxy + q.nx;
  hoff[0] = 0;
  hoff[1] = (int64_t)((q.nx + tw - 1) / tw) * tw * (int64_t)((q.ny + th - 1) / th) * th;
  hl->ew = pit->second;
  hl->out = d_out_cube;
  hl->lambda0 = t.lambda0;
  hl->lwa = q.lambda_width * t.lambda0 / FOMO_SPEED_OF_LIGHT;  // nn:116
  hl->shift_k = (float)(t.lambda0 / FOMO_SPEED_OF_LIGHT);
  hl->is_dn = t.is_dn ? 1 : 0;
  hl->lam = reinterpret_cast<const float*>(base + kOffLam);
  for (int il = 0; il < q.nlambda && q.nlambda > 1; ++il)
    hlam[il] = (float)(double(il) / (q.nlambda - 1) * hl->lwa - hl->lwa / 2.);  // nn:200
  line_window(hl->lwa, q.nlambda, t.lambda0, snap.vmax,
              payload_wmax(ctx, q.snapshot, q.table, imaging, q.abundratio), &hl->wstart, &hl->nw);

  ViewDesc* dv = reinterpret_cast<ViewDesc*>(base + kOffView);
  double3* ktab = reinterpret_cast<double3*>(base + kOffKtab);
  unsigned long long* counter = reinterpret_cast<unsigned long long*>(base + kOffCounter);
  put_header<<<1, 128, 0, s>>>(blob, reinterpret_cast<uint4*>(base));
  e = cudaGetLastError();
  const SnapDev sd = snap_dev(snap);
  if (e == cudaSuccess) e = launch_view_init(dv, 1, s);
  if (e == cudaSuccess) e = launch_view_extents(sd, dv, 1, nullptr, s);
  if (e == cudaSuccess) e = launch_view_finalize(dv, 1, ktab, q.nz, s);
  MarchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.snap = sd;
  a.views = dv;
  a.ray_offset = reinterpret_cast<const int64_t*>(base + kOffRayOff);
  a.lines = reinterpret_cast<const LineDesc*>(base + kOffLine);
  a.nviews = 1;
  a.nlines = 1;
  a.counter = counter;
  a.deferred = reinterpret_cast<DeferredRec*>(base + kOffDeferred);
  a.deferred_cap = kNoAllocDeferredCap;
  const int64_t chunk = kNoAllocDeferredCap / ((q.nz + 63) / 64);  // rays whose segments fit the queue
  for (int64_t b = 0; b < hoff[1] && e == cudaSuccess; b += chunk) {
    a.item_base = b;
    a.total_items = std::min<int64_t>(b + chunk, hoff[1]);
    e = cudaMemsetAsync(counter, 0, kCtrCount * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = launch_march(a, ktab, q.nz, hl->nw, ctx->sm_count, s, 0, imaging != 0);
  }
  if (e != cudaSuccess) return cuda_err(ctx, e, "fomo_render_noalloc launch");
  return FOMO_OK;
}

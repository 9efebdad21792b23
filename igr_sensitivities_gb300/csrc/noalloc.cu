// igr2d_apply_sip_noalloc: the SIP operator application y = A(rho, alpha) x
// for callers that cannot allocate device memory.
//
// Who needs it: a host whose device memory is owned by another allocator —
// e.g. a Julia process whose CUDA.jl pool holds the GPU, or a framework with
// its own caching allocator and a fixed memory budget — must not have this
// library call cudaMalloc behind its back (it would fragment or overrun the
// pool, and cudaMalloc can synchronise the device in a latency-critical loop).
// The regular igr2d_apply_sip keeps its operator coefficients in
// context-owned scratch that it grows with cudaMalloc; this entry point
// takes device pointers for its input and output and keeps its scratch in a
// fixed file-scope device array instead, so it allocates nothing.
//
// Limits and sharing:
//  * at most NOALLOC_MAX_NODES nodes ((p+1)^2 * n_ex * n_ey <= 65,536, e.g.
//    P3 on 64 x 64 elements, or P1 on 1 x 16,384); larger problems are
//    rejected with IGR_EINVAL. The tile list is sized for every mesh under
//    that node limit (at most 4,096 tiles, reached by P1 meshes one element
//    wide), so the node count is the only limit;
//  * the array (about 4.8 MB) lives on every GPU that loads the library until
//    the process exits. With CUDA's lazy module loading it is reserved when the
//    first call on a device loads the library's kernels there, so a caller with
//    a fixed memory budget should make its first call during its own set-up;
//  * all calls share it and it keeps the last call's contents: calls that
//    overlap on the GPU (different streams, or different host threads on one
//    device) race. Every scratch field is written in full before it is read,
//    so nothing needs clearing between calls;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current); make that first call
//    before any stream capture. The address is kept per device together with
//    the identity of the device's CUDA context, and looked up again when that
//    context changes (after a cudaDeviceReset or a CUDA.jl device_reset!, the
//    module and its array are loaded anew at another address).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "../../include/igr_gb300.h"
#include "igr2d_kernels.cuh"
#include "igr2d_launch.h"
#include "igr_engine.h"

namespace igrgpu {
namespace {

constexpr long long NOALLOC_MAX_NODES = 65536;
constexpr int NOALLOC_FIELDS = 9;                 // invr, (unused), cm, ckx, cky, cinvM, cpx, cpy, (spare)
// Tiles of the largest admitted mesh of any degree: P1 tiles are 4 x 4
// elements, and a mesh one element wide with 16,384 elements has 4,096 of them
// (P2: at most 1,821, P3: 1,024, P4 with 2 x 4 tiles: 1,311).
constexpr int NOALLOC_MAX_TILES = 4096;
constexpr size_t NOALLOC_INST_BYTES = 256;        // the Inst2D record
constexpr size_t NOALLOC_META = 68 * 1024;        // Inst2D + tile list, rounded to 256 B
constexpr size_t NOALLOC_BYTES = NOALLOC_META + (size_t)NOALLOC_FIELDS * NOALLOC_MAX_NODES * sizeof(double);
static_assert(sizeof(Inst2D) <= NOALLOC_INST_BYTES, "Inst2D must fit its slot of the scratch array");
static_assert(NOALLOC_INST_BYTES + NOALLOC_MAX_TILES * sizeof(Tile2D) <= NOALLOC_META, "tile list must fit");
static_assert(NOALLOC_META % 256 == 0, "fields start 256-byte aligned");
static_assert((NOALLOC_MAX_NODES / 4 + 3) / 4 <= NOALLOC_MAX_TILES, "P1 meshes one element wide must fit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int MAX_DEVICES = 64;
struct ScratchSlot {
  unsigned char* ptr = nullptr;
  unsigned long long ctx_id = 0;
  bool have_id = false;
};
ScratchSlot g_scratch[MAX_DEVICES];
std::mutex g_scratch_mutex;

// Identity of the calling thread's current CUDA context (unique for the life
// of the process, so a reset device's new context never matches the old one).
// The driver functions are reached through the runtime's entry-point query,
// so the library links only the CUDA runtime. false: no context or no query.
bool current_context_id(unsigned long long* id) {
  static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
  });
  CUcontext ctx = nullptr;
  if (!get_cur || !get_id || get_cur(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

// Set-up, with the device current: the scratch array's device address on the
// current device, looked up with cudaGetSymbolAddress on the first call on the
// device and again whenever the device's context has changed since (or on
// every call when the context identity cannot be read).
int scratch_on_current_device(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return IGR_ECUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  ScratchSlot& slot = g_scratch[dev];
  unsigned long long id = 0;
  const bool have_id = current_context_id(&id);
  if (!slot.ptr || !have_id || !slot.have_id || slot.ctx_id != id) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return IGR_ECUDA;
    slot.ptr = static_cast<unsigned char*>(p);
    // the lookup makes the device's primary context current when none was
    slot.have_id = have_id || current_context_id(&id);
    slot.ctx_id = id;
  }
  *out = slot.ptr;
  return IGR_OK;
}

}  // namespace
}  // namespace igrgpu

using namespace igrgpu;

extern "C" int igr2d_apply_sip_noalloc(const igr_disc2d* d, double alpha, const double* x_dev, const double* rho_dev,
                                       double* y_dev, void* stream) {
  if (!d || !d->xi || !d->w || !d->D || !x_dev || !rho_dev || !y_dev) return IGR_EINVAL;
  if (d->p < 1 || d->p > 4 || d->n_ex < 1 || d->n_ey < 1 || !(d->lx > 0) || !(d->ly > 0)) return IGR_EINVAL;
  const int np = d->p + 1;
  const long long N = (long long)np * np * d->n_ex * d->n_ey;
  if (N > NOALLOC_MAX_NODES) return IGR_EINVAL;  // beyond the fixed scratch: use igr2d_apply_sip
  int tx = 4, ty = 4;
  switch (np) {
    case 2: tile_shape2d<2>(&tx, &ty); break;
    case 3: tile_shape2d<3>(&tx, &ty); break;
    case 4: tile_shape2d<4>(&tx, &ty); break;
    default: tile_shape2d<5>(&tx, &ty); break;
  }
  const int ntx = (d->n_ex + tx - 1) / tx, nty = (d->n_ey + ty - 1) / ty;
  if ((long long)ntx * nty > NOALLOC_MAX_TILES) return IGR_EINVAL;  // not reachable under the node limit
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the call ends by synchronising its stream and stages the tile list from a reused host array: not capturable
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) return IGR_EINVAL;
  unsigned char* base = nullptr;
  int rc = scratch_on_current_device(&base);
  if (rc != IGR_OK) return rc;
  BasisDev B;
  try {
    B = make_basis_dev(d->p, d->xi, d->w, d->D);
  } catch (...) {
    return IGR_EINVAL;
  }
  // instance and tile list, staged from fixed host arrays
  Inst2D I;
  I.off = 0;
  I.nex = d->n_ex; I.ney = d->n_ey;
  I.lx = d->lx; I.ly = d->ly;
  I.dx = d->lx / d->n_ex; I.dy = d->ly / d->n_ey;
  I.jx = I.dx / 2.0; I.jy = I.dy / 2.0;
  I.gamma = 1.4; I.alpha = alpha; I.dt = 0.0;
  I.ijx = 1.0 / I.jx; I.ijy = 1.0 / I.jy; I.idx = 1.0 / I.dx; I.idy = 1.0 / I.dy;
  I.ialpha = alpha > 0 ? 1.0 / alpha : 0.0;
  static thread_local Tile2D tiles[NOALLOC_MAX_TILES];
  int nt = 0;
  for (int ey0 = 0; ey0 < d->n_ey; ey0 += ty)
    for (int ex0 = 0; ex0 < d->n_ex; ex0 += tx) tiles[nt++] = Tile2D{0, ex0, ey0, 0};
  I.tile0 = 0;
  I.ntiles = nt;
  Inst2D* d_inst = reinterpret_cast<Inst2D*>(base);
  Tile2D* d_tiles = reinterpret_cast<Tile2D*>(base + NOALLOC_INST_BYTES);
  double* f = reinterpret_cast<double*>(base + NOALLOC_META);
  double* invr = f;  // field 1 is not used (the IGR source is not formed)
  double* cm = f + 2 * N;
  double* ckx = f + 3 * N;
  double* cky = f + 4 * N;
  double* cinvM = f + 5 * N;
  double* cpx = f + 6 * N;
  double* cpy = f + 7 * N;
  if (cudaMemcpyAsync(d_inst, &I, sizeof(I), cudaMemcpyHostToDevice, s) != cudaSuccess) return IGR_ECUDA;
  if (cudaMemcpyAsync(d_tiles, tiles, sizeof(Tile2D) * nt, cudaMemcpyHostToDevice, s) != cudaSuccess) return IGR_ECUDA;
  launch_recip(rho_dev, invr, N, s);
  SetupArgs2D sa;
  std::memset(&sa, 0, sizeof(sa));
  sa.tiles = d_tiles; sa.inst = d_inst; sa.B = B;
  sa.invr = invr;
  sa.b = nullptr;  // the IGR source is not part of the operator: not formed
  sa.cm = cm; sa.ckx = ckx; sa.cky = cky; sa.cinvM = cinvM; sa.cpx = cpx; sa.cpy = cpy; sa.cM = nullptr;
  sa.always = 1;
  ApplyArgs2D a;
  std::memset(&a, 0, sizeof(a));
  a.tiles = d_tiles; a.inst = d_inst; a.B = B;
  a.x = x_dev; a.cm = cm; a.ckx = ckx; a.cky = cky; a.cpx = cpx; a.cpy = cpy; a.b = nullptr; a.cinvM = cinvM;
  a.y_out = y_dev;
  switch (np) {
    case 2: launch_k2_setup<2>(sa, nt, s); launch_k2_apply<2>(EPI_RESID, a, nt, s); break;
    case 3: launch_k2_setup<3>(sa, nt, s); launch_k2_apply<3>(EPI_RESID, a, nt, s); break;
    case 4: launch_k2_setup<4>(sa, nt, s); launch_k2_apply<4>(EPI_RESID, a, nt, s); break;
    default: launch_k2_setup<5>(sa, nt, s); launch_k2_apply<5>(EPI_RESID, a, nt, s); break;
  }
  if (cudaGetLastError() != cudaSuccess) return IGR_ECUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return IGR_ECUDA;  // the tile list is staged from host memory
  return IGR_OK;
}

// noalloc.cu — b2d_collide_substeps_noalloc: particle-collision sub-steps on
// caller-owned device arrays, with every byte of scratch memory in one
// file-scope device array, so the call itself allocates nothing.
//
// Who needs it: callers that must not allocate GPU memory once they are
// running — game and simulation frame loops that reserve all device memory
// at start-up and forbid allocation per frame (cudaMalloc can synchronise
// the device and stall the frame), and hosts that hand this library device
// buffers they own and manage themselves.
//
// The scratch array (NOALLOC_BYTES, about 3.6 MB) is part of the library's
// device image: a GPU maps it when the library's kernels are first loaded on
// it (with lazy module loading, at the first call on that device) and holds it
// until the process exits.  Every call shares it and it keeps the previous
// call's contents, so each call clears what must start at zero; calls whose
// GPU work overlaps (different streams, or host threads racing) corrupt each
// other.  The scan's cursor lives there too (cleared at the start of every
// call and by each sub-step's collide kernel); a range past the scratch
// entries would be refused and recorded
// as ERR_BIT_GRID_OVERFLOW in a scratch word (O_ERR) that a debugger can
// read, since this asynchronous call returns before the GPU work runs.
//
// The array's device address: host code cannot use the array's name (that is
// a host-side stand-in), so every call outside stream capture looks the
// address up with cudaGetSymbolAddress on the current device, which also
// stays right after a cudaDeviceReset gave the device a new context.  A call
// made while its stream is being captured reuses the address that the last
// call outside capture found on that device, because the lookup may load the
// module, which capture does not allow: make the first call on each device
// before capturing.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../../include/bendy2d.h"
#include "kernels.cuh"

namespace b2d {

void set_last_error(const std::string& msg);  // capi.cpp: message for b2d_last_error()

namespace {

constexpr uint32_t NOALLOC_MAX_PARTICLES = 65536;
constexpr uint32_t NOALLOC_MAX_BUCKETS = 2 * NOALLOC_MAX_PARTICLES;  // power of two >= 2n
constexpr uint32_t NOALLOC_MAX_CHUNKS = (NOALLOC_MAX_PARTICLES + CHUNK - 1) / CHUNK;

constexpr size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }
// layout of the scratch array
constexpr size_t O_WORLD = 0;
constexpr size_t O_CHUNKS = O_WORLD + up256(sizeof(DWorld));
constexpr size_t O_COUNT = O_CHUNKS + up256(8 * NOALLOC_MAX_CHUNKS);
constexpr size_t O_RANGE = O_COUNT + up256(4 * NOALLOC_MAX_BUCKETS);
constexpr size_t O_CURSOR = O_RANGE + up256(8 * NOALLOC_MAX_BUCKETS);
constexpr size_t O_ERR = O_CURSOR + 256;
constexpr size_t O_PBR = O_ERR + 256;
constexpr size_t O_SORTED = O_PBR + up256(8 * NOALLOC_MAX_PARTICLES);
constexpr size_t O_POS1 = O_SORTED + up256(16 * NOALLOC_MAX_PARTICLES);
constexpr size_t NOALLOC_BYTES = O_POS1 + up256(8 * NOALLOC_MAX_PARTICLES);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// device address of g_noalloc_scratch per device ordinal, as found by the
// last call outside stream capture
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};

int fail(int code, const std::string& m) {
  set_last_error(m);
  return code;
}

// one launch; returns its own status (an error left by earlier, unrelated
// work on this thread is neither reported nor cleared)
template <typename... P, typename... A>
cudaError_t launch(void (*k)(P...), uint32_t grid, uint32_t block, cudaStream_t st, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.stream = st;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

// Writes the world record and the chunk list into the scratch array; the
// parameters arrive as kernel arguments, so nothing is copied from the host.
__global__ void k_noalloc_setup(DWorld w, uint2* chunks, uint32_t nchunks, DWorld* dst) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *dst = w;
  if (i < nchunks) chunks[i] = make_uint2(0u, i * CHUNK);
}

}  // namespace

}  // namespace b2d

using namespace b2d;

extern "C" int b2d_collide_substeps_noalloc(float* d_pos_xy, float* d_prev_xy, size_t n,
                                            const b2d_noalloc_params* p, void* cuda_stream) {
  if (!p || (n && (!d_pos_xy || !d_prev_xy))) return fail(B2D_ERR_NULL, "null argument");
  if (n > NOALLOC_MAX_PARTICLES)
    return fail(B2D_ERR_CAPACITY, "b2d_collide_substeps_noalloc handles at most " +
                                      std::to_string(NOALLOC_MAX_PARTICLES) + " particles, got " +
                                      std::to_string(n));
  if (!(p->particle_radius >= 0.0f && p->grid_cell > 0.0f &&
        p->grid_cell >= 2.0f * p->particle_radius))
    return fail(B2D_ERR_ARG, "needs radius >= 0 and grid cell >= 2 * radius");
  if (n == 0 || p->sub_steps == 0) return B2D_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(B2D_ERR_CUDA, "no current CUDA device");
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess)
    return fail(B2D_ERR_CUDA, "cudaStreamIsCapturing failed on the given stream");
  unsigned char* base;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (cap == cudaStreamCaptureStatusNone) {
      void* a = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
      if (e != cudaSuccess || !a)
        return fail(B2D_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_addr[dev] = static_cast<unsigned char*>(a);
    } else if (!g_addr[dev]) {
      return fail(B2D_ERR_STATE, "the first b2d_collide_substeps_noalloc call on a device must "
                                 "come before stream capture");
    }
    base = g_addr[dev];
  }
  const uint32_t np = (uint32_t)n;
  uint32_t nb = 64;
  while (nb < 2 * np) nb <<= 1;
  const uint32_t nch = (np + CHUNK - 1) / CHUNK;
  const uint32_t nt = (nb + SCAN_SMALL_TILE - 1) / SCAN_SMALL_TILE;

  DWorld w;
  std::memset(&w, 0, sizeof(w));
  w.gx = 0.0f + p->gravity_x;  // acc = 0 + g at integrate time
  w.gy = 0.0f + p->gravity_y;
  w.bx = p->bounds_x;
  w.by = p->bounds_y;
  w.bw = p->bounds_w;
  w.bh = p->bounds_h;
  w.h = p->dt * (1.0f / (float)p->sub_steps);  // src/solver.rs:107-108
  w.radius = p->particle_radius;
  w.cell = p->grid_cell;
  w.icell = pow2_reciprocal(p->grid_cell);
  w.S = p->sub_steps;
  w.I = 1;
  w.flags = COLLIDE_PP;
  w.np = np;
  w.gb0 = 0;
  w.gmask = nb - 1;
  w.gp0 = 0;
  w.pos[0] = reinterpret_cast<float2*>(d_pos_xy);
  w.pos[1] = reinterpret_cast<float2*>(base + O_POS1);
  w.prev = reinterpret_cast<float2*>(d_prev_xy);

  DWorld* dW = reinterpret_cast<DWorld*>(base + O_WORLD);
  uint2* chunks = reinterpret_cast<uint2*>(base + O_CHUNKS);
  DGrid G;
  G.count = reinterpret_cast<uint32_t*>(base + O_COUNT);
  G.range = reinterpret_cast<uint2*>(base + O_RANGE);
  G.cursor = reinterpret_cast<uint32_t*>(base + O_CURSOR);
  G.err = reinterpret_cast<uint32_t*>(base + O_ERR);
  G.pbr = reinterpret_cast<uint2*>(base + O_PBR);
  G.sorted = reinterpret_cast<uint4*>(base + O_SORTED);
  G.nbuckets = nb;
  G.cap = np;

  auto bad = [](cudaError_t e, const char* what) {
    return fail(B2D_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  cudaError_t e = launch(k_noalloc_setup, (nch + 255) / 256, 256, st, w, chunks, nch, dW);
  if (e != cudaSuccess) return bad(e, "setup launch");
  // bucket counts start from zero (each scan clears what it read; this also
  // covers a call that stopped part-way)
  if ((e = cudaMemsetAsync(G.count, 0, (size_t)nb * 4, st)) != cudaSuccess)
    return bad(e, "clearing the bucket counts");
  if ((e = cudaMemsetAsync(G.cursor, 0, 4, st)) != cudaSuccess)
    return bad(e, "clearing the scan cursor");
  for (uint32_t s = 0; s < w.S; ++s) {
    const uint32_t cur = s & 1u;
    if ((e = launch(k_grid_count, nch, CHUNK, st, (const DWorld*)dW, G, (const uint2*)chunks, nch,
                    cur, s)) != cudaSuccess)
      return bad(e, "count launch");
    // nb <= 131072: small tiles
    if ((e = launch(k_grid_scan<1, 256>, nt, 256, st, G, nb, nt)) != cudaSuccess)
      return bad(e, "scan launch");
    if ((e = launch(k_grid_scatter, nch, CHUNK, st, (const DWorld*)dW, G, (const uint2*)chunks,
                    nch, cur, s)) != cudaSuccess)
      return bad(e, "scatter launch");
    if ((e = launch(k_collide_integrate<DGrid>, nch * COLLIDE_CTAS, COLLIDE_THREADS, st,
                    (const DWorld*)dW, G, (const uint2*)chunks, nch, cur, s)) != cudaSuccess)
      return bad(e, "collide launch");
  }
  if ((e = launch(k_copy_back, nch, CHUNK, st, (const DWorld*)dW, (const uint2*)chunks, nch,
                  (uint2*)nullptr, 0u)) != cudaSuccess)
    return bad(e, "copy-back launch");
  return B2D_OK;
}

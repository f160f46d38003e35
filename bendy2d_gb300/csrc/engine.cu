// engine.cu — device memory, work lists and the launch sequence of one
// Solver::update over every world an Engine holds.
//
// Step structure (src/solver.rs:106-116):
//  * worlds without extension collisions: every body runs the whole step
//    (all sub-steps, link iterations, bounds, integration) in one launch of
//    the group or serial executor; circles and polygons run in one CTA per
//    world (k_rigid<0>).
//  * worlds with extension collisions: per sub-step, link passes (group /
//    serial executors), circle+polygon phase, grid insert, then collide +
//    bounds + integrate; positions ping-pong between two buffers.
// The whole sequence is captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>

#include "engine.hpp"
#include "kernels.cuh"

namespace b2d {

#define B2D_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      last_error = std::string(#call) + ": " + cudaGetErrorString(e_);        \
      return ERR_CUDA;                                                        \
    }                                                                         \
  } while (0)

static uint32_t pow2ceil_u(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

static int g_smem_optin = -1;
static int g_num_sms = 0;
static constexpr uint64_t kRigidSmemCap = 96 * 1024;
// worlds with more pair tests than this run their circle/polygon phases in
// 1024-thread CTAs (k_rigid<MODE, 1024>), the others in 256-thread CTAs
static constexpr uint64_t kRigidWideTests = 4096;
static constexpr uint32_t kSerialPackBytes = 96 * 1024;  // shared memory per small-body pack
static constexpr uint32_t kSerialPackThreads = 64;       // bodies per serial pack

// Kernel launch; pdl: programmatic dependent launch — the kernel may start
// while the previous kernel in the stream finishes (it calls pdl_wait()
// before touching that kernel's results).  Returns the launch's own status.
template <typename... P, typename... A>
static cudaError_t launch_k(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                            bool pdl, A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1u : 0u;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

Engine::Engine(cudaStream_t stream) : stream_(stream) {
  if (!stream_) {
    cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
    own_stream_ = true;
  }
  for (auto& a : aux_) cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking);
  for (auto& a : lx_) cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking);
  evpool_.resize(256);
  for (auto& e : evpool_) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  if (g_smem_optin < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    g_smem_optin = v;
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    for (auto fn : {k_rigid<0, 256>, k_rigid<1, 256>, k_rigid<2, 256>, k_rigid<3, 256>,
                    k_rigid<0, 1024>, k_rigid<1, 1024>, k_rigid<2, 1024>, k_rigid<3, 1024>})
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRigidSmemCap);
    for (auto fn : {k_exec_serial_smem<true, false>, k_exec_serial_smem<false, false>,
                    k_exec_serial_smem<true, true>, k_exec_serial_smem<false, true>})
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
    for (auto fn : {k_exec_large<true, true>, k_exec_large<false, true>,
                    k_exec_large<true, false>, k_exec_large<false, false>})
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
    for (auto fn : {k_exec_large<true, true>, k_exec_large<false, true>})
      cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (auto fn : {k_exec_groups<true, true, false>, k_exec_groups<false, true, false>,
                    k_exec_groups<true, false, false>, k_exec_groups<false, false, false>,
                    k_exec_groups<true, true, true>, k_exec_groups<false, true, true>})
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  }
  tune_.res_max = std::min<uint32_t>(tune_.res_max, (uint32_t)std::max(g_smem_optin, 48 * 1024));
  tune_.smem_max = std::min<uint32_t>(
      tune_.smem_max, (uint32_t)std::max(g_smem_optin - (int)STREAM_BYTES, 16 * 1024));
}

Engine::~Engine() {
  if (graph_) cudaGraphExecDestroy(graph_);
  cudaStreamSynchronize(stream_);
  for (Slot& s : slots_)
    if (s.block) cudaFree(s.block);
  cudaFree(d_worlds_);
  cudaFree(d_scheds_);
  cudaFree(d_chunk_off_);
  cudaFree(d_chunk_len_);
  cudaFree(d_stream_);
  cudaFree(d_err_);
  cudaFree(d_lists_);
  cudaFree(d_wlists_);
  cudaFree(d_grid_);
  for (auto& e : evpool_) cudaEventDestroy(e);
  for (auto& a : aux_) cudaStreamDestroy(a);
  for (auto& a : lx_) cudaStreamDestroy(a);
  if (ist_) cudaStreamDestroy(ist_);
  if (own_stream_) cudaStreamDestroy(stream_);
}

int Engine::install_beside(bool on) {
  if (on && !ist_) B2D_CUDA(cudaStreamCreateWithFlags(&ist_, cudaStreamNonBlocking));
  beside_ = on;
  return OK;
}

void Engine::invalidate_graph() {
  if (graph_) {
    cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
  }
  graph_valid_ = false;
  stable_steps_ = 0;
}

void Engine::set_stream(cudaStream_t s) {
  cudaStreamSynchronize(stream_);
  if (own_stream_) cudaStreamDestroy(stream_);
  own_stream_ = false;
  stream_ = s;
  if (!stream_) {
    cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
    own_stream_ = true;
  }
  invalidate_graph();
}

void Engine::set_tuning(const PlanTuning& t) {
  const uint32_t cap = tune_.smem_max, rcap = tune_.res_max;
  tune_ = t;
  tune_.smem_max = std::min(tune_.smem_max, cap);  // device limits found at start-up
  tune_.res_max = std::min(tune_.res_max, rcap);
  lists_dirty_ = true;
}

const WorldImage* Engine::image(uint32_t slot) const {
  if (slot >= slots_.size() || !slots_[slot].live) return nullptr;
  return &slots_[slot].img;
}

int Engine::ensure_table(size_t n) {
  if (n <= worlds_cap_) return OK;
  size_t cap = std::max<size_t>(n, worlds_cap_ * 2 + 4);
  DWorld* d = nullptr;
  B2D_CUDA(cudaMalloc(&d, cap * sizeof(DWorld)));
  if (d_worlds_) {
    B2D_CUDA(cudaMemcpyAsync(d, d_worlds_, worlds_cap_ * sizeof(DWorld), cudaMemcpyDeviceToDevice, stream_));
    B2D_CUDA(cudaStreamSynchronize(stream_));
    cudaFree(d_worlds_);
  }
  d_worlds_ = d;
  worlds_cap_ = cap;
  invalidate_graph();
  return OK;
}

int Engine::fill_world_record(uint32_t slot) {
  Slot& s = slots_[slot];
  DWorld W = s.img.params;
  const BlockLayout& L = s.L;
  unsigned char* b = s.block;
  W.pos[0] = reinterpret_cast<float2*>(b + L.o_pos);
  W.pos[1] = reinterpret_cast<float2*>(b + L.o_pos1);
  W.prev = reinterpret_cast<float2*>(b + L.o_prev);
  W.bodies = reinterpret_cast<DBody*>(b + L.o_bodies);
  W.bidx = reinterpret_cast<uint32_t*>(b + L.o_bidx);
  W.lab = reinterpret_cast<uint2*>(b + L.o_lab);
  W.lrest = reinterpret_cast<float*>(b + L.o_lrest);
  W.lstiff = reinterpret_cast<float*>(b + L.o_lstiff);
  W.cpos = reinterpret_cast<float2*>(b + L.o_cpos);
  W.cprev = reinterpret_cast<float2*>(b + L.o_cprev);
  W.cacc = reinterpret_cast<float2*>(b + L.o_cacc);
  W.crad = reinterpret_cast<float*>(b + L.o_crad);
  W.cstatic = reinterpret_cast<uint32_t*>(b + L.o_cstatic);
  W.clab = reinterpret_cast<uint2*>(b + L.o_clab);
  W.clrest = reinterpret_cast<float*>(b + L.o_clrest);
  W.polys = reinterpret_cast<DPoly*>(b + L.o_polys);
  W.vpos = reinterpret_cast<float2*>(b + L.o_vpos);
  W.vprev = reinterpret_cast<float2*>(b + L.o_vprev);
  W.vacc = reinterpret_cast<float2*>(b + L.o_vacc);
  W.pcenter = reinterpret_cast<float2*>(b + L.o_pcenter);
  W.paabb = reinterpret_cast<float4*>(b + L.o_paabb);
  W.plab = reinterpret_cast<uint2*>(b + L.o_plab);
  W.plrest = reinterpret_cast<float*>(b + L.o_plrest);
  W.stage_off = reinterpret_cast<uint32_t*>(b + L.o_stage);
  W.stage_pr = reinterpret_cast<uint32_t*>(b + L.o_stage_pr);
  W.h = s.dt * (1.0f / (float)W.S);  // src/solver.rs:107-108
  if (h_worlds_.size() <= slot) h_worlds_.resize(slot + 1);
  h_worlds_[slot] = W;
  int st = ensure_table(slots_.size());
  if (st != OK) return st;
  B2D_CUDA(cudaMemcpyAsync(d_worlds_ + slot, &h_worlds_[slot], sizeof(DWorld),
                           cudaMemcpyHostToDevice, up_stream()));
  return OK;
}

int Engine::add(WorldHost* w, uint32_t* out_slot, std::string* why) {
  WorldImage img;
  const int st = plan(*w, &img, why);
  if (st != OK) return st;
  return add_planned(w, std::move(img), out_slot);
}

int Engine::plan(const WorldHost& w, WorldImage* img, std::string* why) {
  return plan_world(w, tune_, reg_, *img, why);
}

int Engine::set_fault(int kind, uint64_t value) {
  switch (kind) {
    case FAULT_WAIT_TIMEOUT:
      fault_bits_ = value ? (fault_bits_ | FAULT_BIT_WAIT) : (fault_bits_ & ~FAULT_BIT_WAIT);
      break;
    case FAULT_GRID_CAP:
      fault_grid_cap_ = (uint32_t)std::min<uint64_t>(value, 0xFFFFFFFFu);
      break;
    case FAULT_ALLOC:
      fault_alloc_ = value;
      return OK;  // host side only: the launch sequence is unchanged
    default:
      last_error = "unknown fault kind " + std::to_string(kind);
      return ERR_ARG;
  }
  invalidate_graph();  // the kernels' parameters change
  return OK;
}

// The world block is allocated and uploaded before a slot is taken, so a
// failed allocation or copy leaves the engine as it was.
int Engine::add_planned(WorldHost* w, WorldImage&& img, uint32_t* out_slot) {
  const BlockLayout L = layout_of(img);
  unsigned char* block = nullptr;
  if (fault_alloc_ > 0) {
    --fault_alloc_;
    last_error = "cudaMallocAsync: injected allocation failure";
    return ERR_CUDA;
  }
  const cudaStream_t up = up_stream();
  B2D_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&block), L.total, up));
  std::vector<unsigned char> stage(L.total);
  write_block(img, L, stage.data());
  cudaError_t ce = cudaMemcpyAsync(block, stage.data(), L.total, cudaMemcpyHostToDevice, up);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(up);  // the staging buffer is pageable
  if (ce != cudaSuccess) {
    last_error = std::string("uploading a world block: ") + cudaGetErrorString(ce);
    cudaFreeAsync(block, up);
    return ERR_CUDA;
  }
  uint32_t slot;
  if (!free_slots_.empty()) {
    slot = free_slots_.back();
    free_slots_.pop_back();
  } else {
    slot = (uint32_t)slots_.size();
    slots_.emplace_back();
  }
  Slot& s = slots_[slot];
  s.img = std::move(img);
  s.host = w;
  s.L = L;
  s.block = block;
  s.live = true;
  dev_bytes_ += L.total;
  lists_dirty_ = true;
  int st = fill_world_record(slot);
  // beside a step in flight: the record must have landed before the next
  // step, which the caller launches on the main stream
  if (st == OK && beside_ && cudaStreamSynchronize(ist_) != cudaSuccess) {
    last_error = "uploading a world record";
    st = ERR_CUDA;
  }
  if (st != OK) {
    remove(slot);
    return st;
  }
  *out_slot = slot;
  return OK;
}

int Engine::remove(uint32_t slot) {
  if (slot >= slots_.size() || !slots_[slot].live) return ERR_INDEX;
  Slot& s = slots_[slot];
  // An engine that installs beside its steps frees on the install stream,
  // so that a later install reusing the block has no cross-stream wait on
  // a step in flight (the pool would otherwise order the reuse after the
  // main stream); its callers remove a world only once no launched step
  // uses it (the server: after the tick's synchronisation).
  B2D_CUDA(cudaFreeAsync(s.block, ist_ ? ist_ : stream_));
  dev_bytes_ -= s.L.total;
  s = Slot();
  free_slots_.push_back(slot);
  lists_dirty_ = true;
  return OK;
}

int Engine::set_dt(uint32_t slot, float dt) {
  if (slot >= slots_.size() || !slots_[slot].live) return ERR_INDEX;
  Slot& s = slots_[slot];
  if (s.dt == dt && h_worlds_[slot].h == dt * (1.0f / (float)h_worlds_[slot].S)) return OK;
  s.dt = dt;
  h_worlds_[slot].h = dt * (1.0f / (float)h_worlds_[slot].S);  // src/solver.rs:107-108
  B2D_CUDA(cudaMemcpyAsync(&d_worlds_[slot].h, &h_worlds_[slot].h, sizeof(float),
                           cudaMemcpyHostToDevice, up_stream()));
  B2D_CUDA(cudaStreamSynchronize(up_stream()));
  return OK;
}

int Engine::set_params(uint32_t slot) {
  if (slot >= slots_.size() || !slots_[slot].live) return ERR_INDEX;
  Slot& s = slots_[slot];
  const WorldHost& w = *s.host;
  DWorld& W = h_worlds_[slot];
  W.gx = 0.0f + w.gravity.x;
  W.gy = 0.0f + w.gravity.y;
  W.bx = w.bounds.pos.x;
  W.by = w.bounds.pos.y;
  W.bw = w.bounds.size.x;
  W.bh = w.bounds.size.y;
  s.img.params.gx = W.gx; s.img.params.gy = W.gy;
  s.img.params.bx = W.bx; s.img.params.by = W.by;
  s.img.params.bw = W.bw; s.img.params.bh = W.bh;
  B2D_CUDA(cudaMemcpyAsync(d_worlds_ + slot, &W, sizeof(DWorld), cudaMemcpyHostToDevice, stream_));
  B2D_CUDA(cudaStreamSynchronize(stream_));
  return OK;
}

int Engine::upload_registry() {
  if (!d_err_) {
    B2D_CUDA(cudaMalloc(&d_err_, 16));
    B2D_CUDA(cudaMemsetAsync(d_err_, 0, 16, stream_));
    invalidate_graph();
  }
  auto grow = [&](uint32_t*& ptr, size_t& cap, size_t need, size_t elem) -> int {
    if (need <= cap) return OK;
    size_t nc = std::max(need, cap * 2 + 1024);
    void* d = nullptr;
    B2D_CUDA(cudaMalloc(&d, nc * elem));
    B2D_CUDA(cudaStreamSynchronize(stream_));
    cudaFree(ptr);
    ptr = static_cast<uint32_t*>(d);
    cap = nc;
    invalidate_graph();
    return OK;
  };
  bool grew = false;
  int st;
  if (reg_.scheds.size() > scheds_cap_) {
    size_t nc = std::max(reg_.scheds.size(), scheds_cap_ * 2 + 64);
    DSched* d = nullptr;
    B2D_CUDA(cudaMalloc(&d, nc * sizeof(DSched)));
    B2D_CUDA(cudaStreamSynchronize(stream_));
    cudaFree(d_scheds_);
    d_scheds_ = d;
    scheds_cap_ = nc;
    grew = true;
    invalidate_graph();
  }
  if (reg_.chunk_off.size() > chunks_cap_) {
    size_t cap2 = chunks_cap_;
    if ((st = grow(d_chunk_off_, chunks_cap_, reg_.chunk_off.size(), 4)) != OK) return st;
    if ((st = grow(d_chunk_len_, cap2, reg_.chunk_len.size(), 4)) != OK) return st;
    grew = true;
  }
  if (reg_.stream.size() > stream_cap_) {
    if ((st = grow(d_stream_, stream_cap_, reg_.stream.size(), 4)) != OK) return st;
    grew = true;
  }
  if (grew) reg_.uploaded_scheds = reg_.uploaded_chunks = reg_.uploaded_stream = 0;
  auto put = [&](void* dst, const void* src, size_t from, size_t to, size_t elem) -> int {
    if (to > from)
      B2D_CUDA(cudaMemcpyAsync(static_cast<unsigned char*>(dst) + from * elem,
                               static_cast<const unsigned char*>(src) + from * elem,
                               (to - from) * elem, cudaMemcpyHostToDevice, stream_));
    return OK;
  };
  if ((st = put(d_scheds_, reg_.scheds.data(), reg_.uploaded_scheds, reg_.scheds.size(), sizeof(DSched))) != OK) return st;
  if ((st = put(d_chunk_off_, reg_.chunk_off.data(), reg_.uploaded_chunks, reg_.chunk_off.size(), 4)) != OK) return st;
  if ((st = put(d_chunk_len_, reg_.chunk_len.data(), reg_.uploaded_chunks, reg_.chunk_len.size(), 4)) != OK) return st;
  if ((st = put(d_stream_, reg_.stream.data(), reg_.uploaded_stream, reg_.stream.size(), 4)) != OK) return st;
  const bool any = reg_.uploaded_scheds != reg_.scheds.size() ||
                   reg_.uploaded_stream != reg_.stream.size();
  reg_.uploaded_scheds = reg_.scheds.size();
  reg_.uploaded_chunks = reg_.chunk_off.size();
  reg_.uploaded_stream = reg_.stream.size();
  if (any) B2D_CUDA(cudaStreamSynchronize(stream_));
  return OK;
}

int Engine::check_device_error() {
  if (!d_err_) return OK;
  uint32_t e = 0;
  B2D_CUDA(cudaMemcpyAsync(&e, d_err_, 4, cudaMemcpyDeviceToHost, stream_));
  B2D_CUDA(cudaStreamSynchronize(stream_));
  if (e) {
    grid_reset_ = true;
    B2D_CUDA(cudaMemsetAsync(d_err_, 0, 4, stream_));
    last_error = "device error word " + std::to_string(e) +
                 ((e & ERR_BIT_TMA_TIMEOUT) ? " (a bulk-copy wait timed out)" : "") +
                 ((e & ERR_BIT_GRID_OVERFLOW) ? " (grid entries past their capacity)" : "");
    return ERR_DEVICE;
  }
  return OK;
}

int Engine::ensure_grid(size_t nbuckets, size_t np_pp) {
  // Slot inserts skip the scan and scatter launches but spread the entries
  // over GRID_SLOTS fixed slots per bucket: on GB300 that wins up to a few
  // hundred thousand particles (65,536 scattered cloth particles: 0.544 ->
  // 0.518 ms per update; 131,072: 0.728 -> 0.579), while for a million
  // particles packed on a lattice the sparse slots cost the collide pass
  // more than the two launches (5.91 -> 6.28 ms).
  // (A grid in one form keeps it until the particle count is well past the
  // threshold, so that a serving pool near it does not reallocate each step.)
  const uint64_t lim = tune_.grid_slot_max;
  const bool slotted = !d_grid_ ? np_pp <= lim
                       : grid_slotted_ ? np_pp <= lim
                                       : (uint64_t)np_pp * 2 <= lim;
  if (nbuckets <= grid_.nbuckets && np_pp <= grid_np_ && d_grid_ && slotted == grid_slotted_)
    return OK;
  const size_t nb = std::max(nbuckets, (size_t)grid_.nbuckets);
  const size_t np = std::max<size_t>(std::max(np_pp, grid_np_), 1);
  size_t bytes = 0;
  auto seg = [&](size_t b) { size_t at = bytes; bytes = (bytes + b + 255) & ~(size_t)255; return at; };
  size_t o[5];
  if (slotted) {  // cell words (2 parities), cursor | slots, overflow entries, overflow links
    o[0] = seg(nb * 16);
    o[1] = seg(4);
    o[2] = seg(nb * GRID_SLOTS * 16);
    o[3] = seg(np * 16);
    o[4] = seg(np * 4);
  } else {        // counts, ranges, cursor | (bucket, rank) per particle, sorted entries
    o[0] = seg(nb * 4);
    o[1] = seg(nb * 8);
    o[2] = seg(4);
    o[3] = seg(np * 8);
    o[4] = seg(np * 16);
  }
  B2D_CUDA(cudaStreamSynchronize(stream_));
  if (d_grid_) dev_bytes_ -= grid_bytes_;
  cudaFree(d_grid_);
  d_grid_ = nullptr;
  grid_ = DGrid{};
  gslots_ = DSlots{};
  B2D_CUDA(cudaMalloc(&d_grid_, bytes));
  B2D_CUDA(cudaMemset(d_grid_, 0, bytes));
  if (slotted) {
    gslots_.cell = reinterpret_cast<uint2*>(d_grid_ + o[0]);
    gslots_.cursor = reinterpret_cast<uint32_t*>(d_grid_ + o[1]);
    gslots_.slot = reinterpret_cast<uint4*>(d_grid_ + o[2]);
    gslots_.ovf = reinterpret_cast<uint4*>(d_grid_ + o[3]);
    gslots_.ovf_next = reinterpret_cast<uint32_t*>(d_grid_ + o[4]);
    gslots_.nbuckets = (uint32_t)nb;
    gslots_.cap = (uint32_t)np;
    grid_head_bytes_ = o[2];
  } else {
    grid_.count = reinterpret_cast<uint32_t*>(d_grid_ + o[0]);
    grid_.range = reinterpret_cast<uint2*>(d_grid_ + o[1]);
    grid_.cursor = reinterpret_cast<uint32_t*>(d_grid_ + o[2]);
    grid_.pbr = reinterpret_cast<uint2*>(d_grid_ + o[3]);
    grid_.sorted = reinterpret_cast<uint4*>(d_grid_ + o[4]);
    grid_head_bytes_ = o[3];
  }
  // the bucket count (both forms) is read back through grid_.nbuckets
  grid_.nbuckets = (uint32_t)nb;
  grid_.cap = (uint32_t)np;
  grid_slotted_ = slotted;
  grid_np_ = np;
  grid_bytes_ = bytes;
  grid_reset_ = false;
  dev_bytes_ += bytes;
  invalidate_graph();
  return OK;
}

// First-fit decreasing: bodies sorted by size, each into the first pack with
// room (bytes and threads).  Bodies larger than a pack stay in `rest` for the
// global-memory serial kernel.
// Serial packs.  The step time of a batch of chain-like bodies follows its
// longest chains.  A body whose chain is at least stage_frac (default 2/3)
// of the longest gets a pack of its own with the links staged too (8 or 16 B
// per particle plus 16 B per link, up to the shared-memory limit; at most
// one per SM; allow_large): staging cuts a link from ~333 to ~211 cycles, so
// shorter chains finish in time without it and leave the SMs' shared memory
// to the packs of many bodies (positions only, first-fit decreasing, up to
// kSerialPackBytes and kSerialPackThreads bodies).  What fits neither stays
// in `rest` for the global-memory serial kernel.
void Engine::build_packs(std::vector<uint2>& in, bool full, SerialPacks* out,
                         std::vector<uint2>& rest, bool allow_large) {
  const uint32_t per = full ? 16u : 8u;
  auto body = [&](const uint2& it) -> const DBody& { return slots_[it.x].img.bodies[it.y]; };
  auto bytes_of = [&](const uint2& it) { return body(it).np * per + body(it).nl * 16u; };
  std::stable_sort(in.begin(), in.end(),
                   [&](const uint2& a, const uint2& b) { return bytes_of(a) > bytes_of(b); });
  const uint32_t large_cap = allow_large ? (uint32_t)g_smem_optin : 0u;
  size_t n_large = 0;
  const size_t max_large = (size_t)std::max(g_num_sms, 1);
  uint64_t max_links = 0;
  for (const uint2& it : in) max_links = std::max<uint64_t>(max_links, (uint64_t)body(it).nl);
  auto long_chain = [&](const uint2& it) {
    return (double)body(it).nl >= (double)tune_.stage_frac * (double)max_links;
  };
  std::vector<std::vector<uint2>> bins;
  std::vector<uint32_t> used;
  size_t first_open = 0;
  auto emit = [&](SerialPacks& o, const std::vector<uint2>& bin, bool staged) {
    o.packs.push_back(make_uint2((uint32_t)o.items.size(), (uint32_t)bin.size()));
    uint32_t pb = 0, lb = 0;
    for (const uint2& it : bin) {
      o.items.push_back(it);
      o.base.push_back(make_uint2(pb, lb));
      pb += body(it).np;
      lb += body(it).nl;
    }
    o.max_bytes = std::max(o.max_bytes, pb * per + (staged ? lb * 16u : 0u));
  };
  for (const uint2& it : in) {
    if (n_large < max_large && long_chain(it) && bytes_of(it) <= large_cap) {  // longest chains
      emit(out[1], std::vector<uint2>{it}, true);
      ++n_large;
      continue;
    }
    const uint32_t bytes = body(it).np * per;
    if (bytes > kSerialPackBytes) {
      rest.push_back(it);
      continue;
    }
    size_t k = first_open;
    while (k < bins.size() && (used[k] + bytes > kSerialPackBytes ||
                               bins[k].size() >= kSerialPackThreads))
      ++k;
    if (k == bins.size()) {
      bins.emplace_back();
      used.push_back(0);
    }
    bins[k].push_back(it);
    used[k] += bytes;
    while (first_open < bins.size() && bins[first_open].size() >= kSerialPackThreads) ++first_open;
  }
  for (const auto& bin : bins) emit(out[0], bin, false);
}

int Engine::rebuild_lists() {
  classes_.clear();
  serial_full_.clear();
  serial_links_.clear();
  for (int k = 0; k < 2; ++k) packs_full_[k] = packs_links_[k] = SerialPacks();
  std::vector<uint2> sfull_all, slinks_all;
  chunks_.clear();
  rigid_full_.clear();
  rigid_ext_.clear();
  rigid_wide_full_ = rigid_wide_ext_ = false;
  smax_ext_ = 0;
  any_odd_ext_ = false;
  any_pp_ = false;
  any_count_ = false;
  size_t np_ext = 0;
  size_t nbuckets = 0, np_pp = 0;
  uint64_t rigid_smem = 0;
  // Launch classes: group bodies with the same group size and kind, binned by
  // shared bytes per group in powers of two; a class is sized to its largest
  // member.  Few classes matter: each is a launch whose level chain costs a
  // full link-phase latency.
  std::map<std::tuple<uint32_t, bool, bool, bool, uint32_t>, size_t> cls;
  auto log2c = [](uint32_t x) {
    uint32_t b = 0;
    while (b < 31 && (1u << b) < x) ++b;
    return b;
  };
  // A resident schedule takes most of an SM's shared memory (a 32x32 cloth:
  // ~170 KB, one body per SM) where a streamed one leaves room for about
  // three.  Resident schedules win when a launch has no more bodies than SMs
  // (each body's level chain is the critical path); larger launches are
  // throughput-bound and stream.
  std::map<std::tuple<uint32_t, bool, uint32_t>, size_t> res_count;
  for (const Slot& s : slots_)
    if (s.live)
      for (const GroupBody& gb : s.img.groups)
        if (gb.res) ++res_count[std::make_tuple(gb.T, !s.img.ext, log2c(gb.region + gb.res))];
  wlaunch_.assign(slots_.size(), WorldLaunch());
  // world records whose grid ranges moved (a world joined or left before
  // them) go up in one copy after the loop: one pageable copy per record
  // waited for the stream each time (~2 ms per step for 640 worlds)
  uint32_t rec_lo = UINT32_MAX, rec_hi = 0;
  for (uint32_t si = 0; si < slots_.size(); ++si) {
    const Slot& s = slots_[si];
    if (!s.live) continue;
    const WorldImage& im = s.img;
    const bool full = !im.ext;
    std::vector<size_t> cls_before(classes_.size());
    for (size_t c = 0; c < classes_.size(); ++c) cls_before[c] = classes_[c].items.size();
    wlaunch_[si].sf0 = (uint32_t)serial_full_.size();
    wlaunch_[si].pk0 = (uint32_t)packs_full_[0].packs.size();
    for (const GroupBody& gb : im.groups) {
      const bool use_res =
          gb.res && res_count[std::make_tuple(gb.T, full, log2c(gb.region + gb.res))] <=
                        (size_t)std::max(g_num_sms, 1);
      // large-body classes are keyed by their cluster layout instead of a bin
      const uint32_t bin = gb.large_c ? (0x10000u | (gb.large_c << 8) | gb.log2per)
                           : gb.smem ? log2c(gb.region + (use_res ? gb.res : 0u)) : 0u;
      auto key = std::make_tuple(gb.T, gb.smem, full, use_res, bin);
      auto it = cls.find(key);
      if (it == cls.end()) {
        LaunchClass c;
        c.T = gb.T;
        c.smem = gb.smem;
        c.full = full;
        c.region = 0;
        c.res = 0;
        c.fill = 0;
        c.words = 0;
        c.G = 1;
        c.large_c = gb.large_c;
        c.log2per = gb.log2per;
        it = cls.emplace(key, classes_.size()).first;
        classes_.push_back(std::move(c));
      }
      LaunchClass& c = classes_[it->second];
      if (gb.smem) c.region = std::max(c.region, gb.region);
      if (use_res) c.res = std::max(c.res, gb.res);
      c.words = std::max(c.words, reg_.scheds[im.bodies[gb.body].sched].words);
      c.items.push_back(make_uint2(si, gb.body));
    }
    if (plain_ && full) {  // plain mode: this world's own packs
      std::vector<uint2> mine;
      for (uint32_t b : im.serials) mine.push_back(make_uint2(si, b));
      build_packs(mine, true, packs_full_, serial_full_, false);  // small packs only
    } else {
      for (uint32_t b : im.serials) (full ? sfull_all : slinks_all).push_back(make_uint2(si, b));
    }
    wlaunch_[si].sfn = (uint32_t)serial_full_.size() - wlaunch_[si].sf0;
    wlaunch_[si].pkn = (uint32_t)packs_full_[0].packs.size() - wlaunch_[si].pk0;
    for (size_t c = 0; c < classes_.size(); ++c) {
      const size_t before = c < cls_before.size() ? cls_before[c] : 0;
      if (classes_[c].items.size() > before)
        wlaunch_[si].cls.emplace_back((uint32_t)before,
                                      (uint32_t)(classes_[c].items.size() - before));
      else
        wlaunch_[si].cls.emplace_back(0u, 0u);
    }
    const bool rigid = im.params.nc > 0 || im.params.ng > 0;
    // pair tests of the world's speculative loops: circle pairs and
    // (edge, vertex) tests of every ordered polygon pair
    const uint64_t rigid_tests =
        (uint64_t)im.cpos.size() * (im.cpos.size() > 0 ? im.cpos.size() - 1 : 0) / 2 +
        (im.stage_off.empty() ? 0 : im.stage_off.back());
    const bool wide = rigid_tests > kRigidWideTests;
    if (rigid) {
      const uint64_t ng = im.polys.size(), nc = im.cpos.size(), nv = im.vpos.size();
      // same expression as rigid_smem_bytes() in kernels.cuh
      const uint64_t need = 48 * ng + 28 * nc + 12 * im.clab.size() + 24 * nv +
                            12 * im.plab.size() + 8 * im.stage_off.size() + 272;
      if (need <= kRigidSmemCap) rigid_smem = std::max<uint64_t>(rigid_smem, need);
    }
    if (full) {
      if (rigid) {
        wlaunch_[si].rigid = (int32_t)rigid_full_.size();
        wlaunch_[si].rigid_wide = wide;
        rigid_full_.push_back(si);
        rigid_wide_full_ |= wide;
      }
    } else {
      if (rigid) {
        rigid_ext_.push_back(si);
        rigid_wide_ext_ |= wide;
      }
      smax_ext_ = std::max(smax_ext_, im.params.S);
      any_odd_ext_ |= (im.params.S & 1u) != 0u;
      if (im.params.flags & COLLIDE_PP) {
        any_pp_ = true;
        // this world's bucket range: a power of two >= 2 x its particles
        const uint32_t nbw = pow2ceil_u(std::max<uint32_t>(
            (uint32_t)(tune_.bucket_factor * (float)im.params.np), 64u));
        if (!(im.params.flags & GRID_IN_LINKS)) any_count_ = true;
        if (h_worlds_[si].gb0 != (uint32_t)nbuckets || h_worlds_[si].gmask != nbw - 1 ||
            h_worlds_[si].gp0 != (uint32_t)np_pp) {
          h_worlds_[si].gb0 = (uint32_t)nbuckets;
          h_worlds_[si].gmask = nbw - 1;
          h_worlds_[si].gp0 = (uint32_t)np_pp;
          rec_lo = std::min(rec_lo, si);
          rec_hi = std::max(rec_hi, si);
        }
        nbuckets += nbw;
        np_pp += im.params.np;
      }
      for (uint32_t st = 0; st < im.params.np; st += CHUNK) chunks_.push_back(make_uint2(si, st));
      np_ext += im.params.np;
    }
  }
  // h_worlds_ mirrors the device table, so the records between two moved
  // ones can go up with them
  if (rec_lo <= rec_hi)
    B2D_CUDA(cudaMemcpyAsync(d_worlds_ + rec_lo, &h_worlds_[rec_lo],
                             (size_t)(rec_hi - rec_lo + 1) * sizeof(DWorld),
                             cudaMemcpyHostToDevice, stream_));
  // size each class to its largest member; a resident class whose largest
  // body and largest schedule do not fit together streams instead
  for (LaunchClass& c : classes_) {
    if (c.large_c) continue;  // one body per cluster, shared memory set by its layout
    if (c.res && (size_t)c.region + c.res + GROUP_TAIL_BYTES > (size_t)g_smem_optin) c.res = 0;
    // streamed: one 16 KB chunk per fill, or for launches with no more bodies
    // than SMs (latency-bound) the largest fills that fit beside the body,
    // which cuts the buffer switches of long schedules
    c.fill = STREAM_BUF_BYTES / 2;
    if (!c.res && c.items.size() <= (size_t)std::max(g_num_sms, 1)) {
      const uint32_t room = ((uint32_t)g_smem_optin - c.region - GROUP_TAIL_BYTES) / 2 & ~15u;
      const uint32_t want = (c.words * 4u + 15u) & ~15u;
      c.fill = std::max(c.fill, std::min(room, want));
    }
    const uint32_t per_group = c.region + (c.res ? c.res : 2 * c.fill) + GROUP_TAIL_BYTES;
    uint32_t G = c.T == 32 ? tune_.warp_groups : std::max<uint32_t>(1, 256 / c.T);
    if (c.T != 32) G = std::min<uint32_t>(G, std::min<uint32_t>(tune_.max_groups, 15));
    G = std::max<uint32_t>(G, 1);
    c.G = std::max<uint32_t>(1, std::min<uint32_t>(G, (uint32_t)g_smem_optin / per_group));
  }
  if (!plain_) build_packs(sfull_all, true, packs_full_, serial_full_, true);
  build_packs(slinks_all, false, packs_links_, serial_links_, true);
  // sort serial items longest first (load balance)
  auto serial_cost = [&](const uint2& a) {
    const DBody& B = slots_[a.x].img.bodies[a.y];
    return (uint64_t)B.nl * slots_[a.x].img.params.I + B.np;
  };
  if (!plain_)  // plain mode keeps each world's serial bodies contiguous
    std::stable_sort(serial_full_.begin(), serial_full_.end(),
                     [&](const uint2& a, const uint2& b) { return serial_cost(a) > serial_cost(b); });
  std::stable_sort(serial_links_.begin(), serial_links_.end(),
                   [&](const uint2& a, const uint2& b) { return serial_cost(a) > serial_cost(b); });
  // upload lists
  std::vector<uint2> all;
  for (LaunchClass& c : classes_) {
    c.dev_off = all.size();
    all.insert(all.end(), c.items.begin(), c.items.end());
  }
  off_serial_full_ = all.size();
  all.insert(all.end(), serial_full_.begin(), serial_full_.end());
  off_serial_links_ = all.size();
  all.insert(all.end(), serial_links_.begin(), serial_links_.end());
  off_chunks_ = all.size();
  all.insert(all.end(), chunks_.begin(), chunks_.end());
  for (SerialPacks* sp : {&packs_full_[0], &packs_full_[1], &packs_links_[0], &packs_links_[1]}) {
    sp->off_items = all.size();
    all.insert(all.end(), sp->items.begin(), sp->items.end());
    sp->off_packs = all.size();
    all.insert(all.end(), sp->packs.begin(), sp->packs.end());
    sp->off_base = all.size();
    all.insert(all.end(), sp->base.begin(), sp->base.end());
  }
  std::vector<uint32_t> wl(rigid_full_);
  off_rigid_ext_ = wl.size();
  wl.insert(wl.end(), rigid_ext_.begin(), rigid_ext_.end());
  if (all.size() > lists_cap_) {
    B2D_CUDA(cudaStreamSynchronize(stream_));
    cudaFree(d_lists_);
    lists_cap_ = std::max(all.size(), lists_cap_ * 2 + 64);
    B2D_CUDA(cudaMalloc(&d_lists_, lists_cap_ * sizeof(uint2)));
  }
  if (wl.size() > wlists_cap_) {
    B2D_CUDA(cudaStreamSynchronize(stream_));
    cudaFree(d_wlists_);
    wlists_cap_ = std::max(wl.size(), wlists_cap_ * 2 + 64);
    B2D_CUDA(cudaMalloc(&d_wlists_, wlists_cap_ * sizeof(uint32_t)));
  }
  if (!all.empty())
    B2D_CUDA(cudaMemcpyAsync(d_lists_, all.data(), all.size() * sizeof(uint2), cudaMemcpyHostToDevice, stream_));
  if (!wl.empty())
    B2D_CUDA(cudaMemcpyAsync(d_wlists_, wl.data(), wl.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_));
  B2D_CUDA(cudaStreamSynchronize(stream_));
  collide_per_particle_ = np_ext >= tune_.collide_thread_min;
  if (nbuckets > 0) {
    int st = ensure_grid(nbuckets, np_pp);
    if (st != OK) return st;
  }
  grid_used_ = (uint32_t)nbuckets;
  rigid_smem_ = (uint32_t)rigid_smem;
  lists_dirty_ = false;
  invalidate_graph();
  return OK;
}

int Engine::launch_all(bool profiling) {
  launches_ = 0;
  prof_.clear();
  // the first failed launch of this step (launch_k reports each launch's own
  // status; the <<<>>> launches are covered by cudaGetLastError at the end)
  cudaError_t launch_err = cudaSuccess;
  auto lk = [&](cudaError_t e) {
    if (e != cudaSuccess && launch_err == cudaSuccess) launch_err = e;
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (profiling) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
  }
  auto timed = [&](const char* name, auto&& fn, bool kernel = true) {
    if (profiling) cudaEventRecord(e0, stream_);
    fn();
    if (kernel) ++launches_;
    if (profiling) {
      cudaEventRecord(e1, stream_);
      cudaEventSynchronize(e1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      bool found = false;
      for (auto& p : prof_)
        if (p.first == name) { p.second += ms; found = true; }
      if (!found) prof_.emplace_back(name, ms);
    }
  };
  const DScheds SC{d_scheds_, d_chunk_off_, d_chunk_len_, d_stream_, d_err_, fault_bits_};
  grid_.err = d_err_;
  gslots_.err = d_err_;
  // as launched: the capacity (sorted entries, or overflow entries of the
  // slotted grid) may be lowered by FAULT_GRID_CAP
  DGrid GR = grid_;
  DSlots GS = gslots_;
  if (fault_grid_cap_ && fault_grid_cap_ < GR.cap) GR.cap = fault_grid_cap_;
  if (fault_grid_cap_ && fault_grid_cap_ < GS.cap) GS.cap = fault_grid_cap_;
  const DWorld* W = d_worlds_;
  // Streams: link executors, grid and collide kernels run on the main
  // stream; circle/polygon kernels on aux streams (graph branches), joined
  // before the collide kernel that reads them.  Profiling runs serially.
  cudaStream_t ax = profiling ? stream_ : aux_[0];
  cudaStream_t ax2 = profiling ? stream_ : aux_[1];
  uint32_t evi = 0;
  auto edge = [&](cudaStream_t a, cudaStream_t b) {
    if (a == b) return;
    cudaEvent_t e = evpool_[evi++ % evpool_.size()];
    cudaEventRecord(e, a);
    cudaStreamWaitEvent(b, e, 0);
  };
  // Link-phase launches of one pass (group classes, serial packs, serial
  // bodies) touch disjoint bodies, so they run side by side: the first on the
  // main stream, the others on branch streams forked from one event recorded
  // before the pass, and all joined back before the grid and collide kernels.
  uint32_t br_used = 0, br_next = 0;
  cudaEvent_t fork_ev = nullptr;
  auto begin_pass = [&](bool full) {
    br_used = br_next = 0;
    if (profiling) return;
    const SerialPacks* pk = full ? packs_full_ : packs_links_;
    size_t n = (pk[0].packs.empty() ? 0 : 1) + (pk[1].packs.empty() ? 0 : 1) +
               ((full ? serial_full_ : serial_links_).empty() ? 0 : 1);
    for (const LaunchClass& c : classes_) n += (c.full == full && !c.items.empty()) ? 1 : 0;
    if (n < 2) return;  // a single launch stays on the main stream
    fork_ev = evpool_[evi++ % evpool_.size()];
    cudaEventRecord(fork_ev, stream_);
  };
  auto branch = [&]() -> cudaStream_t {
    const uint32_t i = br_next++;
    if (profiling || i == 0) return stream_;
    const uint32_t k = (i - 1) % kLinkBranches;
    if (!(br_used & (1u << k))) {
      cudaStreamWaitEvent(lx_[k], fork_ev, 0);
      br_used |= 1u << k;
    }
    return lx_[k];
  };
  auto end_pass = [&]() {
    for (uint32_t k = 0; k < kLinkBranches; ++k)
      if (br_used & (1u << k)) edge(lx_[k], stream_);
    br_used = br_next = 0;
  };
  // one launch of a group class over n work items starting at L
  auto launch_class = [&](const LaunchClass& c, const uint2* L, uint32_t n, uint32_t cur,
                          uint32_t sub, cudaStream_t st) {
    if (c.large_c) {  // large-body executor: one cluster of large_c CTAs per body
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(n * c.large_c);
      cfg.blockDim = dim3(c.T);
      cfg.dynamicSmemBytes = (size_t)(c.full ? 16u : 8u) << c.log2per;
      cfg.stream = st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = c.large_c;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = c.large_c > 1 ? 1u : 0u;
      void (*kl)(const DWorld*, DScheds, const uint2*, uint32_t, uint32_t, uint32_t, uint32_t,
                 uint32_t) =
          c.full ? (c.large_c > 1 ? k_exec_large<true, true> : k_exec_large<true, false>)
                 : (c.large_c > 1 ? k_exec_large<false, true> : k_exec_large<false, false>);
      lk(cudaLaunchKernelEx(&cfg, kl, W, SC, L, n, c.large_c, c.log2per, cur, sub));
      return;
    }
    const dim3 grid((n + c.G - 1) / c.G), block(c.T * c.G);
    const uint32_t sb = c.res ? c.res : 2 * c.fill;
    const size_t sm = (size_t)c.G * (c.region + sb + GROUP_TAIL_BYTES);
    const uint32_t rg = c.smem ? c.region : 0u;
    // The sub-step pipeline's main-stream link launch follows the previous
    // sub-step's collide kernel programmatically when its schedules are
    // resident: at most one CTA per SM waits early, leaving the SMs the
    // circle/polygon branch needs.  (Large streamed launches started early
    // filled every SM and delayed that branch: 18 % slower on 1,024 bodies.)
    const bool pdl = !profiling && !c.full && c.res && st == stream_;
    void (*k)(const DWorld*, DScheds, const uint2*, uint32_t, uint32_t, uint32_t, uint32_t,
              uint32_t, uint32_t, uint32_t, uint32_t*, uint2*, DSlots) =
        c.res ? (c.full ? k_exec_groups<true, true, true> : k_exec_groups<false, true, true>)
        : c.full ? (c.smem ? k_exec_groups<true, true, false> : k_exec_groups<true, false, false>)
                 : (c.smem ? k_exec_groups<false, true, false> : k_exec_groups<false, false, false>);
    lk(launch_k(k, grid, block, sm, st, pdl, W, SC, L, n, c.T, c.G, rg, sb, cur, sub, GR.count,
                GR.pbr, GS));
  };
  auto groups = [&](bool full, uint32_t cur, uint32_t sub) {
    for (const LaunchClass& c : classes_) {
      if (c.full != full || c.items.empty()) continue;
      const char* name = c.large_c ? (full ? "exec_large_full" : "exec_large_links")
                         : full ? (c.smem ? "exec_groups_full_smem" : "exec_groups_full_global")
                                : (c.smem ? "exec_groups_links_smem" : "exec_groups_links_global");
      const cudaStream_t st = branch();
      timed(name, [&] { launch_class(c, d_lists_ + c.dev_off, (uint32_t)c.items.size(), cur, sub, st); });
    }
  };
  edge(stream_, ax);
  edge(stream_, ax2);
  if (plain_) {
    // one world at a time, each with its own launches
    for (uint32_t si = 0; si < wlaunch_.size(); ++si) {
      const WorldLaunch& wl = wlaunch_[si];
      if (si >= slots_.size() || !slots_[si].live || slots_[si].img.ext) continue;
      for (size_t c = 0; c < classes_.size() && c < wl.cls.size(); ++c) {
        const LaunchClass& lc = classes_[c];
        const uint32_t n = wl.cls[c].second;
        if (!n || !lc.full) continue;
        const uint2* L = d_lists_ + lc.dev_off + wl.cls[c].first;
        timed("plain_exec_groups", [&] { launch_class(lc, L, n, 0, 0, stream_); });
      }
      if (wl.pkn) {
        const SerialPacks& P = packs_full_[0];
        timed("plain_exec_serial_smem", [&] {
          k_exec_serial_smem<true, false><<<wl.pkn, kSerialPackThreads, P.max_bytes, stream_>>>(
              W, d_lists_ + P.off_items, d_lists_ + P.off_base, d_lists_ + P.off_packs + wl.pk0,
              wl.pkn, 0, 0);
        });
      }
      if (wl.sfn) {
        timed("plain_exec_serial", [&] {
          k_exec_serial<true><<<(wl.sfn + 127) / 128, 128, 0, stream_>>>(
              W, d_lists_ + off_serial_full_ + wl.sf0, wl.sfn, 0, 0);
        });
      }
      if (wl.rigid >= 0) {
        timed("plain_rigid", [&] {
          if (wl.rigid_wide)
            k_rigid<0, 1024><<<1, 1024, rigid_smem_, stream_>>>(W, d_wlists_ + wl.rigid, 1, 0, rigid_smem_);
          else
            k_rigid<0, 256><<<1, 256, rigid_smem_, stream_>>>(W, d_wlists_ + wl.rigid, 1, 0, rigid_smem_);
        });
      }
    }
  } else {
  // worlds without extension collisions: one launch per class for the whole step
  begin_pass(true);
  groups(true, 0, 0);
  for (int k = 0; k < 2; ++k) {
    const SerialPacks& P = packs_full_[k];
    if (P.packs.empty()) continue;
    const uint32_t n = (uint32_t)P.packs.size();
    const cudaStream_t st = branch();
    timed(k == 0 ? "exec_serial_smem_full" : "exec_serial_staged_full", [&] {
      if (k == 0) k_exec_serial_smem<true, false><<<n, kSerialPackThreads, P.max_bytes, st>>>(
          W, d_lists_ + P.off_items, d_lists_ + P.off_base, d_lists_ + P.off_packs, n, 0, 0);
      else k_exec_serial_smem<true, true><<<n, 32, P.max_bytes, st>>>(
          W, d_lists_ + P.off_items, d_lists_ + P.off_base, d_lists_ + P.off_packs, n, 0, 0);
    });
  }
  if (!serial_full_.empty()) {
    const uint32_t n = (uint32_t)serial_full_.size();
    const cudaStream_t st = branch();
    timed("exec_serial_full", [&] {
      k_exec_serial<true><<<(n + 127) / 128, 128, 0, st>>>(W, d_lists_ + off_serial_full_, n, 0, 0);
    });
  }
  end_pass();
  if (!rigid_full_.empty()) {
    const uint32_t n = (uint32_t)rigid_full_.size();
    timed("rigid_full", [&] {
      if (rigid_wide_full_) k_rigid<0, 1024><<<n, 1024, rigid_smem_, ax2>>>(W, d_wlists_, n, 0, rigid_smem_);
      else k_rigid<0, 256><<<n, 256, rigid_smem_, ax2>>>(W, d_wlists_, n, 0, rigid_smem_);
    });
  }
  }
  // worlds with extension collisions: per sub-step pipeline
  const uint32_t nch = (uint32_t)chunks_.size();
  const uint2* CH = d_lists_ + off_chunks_;
  const uint32_t nre = (uint32_t)rigid_ext_.size();
  const uint32_t* RE = d_wlists_ + off_rigid_ext_;
  for (uint32_t s = 0; s < smax_ext_; ++s) {
    const uint32_t cur = s & 1u;
    if (nre) {  // phase B of s-1 (after collide s-1 read the circles), phase A of s
      timed("rigid_ext", [&] {
        if (rigid_wide_ext_) {
          if (s == 0) k_rigid<1, 1024><<<nre, 1024, rigid_smem_, ax>>>(W, RE, nre, s, rigid_smem_);
          else k_rigid<3, 1024><<<nre, 1024, rigid_smem_, ax>>>(W, RE, nre, s, rigid_smem_);
        } else {
          if (s == 0) k_rigid<1, 256><<<nre, 256, rigid_smem_, ax>>>(W, RE, nre, s, rigid_smem_);
          else k_rigid<3, 256><<<nre, 256, rigid_smem_, ax>>>(W, RE, nre, s, rigid_smem_);
        }
      });
    }
    begin_pass(false);
    groups(false, cur, s);
    for (int k = 0; k < 2; ++k) {
      const SerialPacks& P = packs_links_[k];
      if (P.packs.empty()) continue;
      const uint32_t n = (uint32_t)P.packs.size();
      const cudaStream_t st = branch();
      timed(k == 0 ? "exec_serial_smem_links" : "exec_serial_staged_links", [&] {
        if (k == 0) k_exec_serial_smem<false, false><<<n, kSerialPackThreads, P.max_bytes, st>>>(
            W, d_lists_ + P.off_items, d_lists_ + P.off_base, d_lists_ + P.off_packs, n, cur, s);
        else k_exec_serial_smem<false, true><<<n, 32, P.max_bytes, st>>>(
            W, d_lists_ + P.off_items, d_lists_ + P.off_base, d_lists_ + P.off_packs, n, cur, s);
      });
    }
    if (!serial_links_.empty()) {
      const uint32_t n = (uint32_t)serial_links_.size();
      const cudaStream_t st = branch();
      timed("exec_serial_links", [&] {
        k_exec_serial<false><<<(n + 127) / 128, 128, 0, st>>>(W, d_lists_ + off_serial_links_, n, cur, s);
      });
    }
    end_pass();
    // (worlds with collision flags but no solver particles, such as only
    // circles, take part in the sub-step loop without work chunks: the
    // particle kernels below are skipped when there are none)
    if (any_pp_ && grid_slotted_ && nch) {
      // the cell words of this parity are all zero here (cleared by the
      // previous sub-step's collide pass, or by k_copy_back); worlds whose
      // link executor inserted their particles skip the insert pass
      if (any_count_)
        timed("grid_insert", [&] {
          lk(launch_k(k_grid_insert, dim3(nch), dim3(CHUNK), 0, stream_, !profiling, W, GS, CH,
                      nch, cur, s));
        });
    } else if (any_pp_ && nch) {
      // counts are all zero here: the scan of the previous sub-step cleared them.
      // Small grids: one 256-thread CTA per 1,024-bucket tile; large ones:
      // 16,384-bucket tiles over at most one 1024-thread CTA per SM.
      const bool small = grid_used_ <= SCAN_SMALL_MAX;
      const uint32_t tile = small ? SCAN_SMALL_TILE : SCAN_LARGE_TILE;
      const uint32_t nt = (grid_used_ + tile - 1) / tile;
      // worlds whose link executor counted their particles skip this pass
      if (any_count_)
        timed("grid_count", [&] {
          lk(launch_k(k_grid_count, dim3(nch), dim3(CHUNK), 0, stream_, !profiling, W, GR, CH,
                      nch, cur, s));
        });
      const uint32_t ncta = small ? nt : std::min<uint32_t>(nt, (uint32_t)std::max(g_num_sms, 1));
      timed("grid_scan", [&] {
        if (small)
          lk(launch_k(k_grid_scan<1, 256>, dim3(ncta), dim3(256), 0, stream_, !profiling, GR,
                      grid_used_, nt));
        else
          lk(launch_k(k_grid_scan<4, 1024>, dim3(ncta), dim3(1024), 0, stream_, !profiling, GR,
                      grid_used_, nt));
      });
      timed("grid_scatter", [&] {
        lk(launch_k(k_grid_scatter, dim3(nch), dim3(CHUNK), 0, stream_, !profiling, W, GR, CH,
                    nch, cur, s));
      });
    }
    if (nre) edge(ax, stream_);
    if (nch) timed("collide_integrate", [&] {
      if (grid_slotted_ || !any_pp_) {
        if (collide_per_particle_)
          lk(launch_k(k_collide_particle<DSlots>, dim3(nch), dim3(COLLIDE_P_THREADS), 0, stream_,
                      !profiling, W, GS, CH, nch, cur, s));
        else
          lk(launch_k(k_collide_integrate<DSlots>, dim3(nch * COLLIDE_CTAS),
                      dim3(COLLIDE_THREADS), 0, stream_, !profiling, W, GS, CH, nch, cur, s));
      } else {
        if (collide_per_particle_)
          lk(launch_k(k_collide_particle<DGrid>, dim3(nch), dim3(COLLIDE_P_THREADS), 0, stream_,
                      !profiling, W, GR, CH, nch, cur, s));
        else
          lk(launch_k(k_collide_integrate<DGrid>, dim3(nch * COLLIDE_CTAS),
                      dim3(COLLIDE_THREADS), 0, stream_, !profiling, W, GR, CH, nch, cur, s));
      }
    });
    if (nre) edge(stream_, ax);
  }
  if (smax_ext_ > 0) {
    if (nre) timed("rigid_ext", [&] {
      if (rigid_wide_ext_) k_rigid<2, 1024><<<nre, 1024, rigid_smem_, ax>>>(W, RE, nre, smax_ext_ - 1, rigid_smem_);
      else k_rigid<2, 256><<<nre, 256, rigid_smem_, ax>>>(W, RE, nre, smax_ext_ - 1, rigid_smem_);
    });
    // an odd sub-step count leaves parity 0's cell words for k_copy_back to clear
    const bool clear0 = any_pp_ && grid_slotted_ && (smax_ext_ & 1u);
    // nothing to copy back or clear when every world has an even count
    if (nch && (any_odd_ext_ || clear0)) timed("copy_back", [&] {
      k_copy_back<<<nch, CHUNK, 0, stream_>>>(W, CH, nch, clear0 ? GS.cell : nullptr,
                                               clear0 ? GS.nbuckets : 0u);
    });
  }
  edge(ax, stream_);
  edge(ax2, stream_);
  if (profiling) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (launch_err != cudaSuccess) {
    last_error = std::string("cudaLaunchKernelEx: ") + cudaGetErrorString(launch_err);
    cudaGetLastError();  // the same failure, recorded by the runtime too
    return ERR_CUDA;
  }
  B2D_CUDA(cudaGetLastError());
  return OK;
}

int Engine::step() {
  int st;
  if (lists_dirty_ && (st = rebuild_lists()) != OK) return st;
  if ((st = upload_registry()) != OK) return st;
  if (grid_reset_ && d_grid_) {
    // after a failed step the bucket counts and the cursor may be partial
    B2D_CUDA(cudaMemsetAsync(d_grid_, 0, grid_head_bytes_, stream_));
    grid_reset_ = false;
  }
  st = launch_step();
  if (st != OK) grid_reset_ = true;
  return st;
}

int Engine::launch_step() {
  int st;
  if (profile_) return launch_all(true);
  if (!use_graph_ || plain_) return launch_all(false);
  // capture a graph once the composition has been stable for two steps;
  // a batch that changes every step (serving) keeps launching eagerly
  if (!graph_valid_ && stable_steps_ < 2) {
    ++stable_steps_;
    return launch_all(false);
  }
  if (!graph_valid_) {
    cudaGraph_t g = nullptr;
    B2D_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    st = launch_all(false);
    cudaError_t ce = cudaStreamEndCapture(stream_, &g);
    if (st != OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess) {
      last_error = std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce);
      return ERR_CUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      last_error = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie);
      graph_ = nullptr;
      return ERR_CUDA;
    }
    graph_valid_ = true;
  }
  B2D_CUDA(cudaGraphLaunch(graph_, stream_));
  return OK;
}

int Engine::sync() {
  B2D_CUDA(cudaStreamSynchronize(stream_));
  return check_device_error();
}

int Engine::state_span(uint32_t slot, void** dptr, size_t* bytes) {
  if (slot >= slots_.size() || !slots_[slot].live) return ERR_INDEX;
  *dptr = slots_[slot].block;
  *bytes = slots_[slot].L.state_bytes;
  return OK;
}

int Engine::download(uint32_t slot) {
  if (slot >= slots_.size() || !slots_[slot].live) return ERR_INDEX;
  Slot& s = slots_[slot];
  std::vector<float2> buf(s.L.state_bytes / sizeof(float2));
  if (!buf.empty())
    B2D_CUDA(cudaMemcpyAsync(buf.data(), s.block, s.L.state_bytes, cudaMemcpyDeviceToHost, stream_));
  B2D_CUDA(cudaStreamSynchronize(stream_));
  int est = check_device_error();
  if (est != OK) return est;
  WorldHost& w = *s.host;
  const float2* p = buf.data();
  const size_t np = s.img.pos.size();
  for (size_t i = 0; i < np; ++i) {
    w.particles[i].pos = Vec2{p[i].x, p[i].y};
    w.particles[i].prev_pos = Vec2{p[np + i].x, p[np + i].y};
    w.particles[i].acc = Vec2{0.0f, 0.0f};
  }
  p += 2 * np;
  const size_t nc = s.img.cpos.size();
  for (size_t i = 0; i < nc; ++i) {
    w.circles[i].point.pos = Vec2{p[i].x, p[i].y};
    w.circles[i].point.prev_pos = Vec2{p[nc + i].x, p[nc + i].y};
    w.circles[i].point.acc = Vec2{p[2 * nc + i].x, p[2 * nc + i].y};
  }
  p += 3 * nc;
  const size_t nv = s.img.vpos.size();
  size_t v = 0;
  for (size_t g = 0; g < w.polygons.size(); ++g) {
    Polygon& P = w.polygons[g];
    for (Particle& q : P.particles) {
      q.pos = Vec2{p[v].x, p[v].y};
      q.prev_pos = Vec2{p[nv + v].x, p[nv + v].y};
      q.acc = Vec2{p[2 * nv + v].x, p[2 * nv + v].y};
      ++v;
    }
    P.center = Vec2{p[3 * nv + g].x, p[3 * nv + g].y};
  }
  return OK;
}

int Engine::upload_state(uint32_t slot) {
  if (slot >= slots_.size() || !slots_[slot].live) return ERR_INDEX;
  Slot& s = slots_[slot];
  const WorldHost& w = *s.host;
  std::vector<float2> buf(s.L.state_bytes / sizeof(float2));
  float2* p = buf.data();
  const size_t np = w.particles.size();
  for (size_t i = 0; i < np; ++i) {
    p[i] = make_float2(w.particles[i].pos.x, w.particles[i].pos.y);
    p[np + i] = make_float2(w.particles[i].prev_pos.x, w.particles[i].prev_pos.y);
  }
  p += 2 * np;
  const size_t nc = w.circles.size();
  for (size_t i = 0; i < nc; ++i) {
    p[i] = make_float2(w.circles[i].point.pos.x, w.circles[i].point.pos.y);
    p[nc + i] = make_float2(w.circles[i].point.prev_pos.x, w.circles[i].point.prev_pos.y);
    p[2 * nc + i] = make_float2(w.circles[i].point.acc.x, w.circles[i].point.acc.y);
  }
  p += 3 * nc;
  const size_t nv = s.img.vpos.size();
  size_t v = 0;
  for (size_t g = 0; g < w.polygons.size(); ++g) {
    for (const Particle& q : w.polygons[g].particles) {
      p[v] = make_float2(q.pos.x, q.pos.y);
      p[nv + v] = make_float2(q.prev_pos.x, q.prev_pos.y);
      p[2 * nv + v] = make_float2(q.acc.x, q.acc.y);
      ++v;
    }
    p[3 * nv + g] = make_float2(w.polygons[g].center.x, w.polygons[g].center.y);
  }
  if (!buf.empty())
    B2D_CUDA(cudaMemcpyAsync(s.block, buf.data(), s.L.state_bytes, cudaMemcpyHostToDevice, stream_));
  B2D_CUDA(cudaStreamSynchronize(stream_));
  return OK;
}

}  // namespace b2d

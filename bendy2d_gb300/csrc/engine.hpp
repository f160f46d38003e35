// engine.hpp — planner output (one world's device image) and the Engine that
// owns device memory for a set of worlds and steps them together.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "b2d_dev.h"
#include "host.hpp"

typedef struct CUstream_st* cudaStream_t;
typedef struct CUgraphExec_st* cudaGraphExec_t;

namespace b2d {

// Fault injection for tests of failure handling (b2d_set_fault): the kinds.
//  FAULT_WAIT_TIMEOUT  value != 0: every executor group's first bulk-copy wait
//                      reports a timeout (the copy still lands before the CTA
//                      leaves); the step then reports ERR_DEVICE
//  FAULT_GRID_CAP      value > 0: the collision grid hands out at most `value`
//                      sorted entries per sub-step (below the particle count
//                      this makes the scan refuse blocks: ERR_BIT_GRID_OVERFLOW)
//  FAULT_ALLOC         the next `value` world-block allocations fail as if
//                      cudaMallocAsync had failed
enum : int { FAULT_WAIT_TIMEOUT = 1, FAULT_GRID_CAP = 2, FAULT_ALLOC = 3 };

// Tunables of the planner (the autotuner sweeps these).
struct PlanTuning {
  float serial_width = 2.0f;        // single-pass width below which a body runs serially
  uint32_t t_min = 32, t_max = 512; // threads per group
  uint32_t pack_np = 1024;          // pack small components into bodies up to this size
  uint32_t pack_nl = 4096;
  uint32_t free_chunk = 2048;       // particles per body for link-free particles
  uint32_t smem_max = 200 * 1024;   // bytes of shared memory per group region
  uint32_t warp_groups = 8;         // groups per CTA when T == 32
  uint32_t max_groups = 15;         // groups per CTA when T > 32
  float width_per_thread = 0.5f;    // T = pow2 >= avg width / this (issue-bound: wide groups win)
  uint32_t resident = 1;            // load a body's whole schedule when it fits
  uint32_t res_max = 227 * 1024;    // shared bytes per group for body + resident schedule
  float stage_frac = 1.01f;         // serial bodies with chains >= this x the longest: solo
                                    // packs, links staged in shared memory (default: none;
                                    // with positions forwarded in registers ordinary packs
                                    // run the longest chains faster)
  float bucket_factor = 2.0f;       // collision-grid buckets per world: pow2 >= this x particles
  uint32_t collide_thread_min = 131072;  // particles in the collide pass from which it runs
                                         // one thread per particle (else three lanes each)
  uint32_t large_max = 8;           // largest cluster of the large-body executor (0: bodies
                                    // over one CTA's shared memory run from global memory)
  uint32_t grid_slot_max = 262144;  // particles in the collision grid up to which it is
                                    // built by slot inserts; above, by a counting sort per
                                    // sub-step (count, scan, scatter)
  // set a tunable by name; returns false for an unknown name
  bool set(const std::string& key, double value);
};

// Engine-wide registry of level schedules, deduplicated by topology.
struct SchedRegistry {
  std::unordered_map<std::string, uint32_t> index;
  std::vector<DSched> scheds;
  std::vector<uint32_t> chunk_off, chunk_len, stream;
  size_t uploaded_scheds = 0, uploaded_chunks = 0, uploaded_stream = 0;
  // wide: the schedule is for the large-body executor, which runs levels
  // wider than a group (several ops per thread): whole-update schedules are
  // grouped by op kind there whatever their width
  uint32_t get(const uint2* links, uint32_t nl, uint32_t np, uint32_t S, uint32_t I, bool full,
               bool wide = false);
};

struct GroupBody {
  uint32_t body;
  uint32_t T;
  uint32_t region;  // shared bytes for this body (0 when run from global memory)
  uint32_t res;     // bytes of its schedule when held whole in shared memory, else 0
  bool smem;
  uint32_t large_c = 0;  // large-body executor: CTAs in the body's cluster (0: not used)
  uint32_t log2per = 0;  // large-body executor: log2 of the particles per CTA
};


struct PlanStats {
  uint32_t bodies = 0, group_bodies = 0, serial_bodies = 0, global_bodies = 0;
  uint32_t large_bodies = 0;  // group bodies run by the large-body executor
  uint64_t levels = 0, ops = 0;  // summed over group bodies
  uint32_t colours = 0;
};

// Device image of one world: exactly the arrays of its device block.
struct WorldImage {
  DWorld params{};   // parameters; pointers are filled at placement
  bool ext = false;  // extension collisions on: per-sub-step pipeline
  // state prefix (float2 each): pos, prev, cpos, cprev, cacc, vpos, vprev, vacc, pcenter
  std::vector<float2> pos, prev, cpos, cprev, cacc, vpos, vprev, vacc, pcenter;
  std::vector<uint32_t> bidx;
  std::vector<DBody> bodies;
  std::vector<uint2> lab;
  std::vector<float> lrest, lstiff;
  std::vector<float> crad;
  std::vector<uint32_t> cstatic;
  std::vector<uint2> clab;
  std::vector<float> clrest;
  std::vector<DPoly> polys;
  std::vector<uint2> plab;
  std::vector<float> plrest;
  std::vector<uint32_t> stage_off;
  std::vector<uint32_t> stage_pr;
  std::vector<GroupBody> groups;
  std::vector<uint32_t> serials;
  std::vector<uint32_t> link_order;  // fast mode: world link order used
  PlanStats stats;
  size_t nv() const { return vpos.size(); }
};

int plan_world(const WorldHost& w, const PlanTuning& tune, SchedRegistry& reg, WorldImage& out,
               std::string* why);

// byte layout of a world block
struct BlockLayout {
  size_t state_bytes = 0, total = 0;
  size_t o_pos, o_prev, o_cpos, o_cprev, o_cacc, o_vpos, o_vprev, o_vacc, o_pcenter;
  size_t o_pos1, o_bidx, o_bodies, o_lab, o_lrest, o_lstiff, o_crad, o_cstatic, o_clab,
      o_clrest, o_polys, o_paabb, o_plab, o_plrest, o_stage, o_stage_pr;
};
BlockLayout layout_of(const WorldImage& im);
void write_block(const WorldImage& im, const BlockLayout& L, unsigned char* dst);

struct LaunchClass {
  uint32_t T, G, region;
  uint32_t res;    // resident schedule bytes per group (0: streamed in fills)
  uint32_t fill;   // streamed: bytes per fill buffer (two per group)
  uint32_t words;  // largest member schedule, in words
  bool smem, full;
  uint32_t large_c = 0, log2per = 0;  // large-body executor class (large_c CTAs per body)
  std::vector<uint2> items;
  size_t dev_off = 0;  // offset (in uint2) into the device list buffer
};

class Engine {
 public:
  explicit Engine(cudaStream_t stream = nullptr);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  int add(WorldHost* w, uint32_t* slot, std::string* why);
  // add() in two parts: plan() is host work only (it may run while launched
  // work of this engine is in flight; it grows the host side of the schedule
  // registry, which the next step uploads), add_planned() allocates, uploads
  // and registers the world; the image is consumed
  int plan(const WorldHost& w, WorldImage* img, std::string* why);
  int add_planned(WorldHost* w, WorldImage&& img, uint32_t* slot);
  // While on, add_planned() and set_dt() upload on a stream of their own
  // and wait for that stream only, so that they can run while a step
  // launched on the main stream is in flight (the server installs the next
  // tick's worlds that way); the step in flight reads neither the new
  // world's block nor its record.
  int install_beside(bool on);
  int remove(uint32_t slot);
  int set_dt(uint32_t slot, float dt);
  int set_params(uint32_t slot);          // gravity / bounds changed on the host mirror
  int step();                             // one Solver::update for every world
  int download(uint32_t slot);            // device state -> host mirror
  int upload_state(uint32_t slot);        // host mirror state -> device (same topology)
  // raw state prefix (pos, prev, circles, polygons) of a world, for end-to-end
  // transfers from and to pinned host memory
  int state_span(uint32_t slot, void** dptr, size_t* bytes);
  int sync();
  void set_stream(cudaStream_t s);
  cudaStream_t stream() const { return stream_; }
  void set_use_graph(bool on) { use_graph_ = on; invalidate_graph(); }
  void set_profile(bool on) { profile_ = on; }
  // plain mode: every world without extension collisions gets its own
  // launches (no batching, no graph) — the one-world-per-launch baseline
  void set_plain(bool on) { plain_ = on; lists_dirty_ = true; invalidate_graph(); }
  // per-kernel timings of the last profiled step (ms), keyed by kernel name
  const std::vector<std::pair<std::string, float>>& last_profile() const { return prof_; }
  const WorldImage* image(uint32_t slot) const;
  uint32_t launches_per_step() const { return launches_; }
  PlanTuning& tuning() { return tune_; }
  void set_tuning(const PlanTuning& t);
  size_t device_bytes() const { return dev_bytes_; }
  int set_fault(int kind, uint64_t value);  // FAULT_*; ERR_ARG for an unknown kind
  std::string last_error;

 private:
  struct Slot {
    WorldHost* host = nullptr;
    WorldImage img;
    BlockLayout L;
    unsigned char* block = nullptr;
    float dt = 0.0f;
    bool live = false;
  };
  int rebuild_lists();
  int upload_registry();
  int ensure_table(size_t n);
  int ensure_grid(size_t nbuckets, size_t np_ext);
  int launch_step();  // eager launches or the captured graph
  int launch_all(bool profiling);
  void invalidate_graph();
  int fill_world_record(uint32_t slot);

  cudaStream_t stream_ = nullptr;
  bool own_stream_ = false;
  cudaStream_t ist_ = nullptr;  // install_beside's stream
  bool beside_ = false;
  cudaStream_t up_stream() const { return beside_ ? ist_ : stream_; }
  cudaStream_t aux_[2] = {nullptr, nullptr};  // graph branches (circles/polygons)
  static constexpr uint32_t kLinkBranches = 7;
  cudaStream_t lx_[kLinkBranches] = {};       // graph branches of the link phase
  std::vector<struct CUevent_st*> evpool_;
  PlanTuning tune_;
  SchedRegistry reg_;
  std::vector<Slot> slots_;
  std::vector<uint32_t> free_slots_;
  // device tables
  DWorld* d_worlds_ = nullptr;
  size_t worlds_cap_ = 0;
  std::vector<DWorld> h_worlds_;
  DSched* d_scheds_ = nullptr;
  size_t scheds_cap_ = 0;
  uint32_t* d_chunk_off_ = nullptr;
  uint32_t* d_chunk_len_ = nullptr;
  size_t chunks_cap_ = 0;
  uint32_t* d_stream_ = nullptr;
  size_t stream_cap_ = 0;
  uint32_t* d_err_ = nullptr;  // device error word (bounded waits)
  int check_device_error();
  // work lists
  std::vector<LaunchClass> classes_;
  std::vector<uint2> serial_full_, serial_links_, chunks_;
  std::vector<uint32_t> rigid_full_, rigid_ext_;
  bool rigid_wide_full_ = false, rigid_wide_ext_ = false;  // a world there has many pair tests
  uint2* d_lists_ = nullptr;
  size_t lists_cap_ = 0;
  size_t off_serial_full_ = 0, off_serial_links_ = 0, off_chunks_ = 0;
  uint32_t* d_wlists_ = nullptr;
  size_t wlists_cap_ = 0;
  size_t off_rigid_ext_ = 0;
  uint32_t smax_ext_ = 0;
  bool any_odd_ext_ = false;  // a collision world ends its update in the second position buffer
  bool plain_ = false;
  struct WorldLaunch {  // this world's ranges in the lists (plain mode)
    std::vector<std::pair<uint32_t, uint32_t>> cls;  // per class: (offset, count)
    uint32_t sf0 = 0, sfn = 0;                        // serial_full_
    uint32_t pk0 = 0, pkn = 0;                        // packs_full_[0].packs
    int32_t rigid = -1;                               // index into rigid_full_
    bool rigid_wide = false;                          // 1024-thread circle/polygon CTA
  };
  // chain-like bodies packed into shared-memory CTAs (k_exec_serial_smem)
  struct SerialPacks {
    std::vector<uint2> items;     // pack order
    std::vector<uint2> base;      // {first particle slot, first link slot} of each item
    std::vector<uint2> packs;     // {first item, item count}
    uint32_t max_bytes = 0;
    size_t off_items = 0, off_packs = 0, off_base = 0;
  };
  // [0]: packs of many small bodies; [1]: one large body per pack
  SerialPacks packs_full_[2], packs_links_[2];
  void build_packs(std::vector<uint2>& in, bool full, SerialPacks* out, std::vector<uint2>& rest,
                   bool allow_large);
  std::vector<WorldLaunch> wlaunch_;
  bool any_pp_ = false;
  bool any_count_ = false;  // a world with particle collisions needs the insert (count) kernel
  bool collide_per_particle_ = false;  // k_collide_particle instead of k_collide_integrate
  uint32_t rigid_smem_ = 0;
  uint32_t grid_used_ = 0;
  size_t grid_bytes_ = 0;
  // words at the start of d_grid_ that a failed step can leave partial (sorted
  // grid: counts, ranges, cursor; slotted grid: both parities' cell words and
  // the overflow cursor)
  size_t grid_head_bytes_ = 0;
  bool grid_reset_ = false;     // clear them before the next step (after a failure)
  bool lists_dirty_ = true;
  // broadphase: one of the two forms, as allocated
  bool grid_slotted_ = false;
  DGrid grid_{};
  DSlots gslots_{};
  size_t grid_np_ = 0;
  unsigned char* d_grid_ = nullptr;
  // graph
  bool use_graph_ = true;
  cudaGraphExec_t graph_ = nullptr;
  bool graph_valid_ = false;
  uint32_t stable_steps_ = 0;
  bool profile_ = false;
  std::vector<std::pair<std::string, float>> prof_;
  uint32_t launches_ = 0;
  size_t dev_bytes_ = 0;
  // fault injection (tests only; all zero in normal operation)
  uint32_t fault_bits_ = 0;       // FAULT_BIT_* for the kernels
  uint32_t fault_grid_cap_ = 0;   // 0: the grid's real capacity
  uint64_t fault_alloc_ = 0;      // world-block allocations still to fail
};

}  // namespace b2d

// kernels.cuh — CUDA kernels for the bendy2d solver step (sm_103a).
//
// Every floating-point operation that has a counterpart in the reference uses
// the round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn,
// __fsqrt_rn ...).  Those are never contracted into FMA and are IEEE exact, so
// each op rounds exactly like the reference's scalar f32 arithmetic (rustc
// does not contract either).  The file is also compiled with --fmad=false.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

#include "b2d_dev.h"

namespace b2d {


__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// IEEE division and square root with exact zero shortcuts.  Measured on
// sm_103a, __fdiv_rn with a zero numerator takes ~250 cycles against ~55 for
// ordinary operands, and __fsqrt_rn(0) ~130 against ~53; axis-aligned links
// (dx or dy exactly 0) hit that case on most ops.  IEEE 754 fixes those
// results exactly: ±0 / d = ±0 for d > 0 and ∓0 for d < 0 (d not NaN, any
// magnitude including infinity), and sqrt(±0) = ±0.  They are selected
// without executing the operation on a zero (the operation sees 1 instead),
// so every result is bit-identical to the plain intrinsic.
__device__ __forceinline__ float fdiv(float a, float b) {
  const bool z = (a == 0.0f) && (b > 0.0f || b < 0.0f);
  const float q = __fdiv_rn(z ? 1.0f : a, b);
  return z ? (b > 0.0f ? a : -a) : q;
}
__device__ __forceinline__ float fsqrt(float a) {
  const bool z = a == 0.0f;
  const float r = __fsqrt_rn(z ? 1.0f : a);
  return z ? a : r;
}

// nalgebra norm_squared is 0 + (x*x + y*y); a sum of two squares is never
// -0, so adding the leading +0 cannot change the value and is omitted.
__device__ __forceinline__ float norm_sq(float x, float y) { return fadd(fmul(x, x), fmul(y, y)); }
__device__ __forceinline__ float dot2(float ax, float ay, float bx, float by) {
  return fadd(fmul(ax, bx), fmul(ay, by));
}

// ParticleLink::solve, src/link.rs:18-27:
//   d = a - b; dist = |d|; n = d / dist;
//   a -= n*(dist - L)*0.5; b += n*(dist - L)*0.5
// Extension: the correction is multiplied by the stiffness last (1 = exact).
__device__ __forceinline__ void link_solve(float2& a, float2& b, float rest, float stiff) {
  float dx = fsub(a.x, b.x), dy = fsub(a.y, b.y);
  float dist = fsqrt(norm_sq(dx, dy));
  float nx = fdiv(dx, dist), ny = fdiv(dy, dist);
  float m = fsub(dist, rest);
  float cx = fmul(fmul(fmul(nx, m), 0.5f), stiff);
  float cy = fmul(fmul(fmul(ny, m), 0.5f), stiff);
  a.x = fsub(a.x, cx); a.y = fsub(a.y, cy);
  b.x = fadd(b.x, cx); b.y = fadd(b.y, cy);
}

// The same solve with the plain IEEE intrinsics (no zero shortcuts; same
// results).  One thread replaying a sequential chain pays the shortcuts'
// selects on every link (measured ~40 cycles per solve) and rarely meets an
// exact zero, so the serial executors use this form; the level executors,
// whose warps meet axis-aligned links on most levels, keep the shortcuts.
__device__ __forceinline__ void link_solve_plain(float2& a, float2& b, float rest, float stiff) {
  float dx = fsub(a.x, b.x), dy = fsub(a.y, b.y);
  float dist = __fsqrt_rn(norm_sq(dx, dy));
  float nx = __fdiv_rn(dx, dist), ny = __fdiv_rn(dy, dist);
  float m = fsub(dist, rest);
  float cx = fmul(fmul(fmul(nx, m), 0.5f), stiff);
  float cy = fmul(fmul(fmul(ny, m), 0.5f), stiff);
  a.x = fsub(a.x, cx); a.y = fsub(a.y, cy);
  b.x = fadd(b.x, cx); b.y = fadd(b.y, cy);
}

// Particle::solve_bounds, src/particle.rs:27-46 (min side, else max side).
__device__ __forceinline__ void solve_bounds(float2& p, float2& q, const DWorld& w) {
  float hx = fadd(w.bx, w.bw), hy = fadd(w.by, w.bh);
  if (p.x < w.bx) { float v = fsub(q.x, p.x); q.x = fsub(w.bx, v); p.x = w.bx; }
  else if (p.x > hx) { float v = fsub(q.x, p.x); q.x = fsub(hx, v); p.x = hx; }
  if (p.y < w.by) { float v = fsub(q.y, p.y); q.y = fsub(w.by, v); p.y = w.by; }
  else if (p.y > hy) { float v = fsub(q.y, p.y); q.y = fsub(hy, v); p.y = hy; }
}

// Circle::solve_bounds, src/circle.rs:11-30 (bounds inset by the radius).
__device__ __forceinline__ void circle_bounds(float2& p, float2& q, float r, const DWorld& w) {
  float hx = fadd(w.bx, w.bw), hy = fadd(w.by, w.bh);
  float lo_x = fadd(w.bx, r), hi_x = fsub(hx, r);
  float lo_y = fadd(w.by, r), hi_y = fsub(hy, r);
  if (p.x < lo_x) { float v = fsub(q.x, p.x); q.x = fsub(lo_x, v); p.x = lo_x; }
  else if (p.x > hi_x) { float v = fsub(q.x, p.x); q.x = fsub(hi_x, v); p.x = hi_x; }
  if (p.y < lo_y) { float v = fsub(q.y, p.y); q.y = fsub(lo_y, v); p.y = lo_y; }
  else if (p.y > hi_y) { float v = fsub(q.y, p.y); q.y = fsub(hi_y, v); p.y = hi_y; }
}

// Particle::update, src/particle.rs:20-25: pos = (pos + vel) + (acc*dt)*dt.
__device__ __forceinline__ void integrate(float2& p, float2& q, float ax, float ay, float h) {
  float vx = fsub(p.x, q.x), vy = fsub(p.y, q.y);
  q = p;
  p.x = fadd(fadd(p.x, vx), fmul(fmul(ax, h), h));
  p.y = fadd(fadd(p.y, vy), fmul(fmul(ay, h), h));
}

// ----------------------------------------------------------------------------
// Extension collision grid: cells and buckets (used by the grid kernels below
// and by the link executor's counting store-back).
// ----------------------------------------------------------------------------
// Cell index along one axis: floor((p - origin) / cell), clamped.  For a
// power-of-two cell the division is the multiplication by icell (exact, the
// same bits); otherwise icell is 0 and the IEEE division runs.
__device__ __forceinline__ int32_t cell_coord(float p, float origin, float cell, float icell) {
  const float t = fsub(p, origin);
  float v = floorf(icell != 0.0f ? fmul(t, icell) : fdiv(t, cell));
  if (!(v > -1.0e9f)) v = -1.0e9f;
  if (v > 1.0e9f) v = 1.0e9f;
  return (int32_t)v;
}
__device__ __forceinline__ uint32_t cell_hash(int32_t cx, int32_t cy) {
  uint32_t h = ((uint32_t)cx * 73856093u) ^ ((uint32_t)cy * 19349663u);
  h ^= h >> 15;
  h *= 0x2c1b3c6du;
  h ^= h >> 12;
  return h;
}
// Bucket of cell (cx, cy) in world W: four horizontally adjacent cells (a
// strip, cx >> 2) hash together and take four consecutive buckets, so a row
// of neighbour cells lands in one or two runs of `sorted` and its range and
// entry loads mostly share cache lines.  (The world's bucket count is a
// power of two >= 64, so the mask keeps the low two bits.)
__device__ __forceinline__ uint32_t bucket_of(const DWorld& W, int32_t cx, int32_t cy) {
  return W.gb0 + (((cell_hash(cx >> 2, cy) << 2) | ((uint32_t)cx & 3u)) & W.gmask);
}

// Slotted grid (DSlots): slot k of bucket b, interleaved by strip
__device__ __forceinline__ uint32_t slot_index(uint32_t b, uint32_t k) {
  return ((b >> 2) * GRID_SLOTS + k) * 4u + (b & 3u);
}
// Enter a particle at p in cell (cx, cy), bucket b, into the sub-step's
// cell words: a fixed slot while the bucket has one free, else the overflow
// array (refused past its capacity: ERR_BIT_GRID_OVERFLOW, the entry is
// dropped and the update reports the error).
__device__ __forceinline__ void grid_insert(const DSlots& G, uint32_t sub, uint32_t b, float2 p,
                                            int32_t cx, int32_t cy) {
  uint2* cl = G.cell + (size_t)(sub & 1u) * G.nbuckets + b;
  const uint4 e = make_uint4(__float_as_uint(p.x), __float_as_uint(p.y), (uint32_t)cx, (uint32_t)cy);
  const uint32_t r = atomicAdd(&cl->x, 1u);
  if (r < GRID_SLOTS) {
    G.slot[slot_index(b, r)] = e;
    return;
  }
  const uint32_t o = atomicAdd(G.cursor, 1u);
  if (o >= G.cap) {
    atomicOr(G.err, ERR_BIT_GRID_OVERFLOW);
    return;
  }
  G.ovf[o] = e;
  G.ovf_next[o] = atomicExch(&cl->y, o + 1u);
}

// Group barrier: a group is one warp (syncwarp) or a named barrier over T
// threads.  Both order shared and global memory among the group's threads.
__device__ __forceinline__ void group_sync(uint32_t g, uint32_t T) {
  if (T == 32) {
    __syncwarp();
  } else if (T == blockDim.x) {
    __syncthreads();  // one group per CTA: the plain barrier measured ~5% faster per level
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(T) : "memory");
  }
}

// Programmatic dependent launch.  The main-stream kernels of a sub-step are
// launched so that each may start while its predecessor finishes: every CTA
// signals early that dependents may launch, and a kernel does its work that
// does not depend on the predecessor (schedules, link parameters) before
// pdl_wait(), which returns once the predecessor grid has completed and its
// memory is visible.  Every CTA calls pdl_wait() before it exits, early
// exits included: a grid then completes only after its predecessor did, so
// the guarantee carries down the whole chain.  Without a programmatic
// launch both are no-ops.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ----------------------------------------------------------------------------
// Bulk-copy (TMA) helpers.  One elected thread issues cp.async.bulk into
// shared memory and completion is tracked by an mbarrier transaction count.
// Every wait is bounded (about two seconds of SM clock); on timeout the
// kernel records ERR_BIT_TMA_TIMEOUT in the device error word and returns
// instead of trapping.
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// bytes must be a multiple of 16; src and dst 16-byte aligned
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
constexpr long long WAIT_LIMIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (clock64() - t0 > WAIT_LIMIT_CYCLES) return false;
  }
  return true;
}

// shared bytes per group beyond the body region when the schedule streams
// in fills of one chunk: two chunk buffers, then GROUP_TAIL_BYTES (two
// mbarriers, a flag word and the chunk count of each buffer)
constexpr uint32_t STREAM_BUF_BYTES = 2 * SCHED_CHUNK_WORDS * 4;
constexpr uint32_t STREAM_BYTES = STREAM_BUF_BYTES + GROUP_TAIL_BYTES;

// ----------------------------------------------------------------------------
// Body executor (block / warp granularity).
//
// Each CTA holds G groups of T threads; group g runs work item
// list[blockIdx*G + g] = (world, body) through the body's level schedule.  A
// level is a set of ops on pairwise disjoint particles, and the levels keep,
// for every particle, the exact order of the reference's sequential loops, so
// running a level in parallel reproduces Solver::update bit for bit.  FULL
// schedules cover every sub-step of Solver::update (links x I, then bounds +
// integrate, src/solver.rs:109-115); LINKS-only schedules cover the I link
// passes of one sub-step (extension pipeline).
//
// The schedule streams into shared memory in chunks by double-buffered bulk
// copies, so a level costs shared-memory latency only.  SMEM keeps the body's
// positions (and prev) and links in shared memory too; !SMEM runs the same
// schedule on global memory (bodies too large for one CTA).
// ----------------------------------------------------------------------------
// explicit shared-memory accesses on 32-bit shared addresses (so the body
// state never goes through the generic load path)
__device__ __forceinline__ uint32_t lds_u32(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ uint2 lds_u32x2(uint32_t a) {
  uint2 v;
  asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
  return v;
}
__device__ __forceinline__ float2 lds_f32x2(uint32_t a) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
  return v;
}
__device__ __forceinline__ void sts_f32x2(uint32_t a, float2 v) {
  asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}

template <bool FULL, bool SMEM, bool RES>
__global__ void k_exec_groups(const DWorld* __restrict__ worlds, DScheds SC,
                              const uint2* __restrict__ list, uint32_t nlist, uint32_t T,
                              uint32_t G, uint32_t region_bytes, uint32_t sched_bytes,
                              uint32_t cur, uint32_t sub, uint32_t* __restrict__ gcount,
                              uint2* __restrict__ gpbr, DSlots GS) {
  extern __shared__ __align__(128) unsigned char smem[];
  pdl_trigger();
  const uint32_t g = threadIdx.x / T, t = threadIdx.x - g * T;
  const uint32_t item = blockIdx.x * G + g;
  if (item >= nlist) {  // the whole group leaves; its barrier is private
    pdl_wait();
    return;
  }
  const uint2 wi = list[item];
  const DWorld& W = worlds[wi.x];
  if (!FULL && sub >= W.S) {  // world already finished its sub-steps
    pdl_wait();
    return;
  }
  const DBody B = W.bodies[wi.y];
  const DSched S = SC.scheds[B.sched];
  const uint32_t* bidx = W.bidx + B.i0;
  float2* gp = W.pos[cur];
  float2* gq = W.prev;
  const uint2* gab = W.lab + B.l0;
  const float* grest = W.lrest + B.l0;
  const float* gstiff = W.lstiff + B.l0;
  const float gx = W.gx, gy = W.gy, h = W.h;
  DWorld Wb;  // bounds only
  Wb.bx = W.bx; Wb.by = W.by; Wb.bw = W.bw; Wb.bh = W.bh;

  // per group: body region | schedule area (sched_bytes: the whole schedule
  // when RES, else two fill buffers) | two mbarriers, a flag word and the
  // chunk count of each fill buffer
  unsigned char* base = smem + (size_t)g * (region_bytes + sched_bytes + GROUP_TAIL_BYTES);
  uint32_t* cbuf = reinterpret_cast<uint32_t*>(base + region_bytes);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + region_bytes + sched_bytes);
  volatile uint32_t* flag = reinterpret_cast<volatile uint32_t*>(bar + 2);
  volatile uint32_t* fill_n = flag + 2;
  // Streamed schedules arrive in fills: as many whole consecutive chunks as
  // one buffer of fill_words holds (a schedule's chunks are contiguous, so a
  // fill is one bulk copy).  Thread 0 issues fill c.. into buffer k2 and
  // returns the first chunk of the next fill.
  const uint32_t fill_words = sched_bytes / 8u;
  auto issue_fill = [&](uint32_t c, uint32_t k2) {
    uint32_t w = 0, e = c;
    while (e < S.nchunks) {
      const uint32_t l = SC.chunk_len[S.chunk0 + e];
      if (e > c && w + l > fill_words) break;
      w += l;
      ++e;
    }
    fill_n[k2] = e - c;
    bulk_load(cbuf + k2 * fill_words, SC.stream + SC.chunk_off[S.chunk0 + c], w * 4u, &bar[k2]);
    return e;
  };
  uint32_t next_c = 0;  // thread 0: first chunk not yet issued
  if (t == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    if (S.nchunks > 0) {
      if (RES) bulk_load(cbuf, SC.stream + S.off, S.words * 4u, &bar[0]);
      else next_c = issue_fill(0u, 0u);
    }
  }
  // body state in shared memory: pos[np], prev[np] (FULL), {rest, stiff}[nl]
  const uint32_t sp_a = smem_addr(base);
  const uint32_t sq_a = sp_a + 8u * B.np;
  const uint32_t srs_a = sq_a + (FULL ? 8u * B.np : 0u);
  if (SMEM) {
    // Link parameters first (static during a step), then, once the
    // previous kernel's positions are visible, the particles (plain stores,
    // so the compiler keeps many global loads in flight); a body whose
    // particles are contiguous in the world skips the bidx indirection.
    float2* sp = reinterpret_cast<float2*>(base);
    float2* sq = sp + B.np;
    float2* srs = sq + (FULL ? B.np : 0u);
#pragma unroll 4
    for (uint32_t i = t; i < B.nl; i += T) srs[i] = make_float2(grest[i], gstiff[i]);
    pdl_wait();
#pragma unroll 4
    for (uint32_t i = t; i < B.np; i += T) {
      const uint32_t k = B.first != NO_FIRST ? B.first + i : bidx[i];
      sp[i] = gp[k];
      if (FULL) sq[i] = gq[k];
    }
  } else {
    pdl_wait();
  }
  // a resident schedule is waited for once, under the same barrier (the
  // FAULT_BIT_WAIT test switch reports this first wait as timed out)
  if (RES && t == 0 && S.nchunks > 0)
    flag[0] = mbar_wait_bounded(&bar[0], 0u) && !(SC.fault & FAULT_BIT_WAIT) ? 1u : 0u;
  group_sync(g, T);
  if (RES && S.nchunks > 0) {
    if (flag[0] == 0u) {
      if (t == 0) {
        atomicOr(SC.err, ERR_BIT_TMA_TIMEOUT);
        mbar_wait_bounded(&bar[0], 0u);  // let the copy in flight land
      }
      return;  // every thread of the group leaves together
    }
    mbar_try(&bar[0], 0u);  // completed phase: makes the data visible here
  }

  // One op: a link solve or (FULL) bounds + integrate of one particle.
  // PAD: the schedule holds OP_NOP padding (whole-update schedules only);
  // the test is compiled in only for those, as it costs the others ~3 %
  auto run = [&](uint2 op, auto pad) {
    if constexpr (FULL && decltype(pad)::value) {
      if (op.y == OP_NOP) return;
    }
    if (FULL && op.y == OP_INTEG) {
      float2 p, q;
      if (SMEM) {
        p = lds_f32x2(sp_a + 8u * op.x);
        q = lds_f32x2(sq_a + 8u * op.x);
      } else {
        p = gp[bidx[op.x]];
        q = gq[bidx[op.x]];
      }
      solve_bounds(p, q, Wb);
      integrate(p, q, gx, gy, h);
      if (SMEM) {
        sts_f32x2(sp_a + 8u * op.x, p);
        sts_f32x2(sq_a + 8u * op.x, q);
      } else {
        gp[bidx[op.x]] = p;
        gq[bidx[op.x]] = q;
      }
    } else if (SMEM) {
      const float2 rs = lds_f32x2(srs_a + 8u * op.y);
      const uint32_t aa = sp_a + 8u * (op.x & 0xFFFFu), ba = sp_a + 8u * (op.x >> 16);
      float2 pa = lds_f32x2(aa), pb = lds_f32x2(ba);
      link_solve(pa, pb, rs.x, rs.y);
      sts_f32x2(aa, pa);
      sts_f32x2(ba, pb);
    } else {
      uint32_t ia, ib, kl;
      if (op.y == OP_WIDE) {
        kl = op.x;
        ia = gab[kl].x;
        ib = gab[kl].y;
      } else {
        kl = op.y;
        ia = bidx[op.x & 0xFFFFu];
        ib = bidx[op.x >> 16];
      }
      float2 pa = gp[ia], pb = gp[ib];
      link_solve(pa, pb, grest[kl], gstiff[kl]);
      gp[ia] = pa;
      gp[ib] = pb;
    }
  };
  // One chunk at shared address buf_a: its segments in order, each followed
  // by the group barrier; a segment's ops go to the group's threads in turn.
  // Returns the address just past the chunk.
  //
  // Every level is one dependency chain (barrier, op, positions, link solve,
  // stores, barrier), so the loop keeps everything else off it:
  // * ONE (no segment wider than the group): one predicated op per thread
  //   instead of an op loop;
  // * KIND, the group barrier (0 warp, 1 CTA, 2 named), fixed at compile
  //   time; ONE and KIND are chosen once per launch (`walk`);
  // * the segment ends sit in registers (a group is whole warps: lane i
  //   holds the end of segment s0 + i) and the next end is taken by shuffle
  //   before the barrier, so after it a thread's first load is its op.
  // A shared-memory prefetch of the next op ahead of the barrier measured
  // slower.
  auto run_chunk = [&](uint32_t buf_a, auto one, auto kind, auto pad) {
    constexpr bool ONE = decltype(one)::value;
    constexpr int KIND = decltype(kind)::value;
    const uint32_t nseg = lds_u32(buf_a);
    const uint32_t ops_a = buf_a + 4u * ((2u + nseg) & ~1u);
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t beg = 0;
    for (uint32_t s0 = 0; s0 < nseg; s0 += 32u) {
      const uint32_t n = min(32u, nseg - s0);  // uniform over the group
      const uint32_t my_end = lane < n ? lds_u32(buf_a + 4u + 4u * (s0 + lane)) : 0u;
      uint32_t end = __shfl_sync(0xFFFFFFFFu, my_end, 0);
      for (uint32_t j = 0; j < n; ++j) {
        if constexpr (ONE) {
          if (beg + t < end) run(lds_u32x2(ops_a + 8u * (beg + t)), pad);
        } else {
          for (uint32_t k = beg + t; k < end; k += T) run(lds_u32x2(ops_a + 8u * k), pad);
        }
        const uint32_t next = __shfl_sync(0xFFFFFFFFu, my_end, (j + 1u) & 31u);
        if constexpr (KIND == 0) {
          __syncwarp();
        } else if constexpr (KIND == 1) {
          __syncthreads();
        } else {
          asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(T) : "memory");
        }
        beg = end;
        end = next;
      }
    }
    return (ops_a + 8u * beg + 15u) & ~15u;  // chunks are padded to 16 bytes
  };
  const bool one = S.maxw <= T;
  const int kind = T == 32 ? 0 : (T == blockDim.x ? 1 : 2);  // as group_sync
  auto walk_pad = [&](uint32_t buf_a, auto pad) {
    using I0 = std::integral_constant<int, 0>;
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    if (one) {
      return kind == 1 ? run_chunk(buf_a, std::true_type{}, I1{}, pad)
             : kind == 0 ? run_chunk(buf_a, std::true_type{}, I0{}, pad)
                         : run_chunk(buf_a, std::true_type{}, I2{}, pad);
    }
    return kind == 1 ? run_chunk(buf_a, std::false_type{}, I1{}, pad)
           : kind == 0 ? run_chunk(buf_a, std::false_type{}, I0{}, pad)
                       : run_chunk(buf_a, std::false_type{}, I2{}, pad);
  };
  auto walk = [&](uint32_t buf_a) {
    if constexpr (FULL) {
      if (S.nop_pad) return walk_pad(buf_a, std::true_type{});
    }
    return walk_pad(buf_a, std::false_type{});
  };

  const uint32_t cbuf_a = smem_addr(cbuf);
  if (RES) {
    uint32_t buf_a = cbuf_a;
    for (uint32_t c = 0; c < S.nchunks; ++c) buf_a = walk(buf_a);
  } else {
    // buffer k2 = f & 1 holds fill f, used for the (f >> 1)-th time: its
    // mbarrier phase parity is (f >> 1) & 1
    uint32_t c = 0;
    for (uint32_t f = 0; c < S.nchunks; ++f) {
      const uint32_t k2 = f & 1u;
      const uint32_t par = (f >> 1) & 1u;
      if (t == 0)
        flag[0] = mbar_wait_bounded(&bar[k2], par) && !(f == 0 && (SC.fault & FAULT_BIT_WAIT))
                      ? 1u : 0u;
      group_sync(g, T);
      if (flag[0] == 0u) {
        if (t == 0) {
          atomicOr(SC.err, ERR_BIT_TMA_TIMEOUT);
          mbar_wait_bounded(&bar[k2], par);  // let the copy in flight land
        }
        return;  // every thread of the group leaves together
      }
      mbar_try(&bar[k2], par);  // completed phase: makes the data visible here
      const uint32_t n = fill_n[k2];
      if (t == 0 && next_c < S.nchunks) {  // the other buffer is free: next fill
        fence_proxy_async();
        next_c = issue_fill(next_c, k2 ^ 1u);
      }
      uint32_t buf_a = cbuf_a + k2 * fill_words * 4u;
      for (uint32_t j = 0; j < n; ++j) buf_a = walk(buf_a);
      c += n;
    }
  }

  if (SMEM) {
    const float2* sp = reinterpret_cast<const float2*>(base);
    const float2* sq = sp + B.np;
    if (!FULL && (W.flags & GRID_IN_LINKS)) {
      // store back and enter each particle into the grid (what
      // k_grid_insert / k_grid_count do for other worlds): into its bucket's
      // slots, or for the sorted grid its bucket and its rank in the bucket
      for (uint32_t i = t; i < B.np; i += T) {
        const uint32_t k = B.first != NO_FIRST ? B.first + i : bidx[i];
        const float2 p = sp[i];
        gp[k] = p;
        const int32_t cx = cell_coord(p.x, W.bx, W.cell, W.icell);
        const int32_t cy = cell_coord(p.y, W.by, W.cell, W.icell);
        const uint32_t b = bucket_of(W, cx, cy);
        if (GS.cell != nullptr) grid_insert(GS, sub, b, p, cx, cy);
        else gpbr[W.gp0 + k] = make_uint2(b, atomicAdd(&gcount[b], 1u));
      }
      return;
    }
#pragma unroll 4
    for (uint32_t i = t; i < B.np; i += T) {
      const uint32_t k = B.first != NO_FIRST ? B.first + i : bidx[i];
      gp[k] = sp[i];
      if (FULL) gq[k] = sq[i];
    }
  }
}

// ----------------------------------------------------------------------------
// Large-body executor: bodies whose state, link parameters and schedule do
// not fit one CTA's shared memory together, which the group executor would
// run from global memory (measured 2.4-4x slower per level than with the
// body in shared memory).  Here the body's positions (and previous
// positions, whole-step form) stay in shared memory, split over the C CTAs
// of a thread-block cluster (C = 1 when they fit one CTA): particle j lives
// in CTA j >> log2per at slot j & (per - 1), and every thread of the cluster
// reaches it through distributed shared memory (mapa + ld/st
// .shared::cluster).  Link parameters and the level schedule are read from
// global memory through the caches (they are never written during a step).
// A segment's ops go to the cluster's C*T threads in turn, and a cluster
// barrier (release / acquire) follows every segment, so each level sees
// the stores of the one before.  Nothing waits but those barriers, which
// every thread of the cluster reaches through the same sequence of
// segments (the schedule does not depend on the data), so no wait can hang.
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// all threads of the cluster (the non-.aligned form: threads need not be
// converged when they arrive)
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// the address of the same shared-memory offset in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t dsmem_addr(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}
__device__ __forceinline__ float2 ldc_f32x2(uint32_t a) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void stc_f32x2(uint32_t a, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}

template <bool FULL, bool CLUSTER>
__global__ void __launch_bounds__(1024) k_exec_large(const DWorld* __restrict__ worlds, DScheds SC,
                                                     const uint2* __restrict__ list, uint32_t nlist,
                                                     uint32_t C, uint32_t log2per, uint32_t cur,
                                                     uint32_t sub) {
  extern __shared__ __align__(16) unsigned char lsm[];
  // with cluster dimensions (C, 1, 1) the C consecutive CTAs of an item form
  // its cluster; every early return below is uniform over the cluster
  const uint32_t item = blockIdx.x / C;
  if (item >= nlist) return;
  const uint32_t rank = CLUSTER ? cluster_rank() : 0u;
  const uint2 wi = list[item];
  const DWorld& W = worlds[wi.x];
  if (!FULL && sub >= W.S) return;  // world already finished its sub-steps
  const DBody B = W.bodies[wi.y];
  const DSched S = SC.scheds[B.sched];
  const uint32_t* bidx = W.bidx + B.i0;
  float2* gp = W.pos[cur];
  float2* gq = W.prev;
  const uint2* gab = W.lab + B.l0;  // body-local endpoints
  const float* grest = W.lrest + B.l0;
  const float* gstiff = W.lstiff + B.l0;
  const float gx = W.gx, gy = W.gy, h = W.h;
  DWorld Wb;  // bounds only
  Wb.bx = W.bx; Wb.by = W.by; Wb.bw = W.bw; Wb.bh = W.bh;
  const uint32_t T = blockDim.x, t = threadIdx.x;
  const uint32_t per = 1u << log2per, mask = per - 1u;
  const uint32_t sp_a = smem_addr(lsm), sq_a = sp_a + 8u * per;
  // this CTA's slice of the body: particles [j0, j1)
  const uint32_t j0 = rank << log2per, j1 = min(B.np, j0 + per);
  for (uint32_t j = j0 + t; j < j1; j += T) {
    const uint32_t k = B.first != NO_FIRST ? B.first + j : bidx[j];
    sts_f32x2(sp_a + 8u * (j - j0), gp[k]);
    if (FULL) sts_f32x2(sq_a + 8u * (j - j0), gq[k]);
  }
  if (CLUSTER) cluster_barrier(); else __syncthreads();
  auto ld = [&](uint32_t base, uint32_t j) {
    const uint32_t a = base + 8u * (j & mask);
    return CLUSTER ? ldc_f32x2(dsmem_addr(a, j >> log2per)) : lds_f32x2(a);
  };
  auto st = [&](uint32_t base, uint32_t j, float2 v) {
    const uint32_t a = base + 8u * (j & mask);
    if (CLUSTER) stc_f32x2(dsmem_addr(a, j >> log2per), v); else sts_f32x2(a, v);
  };
  auto run = [&](uint2 op) {
    if (FULL && op.y == OP_NOP) return;  // padding of a whole-update schedule
    if (FULL && op.y == OP_INTEG) {  // bounds + integrate, src/solver.rs:155-158, :118-121
      float2 p = ld(sp_a, op.x), q = ld(sq_a, op.x);
      solve_bounds(p, q, Wb);
      integrate(p, q, gx, gy, h);
      st(sp_a, op.x, p);
      st(sq_a, op.x, q);
    } else {  // ParticleLink::solve, src/link.rs:18-27
      uint32_t ia, ib, kl;
      if (op.y == OP_WIDE) {
        kl = op.x;
        const uint2 e = __ldg(gab + kl);
        ia = e.x;
        ib = e.y;
      } else {
        kl = op.y;
        ia = op.x & 0xFFFFu;
        ib = op.x >> 16;
      }
      const float rest = __ldg(grest + kl), stiff = __ldg(gstiff + kl);
      float2 pa = ld(sp_a, ia), pb = ld(sp_a, ib);
      link_solve(pa, pb, rest, stiff);
      st(sp_a, ia, pa);
      st(sp_a, ib, pb);
    }
  };
  const uint32_t g = rank * T + t, CT = C * T;
  for (uint32_t c = 0; c < S.nchunks; ++c) {
    const uint32_t* ch = SC.stream + __ldg(SC.chunk_off + S.chunk0 + c);
    const uint32_t nseg = __ldg(ch);
    const uint2* ops = reinterpret_cast<const uint2*>(ch + ((2u + nseg) & ~1u));
    uint32_t beg = 0;
    for (uint32_t sg = 0; sg < nseg; ++sg) {
      const uint32_t end = __ldg(ch + 1u + sg);
      for (uint32_t k = beg + g; k < end; k += CT) run(__ldg(ops + k));
      if (CLUSTER) cluster_barrier(); else __syncthreads();
      beg = end;
    }
  }
  // every remote access happened before the last barrier: store the slice
  for (uint32_t j = j0 + t; j < j1; j += T) {
    const uint32_t k = B.first != NO_FIRST ? B.first + j : bidx[j];
    gp[k] = lds_f32x2(sp_a + 8u * (j - j0));
    if (FULL) gq[k] = lds_f32x2(sq_a + 8u * (j - j0));
  }
}

// ----------------------------------------------------------------------------
// Serial executor: one thread replays one body's reference loops directly, in
// insertion order (src/solver.rs:143-146, :155-158, :118-121).  Used for
// chain-like bodies (rings, ropes) whose level schedule has width ~1, where a
// whole group would idle.  This variant works on global memory (bodies too
// large for a shared-memory pack).
// ----------------------------------------------------------------------------
template <bool FULL>
__global__ void k_exec_serial(const DWorld* __restrict__ worlds, const uint2* __restrict__ list,
                              uint32_t n, uint32_t cur, uint32_t sub) {
  const uint32_t it0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (it0 >= n) return;
  const uint2 wi = list[it0];
  const DWorld& W = worlds[wi.x];
  if (!FULL && sub >= W.S) return;
  const DBody B = W.bodies[wi.y];
  float2* p = W.pos[cur];
  float2* q = W.prev;
  const uint2* ab = W.lab + B.l0;
  const float* rest = W.lrest + B.l0;
  const float* stiff = W.lstiff + B.l0;
  const uint32_t* bidx = W.bidx + B.i0;
  const uint32_t nsub = FULL ? W.S : 1u, I = W.I;
  const float gx = W.gx, gy = W.gy, h = W.h;
  DWorld Wb;
  Wb.bx = W.bx; Wb.by = W.by; Wb.bw = W.bw; Wb.bh = W.bh;
  // as in k_exec_serial_smem: link k + 1's positions are loaded before
  // link k's stores and forwarded from link k's registers where it wrote
  // them, so the global store-to-load round trip leaves the chain
  const uint32_t nl1 = B.nl ? B.nl - 1u : 0u;
  auto ends = [&](uint32_t k) {
    const uint2 e = ab[k];  // body-local endpoints
    return make_uint2(bidx[e.x], bidx[e.y]);
  };
  auto par = [&](uint32_t k) { return make_float2(rest[k], stiff[k]); };
  for (uint32_t s = 0; s < nsub; ++s) {
    for (uint32_t it = 0; it < I && B.nl; ++it) {
      uint2 e = ends(0), e1 = ends(nl1 < 1u ? nl1 : 1u);
      float2 r = par(0), r1 = par(nl1 < 1u ? nl1 : 1u);
      float2 pa = p[e.x], pb = p[e.y];
      for (uint32_t k = 0; k < B.nl; ++k) {
        const uint32_t k2 = k + 2u < nl1 ? k + 2u : nl1;
        const uint2 e2 = ends(k2);
        const float2 r2 = par(k2);
        float2 na = p[e1.x], nb = p[e1.y];  // link k + 1's, before link k's stores
        link_solve_plain(pa, pb, r.x, r.y);
        p[e.x] = pa;
        p[e.y] = pb;
        na = e1.x == e.x ? pa : (e1.x == e.y ? pb : na);
        nb = e1.y == e.x ? pa : (e1.y == e.y ? pb : nb);
        pa = na;
        pb = nb;
        e = e1;
        e1 = e2;
        r = r1;
        r1 = r2;
      }
    }
    if (FULL) {
      for (uint32_t k = 0; k < B.np; ++k) {
        const uint32_t j = bidx[k];
        float2 pp = p[j], qq = q[j];
        solve_bounds(pp, qq, Wb);
        integrate(pp, qq, gx, gy, h);
        p[j] = pp;
        q[j] = qq;
      }
    }
  }
}

// Serial executor, shared-memory variant: a CTA runs a pack of chain-like
// bodies, one thread per body, with every body's positions (and prev) in
// shared memory, so each step of the chain costs shared-memory latency
// instead of a global round trip.  STAGED packs also hold the links
// (endpoints, {rest, stiffness}) in shared memory: measured on one thread
// replaying a 4,088-particle ring, 211 cycles per link (with the next link's
// data loaded one link ahead) against 333 with the link data read through
// the read-only cache.  pack = {first item, item count}; base[i] = item i's
// first particle slot and first link slot.
template <bool FULL, bool STAGED>
__global__ void k_exec_serial_smem(const DWorld* __restrict__ worlds,
                                   const uint2* __restrict__ items,
                                   const uint2* __restrict__ base,
                                   const uint2* __restrict__ packs, uint32_t npacks, uint32_t cur,
                                   uint32_t sub) {
  extern __shared__ __align__(16) float2 sstate[];
  if (blockIdx.x >= npacks) return;
  const uint2 pk = packs[blockIdx.x];
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  const uint32_t warp = tid >> 5, lane = tid & 31u, nwarps = nt >> 5;
  // pack-wide particle and link counts: [pos | prev (FULL) | ab | {rest, stiff}]
  const uint32_t last = pk.x + pk.y - 1;
  const DBody BL = worlds[items[last].x].bodies[items[last].y];
  const uint32_t total = base[last].x + BL.np, ltotal = STAGED ? base[last].y + BL.nl : 0u;
  float2* spos = sstate;
  float2* sprev = sstate + total;
  uint2* sab = reinterpret_cast<uint2*>(sstate + (FULL ? 2u : 1u) * total);
  float2* srs = reinterpret_cast<float2*>(sab + ltotal);
  // cooperative load, one warp per body
  for (uint32_t it = warp; it < pk.y; it += nwarps) {
    const uint2 wi = items[pk.x + it];
    const DWorld& W = worlds[wi.x];
    if (!FULL && sub >= W.S) continue;
    const DBody B = W.bodies[wi.y];
    const uint32_t* bidx = W.bidx + B.i0;
    const uint2 sb = base[pk.x + it];
    for (uint32_t i = lane; i < B.np; i += 32) {
      const uint32_t k = B.first != NO_FIRST ? B.first + i : bidx[i];
      spos[sb.x + i] = W.pos[cur][k];
      if (FULL) sprev[sb.x + i] = W.prev[k];
    }
    if (STAGED) {
      for (uint32_t i = lane; i < B.nl; i += 32) {
        sab[sb.y + i] = W.lab[B.l0 + i];  // body-local endpoints
        srs[sb.y + i] = make_float2(W.lrest[B.l0 + i], W.lstiff[B.l0 + i]);
      }
    } else {
      // the chain reads each link's data one link ahead, which hides an L2
      // hit but not a DRAM access: bring the body's link arrays into L2
      // now, one prefetch per 128-byte line (endpoints 8 B, rest and
      // stiffness 4 B a link)
      const char* ab = reinterpret_cast<const char*>(W.lab + B.l0);
      const char* rs = reinterpret_cast<const char*>(W.lrest + B.l0);
      const char* sf = reinterpret_cast<const char*>(W.lstiff + B.l0);
      for (uint32_t o = 128u * lane; o < 8u * B.nl; o += 32u * 128u)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(ab + o));
      for (uint32_t o = 128u * lane; o < 4u * B.nl; o += 32u * 128u) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(rs + o));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(sf + o));
      }
    }
  }
  __syncthreads();
  if (tid < pk.y) {
    const uint2 wi = items[pk.x + tid];
    const DWorld& W = worlds[wi.x];
    if (FULL || sub < W.S) {
      const DBody B = W.bodies[wi.y];
      const uint2 sb = base[pk.x + tid];
      float2* p = spos + sb.x;
      float2* q = sprev + sb.x;
      const uint2* ab = STAGED ? sab + sb.y : W.lab + B.l0;  // body-local endpoints
      const float2* rs = srs + sb.y;
      const float* grest = W.lrest + B.l0;
      const float* gstiff = W.lstiff + B.l0;
      const uint32_t nsub = FULL ? W.S : 1u, I = W.I;
      const float gx = W.gx, gy = W.gy, h = W.h;
      DWorld Wb;
      Wb.bx = W.bx; Wb.by = W.by; Wb.bw = W.bw; Wb.bh = W.bh;
      // Link k's endpoints and parameters are loaded two links ahead and its
      // positions one link ahead, before link k - 1's stores: a position
      // that link k - 1 writes is taken from its registers instead
      // (forwarded), so neither the parameter loads nor the shared-memory
      // store-to-load round trip sit on the chain, which is then one link
      // solve and two selects per link.
      auto link_at = [&](uint32_t k, uint2& e, float2& r) {
        e = STAGED ? ab[k] : __ldg(ab + k);
        r = STAGED ? rs[k] : make_float2(__ldg(grest + k), __ldg(gstiff + k));
      };
      const uint32_t nl1 = B.nl ? B.nl - 1u : 0u;
      for (uint32_t s = 0; s < nsub; ++s) {
        for (uint32_t it = 0; it < I && B.nl; ++it) {
          uint2 e, e1;
          float2 r, r1;
          link_at(0, e, r);
          link_at(nl1 < 1u ? nl1 : 1u, e1, r1);
          float2 pa = p[e.x], pb = p[e.y];
          for (uint32_t k = 0; k < B.nl; ++k) {
            uint2 e2;
            float2 r2;
            link_at(k + 2u < nl1 ? k + 2u : nl1, e2, r2);
            float2 na = p[e1.x], nb = p[e1.y];  // link k + 1's, before link k's stores
            link_solve_plain(pa, pb, r.x, r.y);
            p[e.x] = pa;
            p[e.y] = pb;
            na = e1.x == e.x ? pa : (e1.x == e.y ? pb : na);
            nb = e1.y == e.x ? pa : (e1.y == e.y ? pb : nb);
            pa = na;
            pb = nb;
            e = e1;
            r = r1;
            e1 = e2;
            r1 = r2;
          }
        }
        if (FULL) {
          // particles are independent here: four at a time, loads before
          // stores (measured 100 instead of 134 cycles per particle)
          uint32_t k = 0;
          for (; k + 4 <= B.np; k += 4) {
            float2 pp[4], qq[4];
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) {
              pp[j] = p[k + j];
              qq[j] = q[k + j];
            }
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) {
              solve_bounds(pp[j], qq[j], Wb);
              integrate(pp[j], qq[j], gx, gy, h);
            }
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) {
              p[k + j] = pp[j];
              q[k + j] = qq[j];
            }
          }
          for (; k < B.np; ++k) {
            float2 pp = p[k], qq = q[k];
            solve_bounds(pp, qq, Wb);
            integrate(pp, qq, gx, gy, h);
            p[k] = pp;
            q[k] = qq;
          }
        }
      }
    }
  }
  __syncthreads();
  for (uint32_t it = warp; it < pk.y; it += nwarps) {
    const uint2 wi = items[pk.x + it];
    const DWorld& W = worlds[wi.x];
    if (!FULL && sub >= W.S) continue;
    const DBody B = W.bodies[wi.y];
    const uint32_t* bidx = W.bidx + B.i0;
    const uint32_t sb = base[pk.x + it].x;
    for (uint32_t i = lane; i < B.np; i += 32) {
      const uint32_t k = B.first != NO_FIRST ? B.first + i : bidx[i];
      W.pos[cur][k] = spos[sb + i];
      if (FULL) W.prev[k] = sprev[sb + i];
    }
  }
}

// ----------------------------------------------------------------------------
// Rigid executor: the circles and polygons of one world per CTA.  The
// reference's sequential pair loops (circle pairs i<j; polygon pairs i<j in
// both directions) run speculatively: every remaining test of a window is
// evaluated in parallel on the current state; the first test, in reference
// order, that changes state is applied alone and evaluation resumes right
// after it.  Tests before the first hit changed nothing, so the outcome is
// the sequential one.
// ----------------------------------------------------------------------------
__device__ __forceinline__ void calc_center(const float2* v, uint32_t n, float2& c) {
  // Polygon::calc_center, src/polygon.rs:231-237: sequential sum from 0, / n
  float cx = 0.0f, cy = 0.0f;
  for (uint32_t i = 0; i < n; ++i) { cx = fadd(cx, v[i].x); cy = fadd(cy, v[i].y); }
  c.x = fdiv(cx, (float)n);
  c.y = fdiv(cy, (float)n);
}

// common::line_intersection, src/common.rs:3-26
// Both parameters are quotients by the same denominator and a hit needs both
// in [0, 1].  When a numerator's magnitude exceeds 2|den| (or it is NaN), the
// correctly rounded quotient is at least 2 in magnitude, infinite or NaN, so
// the test fails whatever the division returns: the divisions are skipped.
// 2|den| is exact (or infinite on overflow, which skips nothing), so the
// outcome is the reference's in every case.  Most pair tests of separated
// polygons end here.
__device__ __forceinline__ bool line_intersection(float2 p1, float2 p2, float2 p3, float2 p4,
                                                  float2& out) {
  float s1x = fsub(p2.x, p1.x), s1y = fsub(p2.y, p1.y);
  float s2x = fsub(p4.x, p3.x), s2y = fsub(p4.y, p3.y);
  float d13x = fsub(p1.x, p3.x), d13y = fsub(p1.y, p3.y);
  float den = fadd(fmul(-s2x, s1y), fmul(s1x, s2y));
  const float ns = fadd(fmul(-s1y, d13x), fmul(s1x, d13y));
  const float nt = fsub(fmul(s2x, d13y), fmul(s2y, d13x));
  const float lim = fmul(2.0f, fabsf(den));
  if (!(fabsf(ns) <= lim && fabsf(nt) <= lim)) return false;
  float s = fdiv(ns, den);
  float t = fdiv(nt, den);
  if (s >= 0.0f && s <= 1.0f && t >= 0.0f && t <= 1.0f) {
    out.x = fadd(p1.x, fmul(t, s1x));
    out.y = fadd(p1.y, fmul(t, s1y));
    return true;
  }
  return false;
}

__device__ __forceinline__ float2 normalize2(float x, float y) {
  float n = fsqrt(norm_sq(x, y));
  return make_float2(fdiv(x, n), fdiv(y, n));
}

// Polygon::resolve_line_intersection, src/polygon.rs:164-216
static __device__ bool resolve_line(float2 self_center, float2 pa, float2 pb, float2 q,
                             float2 other_center, float2& na, float2& nb, float2& nq) {
  float2 I;
  if (!line_intersection(pa, pb, q, other_center, I)) return false;
  float2 nl = normalize2(fsub(pb.x, pa.x), fsub(pb.y, pa.y));
  float k = fdiv(dot2(nl.x, nl.y, fsub(self_center.x, I.x), fsub(self_center.y, I.y)),
                 dot2(nl.x, nl.y, nl.x, nl.y));
  float2 cp = make_float2(fmul(nl.x, k), fmul(nl.y, k));
  float2 ni = normalize2(fsub(self_center.x, fadd(I.x, cp.x)), fsub(self_center.y, fadd(I.y, cp.y)));
  float dax = fsub(I.x, pa.x), day = fsub(I.y, pa.y);
  float dbx = fsub(I.x, pb.x), dby = fsub(I.y, pb.y);
  float dist_a = fsqrt(norm_sq(dax, day));
  float dist_b = fsqrt(norm_sq(dbx, dby));
  float dab = fadd(dist_a, dist_b);
  float inf_a = fdiv(dist_b, dab), inf_b = fdiv(dist_a, dab);
  float dx = fsub(I.x, q.x), dy = fsub(I.y, q.y);
  float kk = fdiv(dot2(ni.x, ni.y, dx, dy), dot2(ni.x, ni.y, ni.x, ni.y));
  float onx = fmul(ni.x, kk), ony = fmul(ni.y, kk);
  float lx = fmul(fdiv(onx, 3.0f), 2.0f), ly = fmul(fdiv(ony, 3.0f), 2.0f);
  float2 a2 = make_float2(fsub(pa.x, fmul(lx, inf_a)), fsub(pa.y, fmul(ly, inf_a)));
  float2 b2 = make_float2(fsub(pb.x, fmul(lx, inf_b)), fsub(pb.y, fmul(ly, inf_b)));
  float2 far = make_float2(fsub(q.x, fmul(ni.x, 10000.0f)), fsub(q.y, fmul(ni.y, 10000.0f)));
  float2 hit;
  if (line_intersection(pa, pb, q, far, hit)) {
    na = a2; nb = b2; nq = hit;
    return true;
  }
  return false;
}

// Circle::solve_circle, src/circle.rs:32-45 (state-changing part)
__device__ __forceinline__ bool circle_pair_hits(float2 pi, float ri, float2 pj, float rj) {
  float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y);
  float rs = fadd(ri, rj);
  return norm_sq(dx, dy) < fmul(rs, rs);
}
__device__ __forceinline__ void circle_pair_apply(float2& pi, float ri, float2& pj, float rj) {
  float dx = fsub(pi.x, pj.x), dy = fsub(pi.y, pj.y);
  float d2 = norm_sq(dx, dy);
  float rs = fadd(ri, rj);
  if (d2 < fmul(rs, rs)) {
    float2 n = normalize2(dx, dy);
    float overlap = fsub(rs, fsqrt(d2));
    float ri2 = fmul(ri, ri), rj2 = fmul(rj, rj);
    float scale = fdiv(1.0f, fadd(ri2, rj2));
    pi.x = fadd(pi.x, fmul(fmul(fmul(n.x, scale), overlap), rj2));
    pi.y = fadd(pi.y, fmul(fmul(fmul(n.y, scale), overlap), rj2));
    pj.x = fsub(pj.x, fmul(fmul(fmul(n.x, scale), overlap), ri2));
    pj.y = fsub(pj.y, fmul(fmul(fmul(n.y, scale), overlap), ri2));
  }
}

// CircleLink::solve, src/link.rs:36-48
__device__ __forceinline__ void circle_link_solve(float2& a, float ra, float2& b, float rb,
                                                  float rest) {
  float dx = fsub(a.x, b.x), dy = fsub(a.y, b.y);
  float dist = fsqrt(norm_sq(dx, dy));
  float nx = fdiv(dx, dist), ny = fdiv(dy, dist);
  float ra2 = fmul(ra, ra), rb2 = fmul(rb, rb);
  float scale = fdiv(1.0f, fadd(ra2, rb2));
  float m = fsub(dist, rest);
  a.x = fsub(a.x, fmul(fmul(fmul(nx, m), scale), rb2));
  a.y = fsub(a.y, fmul(fmul(fmul(ny, m), scale), rb2));
  b.x = fadd(b.x, fmul(fmul(fmul(nx, m), scale), ra2));
  b.y = fadd(b.y, fmul(fmul(fmul(ny, m), scale), ra2));
}

__device__ __forceinline__ uint64_t pair_row_off(uint64_t i, uint64_t n) {
  return i * (2 * n - i - 1) / 2;
}
// k-th pair (i<j) in row-major order over n items
// k-th pair (i<j) in row-major order over n items: binary search for the
// last row whose first pair index is <= k (integer arithmetic only)
__device__ __forceinline__ void unrank_pair(uint64_t k, uint32_t n, uint32_t& i, uint32_t& j) {
  uint32_t lo = 0, hi = n - 1;  // row in [lo, hi)
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (pair_row_off(mid, n) <= k) lo = mid; else hi = mid;
  }
  i = lo;
  j = (uint32_t)(k - pair_row_off(lo, n) + lo + 1);
}

// Polygon pair "stages": stage s = (self, other) in reference order (pairs
// i<j row-major; (i,j) then (j,i)).  Test x within a stage is (edge e of
// self, point q of other), numbered e*nv_other + q.  The host stores
// stage_off[s] = first test of stage s (and the total after the last stage)
// and stage_pr[s] = self | other << 16.
__device__ __forceinline__ void stage_pair(const uint32_t* pr, uint32_t s, uint32_t& self,
                                           uint32_t& other) {
  const uint32_t v = pr[s];  // self | other << 16, precomputed on the host
  self = v & 0xFFFFu;
  other = v >> 16;
}

__device__ __forceinline__ uint32_t stage_of(const uint32_t* so, uint32_t nstage, uint32_t x) {
  uint32_t lo = 0, hi = nstage;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (so[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}

// Circle and polygon arrays of one world, in global or shared memory.
struct RigidView {
  float2* cp; float2* cq; float2* ca; float* cr; uint32_t* cst;
  uint2* clab; float* clrest;
  DPoly* polys; float2* vpos; float2* vprev; float2* vacc; float2* pcenter; float4* paabb;
  uint2* plab; float* plrest; uint32_t* stage_off; uint32_t* stage_pr;
  uint32_t nc, ncl, ng, nv, npl, nst;
};

__device__ __forceinline__ RigidView global_view(const DWorld& W) {
  RigidView v;
  v.cp = W.cpos; v.cq = W.cprev; v.ca = W.cacc; v.cr = W.crad; v.cst = W.cstatic;
  v.clab = W.clab; v.clrest = W.clrest;
  v.polys = W.polys; v.vpos = W.vpos; v.vprev = W.vprev; v.vacc = W.vacc;
  v.pcenter = W.pcenter; v.paabb = W.paabb; v.plab = W.plab; v.plrest = W.plrest;
  v.stage_off = W.stage_off;
  v.stage_pr = W.stage_pr;
  v.nc = W.nc; v.ncl = W.ncl; v.ng = W.ng;
  v.nv = W.ng ? W.polys[W.ng - 1].v0 + W.polys[W.ng - 1].nv : 0u;
  v.npl = W.ng ? W.polys[W.ng - 1].l0 + W.polys[W.ng - 1].nl : 0u;
  v.nst = W.ng >= 2 ? W.ng * (W.ng - 1) + 1 : 0u;
  return v;
}

__device__ __forceinline__ uint32_t rigid_smem_bytes(const RigidView& v) {
  // payload plus 16-byte rounding of the 16 pieces (stage_view)
  return 48u * v.ng + 28u * v.nc + 12u * v.ncl + 24u * v.nv + 12u * v.npl + 8u * v.nst + 272u;
}

// carve a shared-memory view (16-byte aligned pieces first)
__device__ __forceinline__ RigidView stage_view(const RigidView& g, unsigned char* sm) {
  RigidView v = g;
  unsigned char* p = sm;
  auto take = [&](size_t bytes) { unsigned char* q = p; p += (bytes + 15) & ~(size_t)15; return q; };
  v.paabb = reinterpret_cast<float4*>(take(16u * g.ng));
  v.polys = reinterpret_cast<DPoly*>(take(24u * g.ng));
  v.pcenter = reinterpret_cast<float2*>(take(8u * g.ng));
  v.cp = reinterpret_cast<float2*>(take(8u * g.nc));
  v.cq = reinterpret_cast<float2*>(take(8u * g.nc));
  v.ca = reinterpret_cast<float2*>(take(8u * g.nc));
  v.vpos = reinterpret_cast<float2*>(take(8u * g.nv));
  v.vprev = reinterpret_cast<float2*>(take(8u * g.nv));
  v.vacc = reinterpret_cast<float2*>(take(8u * g.nv));
  v.clab = reinterpret_cast<uint2*>(take(8u * g.ncl));
  v.plab = reinterpret_cast<uint2*>(take(8u * g.npl));
  v.cr = reinterpret_cast<float*>(take(4u * g.nc));
  v.cst = reinterpret_cast<uint32_t*>(take(4u * g.nc));
  v.clrest = reinterpret_cast<float*>(take(4u * g.ncl));
  v.plrest = reinterpret_cast<float*>(take(4u * g.npl));
  v.stage_off = reinterpret_cast<uint32_t*>(take(4u * g.nst));
  v.stage_pr = reinterpret_cast<uint32_t*>(take(4u * g.nst));
  return v;
}

// copy a view's arrays: everything when `all`, else only the mutable state
__device__ __forceinline__ void copy_view(const RigidView& d, const RigidView& s, bool all) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  for (uint32_t i = tid; i < s.nc; i += nt) {
    d.cp[i] = s.cp[i]; d.cq[i] = s.cq[i]; d.ca[i] = s.ca[i];
    if (all) { d.cr[i] = s.cr[i]; d.cst[i] = s.cst[i]; }
  }
  for (uint32_t i = tid; i < s.nv; i += nt) {
    d.vpos[i] = s.vpos[i]; d.vprev[i] = s.vprev[i]; d.vacc[i] = s.vacc[i];
  }
  for (uint32_t i = tid; i < s.ng; i += nt) {
    d.pcenter[i] = s.pcenter[i]; d.paabb[i] = s.paabb[i];
    if (all) d.polys[i] = s.polys[i];
  }
  if (all) {
    for (uint32_t i = tid; i < s.ncl; i += nt) { d.clab[i] = s.clab[i]; d.clrest[i] = s.clrest[i]; }
    for (uint32_t i = tid; i < s.npl; i += nt) { d.plab[i] = s.plab[i]; d.plrest[i] = s.plrest[i]; }
    for (uint32_t i = tid; i < s.nst; i += nt) d.stage_off[i] = s.stage_off[i];
    for (uint32_t i = tid + 1; i < s.nst; i += nt) d.stage_pr[i - 1] = s.stage_pr[i - 1];
  }
}

// gravity + links + circle pairs + polygon pairs of one sub-step for the
// circles and polygons (src/solver.rs:110-112)
__device__ __forceinline__ void rigid_phase_a(const DWorld& W, const RigidView& R, bool want_aabb) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  float2* cp = R.cp;
  float2* ca = R.ca;
  const float* cr = R.cr;
  const DPoly* polys = R.polys;
  __shared__ uint32_t s_first;
  // gravity, src/solver.rs:130-141 (static bodies included)
  for (uint32_t i = tid; i < W.nc; i += nt) {
    float2 a = ca[i];
    a.x = fadd(a.x, W.gx); a.y = fadd(a.y, W.gy);
    ca[i] = a;
  }
  for (uint32_t g = 0; g < W.ng; ++g) {
    const DPoly P = polys[g];
    for (uint32_t v = tid; v < P.nv; v += nt) {
      float2 a = R.vacc[P.v0 + v];
      a.x = fadd(a.x, W.gx); a.y = fadd(a.y, W.gy);
      R.vacc[P.v0 + v] = a;
    }
  }
  __syncthreads();
  // links, src/solver.rs:143-153, repeated I times (extension)
  for (uint32_t it = 0; it < W.I; ++it) {
    if (tid == 0) {
      for (uint32_t k = 0; k < W.ncl; ++k) {
        const uint2 e = R.clab[k];
        float2 pa = cp[e.x], pb = cp[e.y];
        circle_link_solve(pa, cr[e.x], pb, cr[e.y], R.clrest[k]);
        cp[e.x] = pa; cp[e.y] = pb;
      }
    }
    for (uint32_t g = tid; g < W.ng; g += nt) {  // one thread per polygon
      const DPoly P = polys[g];
      float2* v = R.vpos + P.v0;
      float2 c;
      calc_center(v, P.nv, c);  // Polygon::solve_links, src/polygon.rs:218-223
      R.pcenter[g] = c;
      for (uint32_t k = 0; k < P.nl; ++k) {
        const uint2 e = R.plab[P.l0 + k];
        float2 pa = v[e.x], pb = v[e.y];
        link_solve(pa, pb, R.plrest[P.l0 + k], 1.0f);
        v[e.x] = pa; v[e.y] = pb;
      }
    }
    __syncthreads();
  }
  // circle pairs, src/solver.rs:168-177, speculative windows of nt pairs
  {
    const uint64_t npairs = W.nc >= 2 ? (uint64_t)W.nc * (W.nc - 1) / 2 : 0;
    uint64_t start = 0;
    while (start < npairs) {
      if (tid == 0) s_first = 0xFFFFFFFFu;
      __syncthreads();
      const uint64_t k = start + tid;
      if (k < npairs) {
        uint32_t i, j;
        unrank_pair(k, W.nc, i, j);
        if (circle_pair_hits(cp[i], cr[i], cp[j], cr[j])) atomicMin(&s_first, tid);
      }
      __syncthreads();
      const uint32_t f = s_first;
      if (f == 0xFFFFFFFFu) {
        start += nt;
      } else {
        if (tid == f) {
          uint32_t i, j;
          unrank_pair(k, W.nc, i, j);
          float2 pi = cp[i], pj = cp[j];
          circle_pair_apply(pi, cr[i], pj, cr[j]);
          cp[i] = pi; cp[j] = pj;
        }
        start += f + 1;
      }
      __syncthreads();
    }
  }
  // polygon pairs, src/solver.rs:178-187 + src/polygon.rs:142-216
  const uint32_t nstage = W.ng >= 2 ? W.ng * (W.ng - 1) : 0;
  if (nstage > 0) {
    const uint32_t* so = R.stage_off;
    const uint32_t total = so[nstage];
    uint32_t start = 0;
    while (start < total) {
      if (tid == 0) s_first = 0xFFFFFFFFu;
      __syncthreads();
      const uint32_t x = start + tid;
      if (x < total) {
        const uint32_t st = stage_of(so, nstage, x);
        uint32_t self, other;
        stage_pair(R.stage_pr, st, self, other);
        const DPoly PS = polys[self], PO = polys[other];
        const uint32_t r = x - so[st];
        const uint32_t e = r / PO.nv;
        const uint32_t q = r - e * PO.nv;
        const uint32_t b = (e + 1) % PS.nv;
        float2 na, nb, nq;
        if (resolve_line(R.pcenter[self], R.vpos[PS.v0 + e], R.vpos[PS.v0 + b],
                         R.vpos[PO.v0 + q], R.pcenter[other], na, nb, nq))
          atomicMin(&s_first, x);
      }
      __syncthreads();
      const uint32_t f = s_first;
      __syncthreads();
      if (f == 0xFFFFFFFFu) {
        start += nt;
        continue;
      }
      // Apply the whole edge step holding test f: every point of `other`, in
      // order.  The edge endpoints are copies taken before the point loop, so
      // the last hit sets them (src/polygon.rs:148-160).
      if (tid == 0) {
        const uint32_t st = stage_of(so, nstage, f);
        uint32_t self, other;
        stage_pair(R.stage_pr, st, self, other);
        const DPoly PS = polys[self], PO = polys[other];
        const uint32_t e = (f - so[st]) / PO.nv;
        const uint32_t b = (e + 1) % PS.nv;
        const float2 pa = R.vpos[PS.v0 + e], pb = R.vpos[PS.v0 + b];
        const float2 sc = R.pcenter[self], oc = R.pcenter[other];
        for (uint32_t q = 0; q < PO.nv; ++q) {
          float2 na, nb, nq;
          if (resolve_line(sc, pa, pb, R.vpos[PO.v0 + q], oc, na, nb, nq)) {
            R.vpos[PS.v0 + e] = na;
            R.vpos[PS.v0 + b] = nb;
            R.vpos[PO.v0 + q] = nq;
          }
        }
        s_first = so[st] + (e + 1) * PO.nv;  // first test of the next edge step
      }
      __syncthreads();
      start = s_first;
      __syncthreads();
    }
  }
  // extension: polygon vertex bounding boxes for particle-polygon contacts
  if (want_aabb) {
    for (uint32_t g = tid; g < W.ng; g += nt) {
      const DPoly P = polys[g];
      const float2* v = R.vpos + P.v0;
      float4 bb = make_float4(0.f, 0.f, 0.f, 0.f);
      if (P.nv > 0) {
        bb = make_float4(v[0].x, v[0].y, v[0].x, v[0].y);
        for (uint32_t i = 1; i < P.nv; ++i) {
          if (v[i].x < bb.x) bb.x = v[i].x;
          if (v[i].y < bb.y) bb.y = v[i].y;
          if (v[i].x > bb.z) bb.z = v[i].x;
          if (v[i].y > bb.w) bb.w = v[i].y;
        }
      }
      R.paabb[g] = bb;
    }
  }
  __syncthreads();
}

// bounds + integrate of one sub-step for the circles and polygons
// (src/solver.rs:113-114)
__device__ __forceinline__ void rigid_phase_b(const DWorld& W, const RigidView& R) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  float2* cp = R.cp;
  float2* cq = R.cq;
  float2* ca = R.ca;
  const float* cr = R.cr;
  const DPoly* polys = R.polys;
  // bounds, src/solver.rs:155-165
  for (uint32_t i = tid; i < W.nc; i += nt) {
    float2 p = cp[i], q = cq[i];
    circle_bounds(p, q, cr[i], W);
    cp[i] = p; cq[i] = q;
  }
  for (uint32_t g = 0; g < W.ng; ++g) {
    const DPoly P = polys[g];
    for (uint32_t v = tid; v < P.nv; v += nt) {
      float2 p = R.vpos[P.v0 + v], q = R.vprev[P.v0 + v];
      solve_bounds(p, q, W);
      R.vpos[P.v0 + v] = p; R.vprev[P.v0 + v] = q;
    }
  }
  __syncthreads();
  // update_positions, src/solver.rs:118-128
  for (uint32_t i = tid; i < W.nc; i += nt) {
    if (R.cst[i]) continue;  // extension: static circle
    float2 p = cp[i], q = cq[i];
    const float2 a = ca[i];
    integrate(p, q, a.x, a.y, W.h);
    cp[i] = p; cq[i] = q; ca[i] = make_float2(0.0f, 0.0f);
  }
  for (uint32_t g = tid; g < W.ng; g += nt) {  // Polygon::update, src/polygon.rs:125-134
    const DPoly P = polys[g];
    if (P.is_static) continue;
    float2 c;
    calc_center(R.vpos + P.v0, P.nv, c);
    R.pcenter[g] = c;
  }
  __syncthreads();
  for (uint32_t g = 0; g < W.ng; ++g) {
    const DPoly P = polys[g];
    if (P.is_static) continue;
    for (uint32_t v = tid; v < P.nv; v += nt) {
      float2 p = R.vpos[P.v0 + v], q = R.vprev[P.v0 + v];
      const float2 a = R.vacc[P.v0 + v];
      integrate(p, q, a.x, a.y, W.h);
      R.vpos[P.v0 + v] = p; R.vprev[P.v0 + v] = q;
      R.vacc[P.v0 + v] = make_float2(0.0f, 0.0f);
    }
  }
  __syncthreads();
}

// MODE 0: the whole Solver::update step; 1: phase A of sub-step `sub`;
// 2: phase B of sub-step `sub`; 3: phase B of `sub`-1, then phase A of `sub`.
// The world's circles and polygons are staged in shared memory when they fit
// in `smem_bytes` (serial chains then cost shared-memory latency), else the
// phases run on global memory.  THREADS (256 or 1024) is the window of the
// speculative pair loops: worlds with thousands of pair tests take the wide
// CTA (four times fewer windows and barriers, and four times the warps to
// hide each window's latency on the one SM that runs the world).
template <int MODE, int THREADS = 256>
__global__ void __launch_bounds__(THREADS) k_rigid(const DWorld* __restrict__ worlds,
                                               const uint32_t* __restrict__ wlist, uint32_t n,
                                               uint32_t sub, uint32_t smem_bytes) {
  extern __shared__ __align__(16) unsigned char rsm[];
  if (blockIdx.x >= n) return;
  const DWorld& W = worlds[wlist[blockIdx.x]];
  if (MODE == 1 && sub >= W.S) return;
  if (MODE == 2 && sub >= W.S) return;
  if (MODE == 3 && sub > W.S) return;
  const bool aabb = (W.flags & COLLIDE_PPOLY) != 0;
  RigidView G = global_view(W);
  RigidView R = G;
  const bool staged = rigid_smem_bytes(G) <= smem_bytes;
  if (staged) {
    R = stage_view(G, rsm);
    copy_view(R, G, true);
    __syncthreads();
  }
  if (MODE == 0) {
    for (uint32_t s = 0; s < W.S; ++s) {
      rigid_phase_a(W, R, false);
      rigid_phase_b(W, R);
    }
  } else if (MODE == 1) {
    rigid_phase_a(W, R, aabb);
  } else if (MODE == 2) {
    rigid_phase_b(W, R);
  } else {
    if (sub >= 1 && sub - 1 < W.S) rigid_phase_b(W, R);
    if (sub < W.S) rigid_phase_a(W, R, aabb);
  }
  if (staged) {
    __syncthreads();
    copy_view(G, R, false);
  }
}

// ----------------------------------------------------------------------------
// Extension: particle collisions (not in the reference, whose solver
// particles only interact through links, src/solver.rs:143-188).  Hashed
// uniform grid, rebuilt every sub-step (slot inserts, or a counting sort for
// large grids); Jacobi contacts against every particle of the 9 surrounding
// cells, summed in fixed point so that the result does not depend on the
// visiting order.
// ----------------------------------------------------------------------------
// particles per work chunk: one CTA of the insert / count / scatter /
// copy-back kernels, four collide CTAs of 8 warps x 10 particles
constexpr uint32_t CHUNK = 320;

// Bucket entry: {pos.x bits, pos.y bits, cell x, cell y}.  Cells that hash
// to the same bucket are told apart by the stored cell coordinates, so the
// neighbour search is exact whatever the hashing.
static __global__ void __launch_bounds__(CHUNK) k_grid_count(const DWorld* __restrict__ worlds, DGrid G,
                                                      const uint2* __restrict__ chunks,
                                                      uint32_t nchunks, uint32_t cur, uint32_t sub) {
  pdl_trigger();
  // chunk and world records are fixed during a step: read before the wait
  const uint2 ch = chunks[blockIdx.x < nchunks ? blockIdx.x : 0u];
  const DWorld& W = worlds[ch.x];
  const uint32_t j = ch.y + threadIdx.x;
  const bool act = blockIdx.x < nchunks && j < W.np && sub < W.S &&
                   (W.flags & (COLLIDE_PP | GRID_IN_LINKS)) == COLLIDE_PP;
  const float2* P = W.pos[cur];
  pdl_wait();  // positions from the link phase
  if (!act) return;
  const float2 p = P[j];
  const int32_t cx = cell_coord(p.x, W.bx, W.cell, W.icell), cy = cell_coord(p.y, W.by, W.cell, W.icell);
  const uint32_t b = bucket_of(W, cx, cy);
  const uint32_t r = atomicAdd(&G.count[b], 1u);
  G.pbr[W.gp0 + j] = make_uint2(b, r);
}

// The slotted grid's whole build: each particle goes straight into its
// bucket (worlds whose link executor inserted them are skipped).  The cell
// words of this sub-step's parity are all zero here: the previous
// sub-step's collide pass cleared them.
static __global__ void __launch_bounds__(CHUNK) k_grid_insert(const DWorld* __restrict__ worlds,
                                                       DSlots G, const uint2* __restrict__ chunks,
                                                       uint32_t nchunks, uint32_t cur,
                                                       uint32_t sub) {
  pdl_trigger();
  const uint2 ch = chunks[blockIdx.x < nchunks ? blockIdx.x : 0u];
  const DWorld& W = worlds[ch.x];
  const uint32_t j = ch.y + threadIdx.x;
  const bool act = blockIdx.x < nchunks && j < W.np && sub < W.S &&
                   (W.flags & (COLLIDE_PP | GRID_IN_LINKS)) == COLLIDE_PP;
  const float2* P = W.pos[cur];
  pdl_wait();  // positions from the link phase
  if (!act) return;
  const float2 p = P[j];
  const int32_t cx = cell_coord(p.x, W.bx, W.cell, W.icell), cy = cell_coord(p.y, W.by, W.cell, W.icell);
  grid_insert(G, sub, bucket_of(W, cx, cy), p, cx, cy);
}

// block-wide exclusive scan of four values per thread at once (THREADS a
// multiple of 32, at most 1024); the four lanes scan independently.
// Returns the exclusive prefix of each lane and stores the four block
// totals in *total.
template <uint32_t THREADS>
__device__ __forceinline__ uint4 block_exclusive_scan4(uint4 v, uint4* total) {
  constexpr uint32_t NW = THREADS / 32;
  __shared__ uint4 warp_sum4[NW];
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  uint4 x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y0 = __shfl_up_sync(0xFFFFFFFFu, x.x, o), y1 = __shfl_up_sync(0xFFFFFFFFu, x.y, o),
                   y2 = __shfl_up_sync(0xFFFFFFFFu, x.z, o), y3 = __shfl_up_sync(0xFFFFFFFFu, x.w, o);
    if (lane >= (uint32_t)o) { x.x += y0; x.y += y1; x.z += y2; x.w += y3; }
  }
  if (lane == 31) warp_sum4[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint4 w = lane < NW ? warp_sum4[lane] : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (int o = 1; o < (int)NW; o <<= 1) {
      const uint32_t y0 = __shfl_up_sync(0xFFFFFFFFu, w.x, o), y1 = __shfl_up_sync(0xFFFFFFFFu, w.y, o),
                     y2 = __shfl_up_sync(0xFFFFFFFFu, w.z, o), y3 = __shfl_up_sync(0xFFFFFFFFu, w.w, o);
      if (lane >= (uint32_t)o) { w.x += y0; w.y += y1; w.z += y2; w.w += y3; }
    }
    if (lane < NW) warp_sum4[lane] = w;  // inclusive
  }
  __syncthreads();
  const uint4 before = wid ? warp_sum4[wid - 1] : make_uint4(0u, 0u, 0u, 0u);
  *total = warp_sum4[NW - 1];
  __syncthreads();
  return make_uint4(before.x + x.x - v.x, before.y + x.y - v.y, before.z + x.z - v.z,
                    before.w + x.w - v.w);
}

// Bucket ranges from the counts.  Each tile (SUBS sub-tiles of 4 x THREADS
// buckets: small grids favour many small tiles, large ones fewer)
// scans its counts and takes one block of `sorted`, of the tile's total size,
// from the sub-step's cursor with a single atomic.  Tiles do not wait on one
// another: a bucket's entries stay contiguous and the buckets of a tile stay
// in order (neighbouring cells' buckets are neighbours, which keeps the
// collide pass's loads together), but the tiles land in `sorted` in the order
// their atomics ran.  Nothing reads that order: the contact sums are exact
// integer sums, so the order of a bucket's entries does not matter either
// (it already follows the count pass's atomics).  The previous sub-step's
// collide kernel reset the cursor; a block that would end past `cap` (a
// cursor left over from a failed launch) is not handed out: its buckets get empty ranges and
// ERR_BIT_GRID_OVERFLOW is set.  The scan also zeroes the counts it read,
// leaving them ready for the next sub-step's count pass.  Within a tile,
// thread t holds buckets 4t .. 4t+3 of each sub-tile, so every load and
// store of a warp is contiguous.
template <uint32_t SUBS, uint32_t THREADS>
__global__ void __launch_bounds__(THREADS) k_grid_scan(DGrid G, uint32_t nbuckets, uint32_t ntiles) {
  constexpr uint32_t SUB = 4u * THREADS;
  __shared__ uint32_t s_base, s_ok;
  pdl_trigger();
  pdl_wait();  // counts from the count pass or the link executor
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    // bucket ranges are whole multiples of 64, so each group of four counts
    // is either all inside or all outside
    uint4 c[4];
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
      const uint32_t base = (tile * SUBS + k) * SUB + threadIdx.x * 4u;
      c[k] = make_uint4(0u, 0u, 0u, 0u);
      if (k < SUBS && base < nbuckets) {
        uint4* cp = reinterpret_cast<uint4*>(G.count + base);
        c[k] = *cp;
        *cp = make_uint4(0u, 0u, 0u, 0u);  // ready for the next count pass
      }
    }
    v.x = c[0].x + c[0].y + c[0].z + c[0].w;
    v.y = c[1].x + c[1].y + c[1].z + c[1].w;
    v.z = c[2].x + c[2].y + c[2].z + c[2].w;
    v.w = c[3].x + c[3].y + c[3].z + c[3].w;
    uint4 sub_tot;
    const uint4 excl = block_exclusive_scan4<THREADS>(v, &sub_tot);
    if (threadIdx.x == 0) {
      const uint32_t tot = sub_tot.x + sub_tot.y + sub_tot.z + sub_tot.w;
      const uint32_t at = tot ? atomicAdd(G.cursor, tot) : 0u;
      const bool ok = at <= G.cap && tot <= G.cap - at;
      if (!ok) atomicOr(G.err, ERR_BIT_GRID_OVERFLOW);
      s_base = at;
      s_ok = ok ? 1u : 0u;
    }
    __syncthreads();
    const uint32_t ok = s_ok;
    const uint32_t sub_off[4] = {0u, sub_tot.x, sub_tot.x + sub_tot.y,
                                 sub_tot.x + sub_tot.y + sub_tot.z};
    const uint32_t ex[4] = {excl.x, excl.y, excl.z, excl.w};
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
      const uint32_t base = (tile * SUBS + k) * SUB + threadIdx.x * 4u;
      if (k < SUBS && base < nbuckets) {
        uint32_t run = s_base + sub_off[k] + ex[k];
        const uint4 n = ok ? c[k] : make_uint4(0u, 0u, 0u, 0u);
        uint4* rp = reinterpret_cast<uint4*>(G.range + base);  // two {start, count} pairs each
        rp[0] = make_uint4(run, n.x, run + n.x, n.y);
        run += n.x + n.y;
        rp[1] = make_uint4(run, n.z, run + n.z, n.w);
      }
    }
    __syncthreads();  // s_base and s_ok are rewritten by the next tile
  }
}

static __global__ void __launch_bounds__(CHUNK) k_grid_scatter(const DWorld* __restrict__ worlds, DGrid G,
                                                        const uint2* __restrict__ chunks,
                                                        uint32_t nchunks, uint32_t cur,
                                                        uint32_t sub) {
  pdl_trigger();
  // chunk and world records are fixed during a step: read before the wait
  const uint2 ch = chunks[blockIdx.x < nchunks ? blockIdx.x : 0u];
  const DWorld& W = worlds[ch.x];
  const uint32_t j = ch.y + threadIdx.x;
  const bool act = blockIdx.x < nchunks && j < W.np && sub < W.S && (W.flags & COLLIDE_PP);
  const float2* P = W.pos[cur];
  pdl_wait();  // ranges from the scan
  if (!act) return;
  const float2 p = P[j];
  const uint2 br = G.pbr[W.gp0 + j];
  const uint2 rg = G.range[br.x];
  if (br.y >= rg.y) return;  // the bucket's block was not handed out (ERR_BIT_GRID_OVERFLOW)
  const int32_t cx = cell_coord(p.x, W.bx, W.cell, W.icell), cy = cell_coord(p.y, W.by, W.cell, W.icell);
  G.sorted[rg.x + br.y] =
      make_uint4(__float_as_uint(p.x), __float_as_uint(p.y), (uint32_t)cx, (uint32_t)cy);
}

// Contact corrections are summed in 64-bit fixed point (units of 2^-32,
// round to nearest even), which makes the sum independent of the order in
// which neighbours are found.
__device__ __forceinline__ long long fix32(float c) { return __float2ll_rn(fmul(c, 4294967296.0f)); }
// A contact sum converts back as float(double(s) * 2^-32).
// For |s| < 2^53 the double holds s exactly, so that is one rounding of
// s * 2^-32 to float, which equals rounding s to float and scaling by 2^-32
// (exact: every nonzero result is a normal float between 2^-32 and 2^21).
// That form needs no FP64 instruction; larger sums take the double path.
__device__ __forceinline__ float unfix32(long long s) {
  if (s > -(1LL << 53) && s < (1LL << 53)) return fmul(__ll2float_rn(s), 2.3283064365386962890625e-10f);
  return __double2float_rn(__dmul_rn(__ll2double_rn(s), 2.3283064365386962890625e-10));
}

// Contacts found by one lane's neighbour walk.  The IEEE square root and
// divisions of a contact (the costly part) are not run inside the walk, where
// a warp would pay for them on every step in which any of its lanes meets a
// contact, but after it: the first CONTACT_SLOTS contacts of a lane wait in
// registers and are solved together at the end (further ones are solved on
// the spot).  The sums are integers, so the order of the solves cannot
// change them.
constexpr uint32_t CONTACT_SLOTS = 2;
struct Contacts {
  float dx[CONTACT_SLOTS], dy[CONTACT_SLOTS], d2[CONTACT_SLOTS];
  uint32_t n;
  long long sx, sy;
  bool hit;
};
__device__ __forceinline__ void contact_solve(float dx, float dy, float d2, float D, Contacts& c) {
  const float dist = fsqrt(d2);
  const float nx = fdiv(dx, dist), ny = fdiv(dy, dist);
  const float ov = fsub(D, dist);
  c.sx += fix32(fmul(fmul(nx, ov), 0.5f));
  c.sy += fix32(fmul(fmul(ny, ov), 0.5f));
  c.hit = true;
}
__device__ __forceinline__ void pp_contact(float2 p, float2 pj, float D, float D2, Contacts& c) {
  const float dx = fsub(p.x, pj.x), dy = fsub(p.y, pj.y);
  const float d2 = fadd(fmul(dx, dx), fmul(dy, dy));
  if (d2 < D2 && d2 > 0.0f) {
    if (c.n < CONTACT_SLOTS) {
#pragma unroll
      for (uint32_t k = 0; k < CONTACT_SLOTS; ++k)
        if (k == c.n) { c.dx[k] = dx; c.dy[k] = dy; c.d2[k] = d2; }
      ++c.n;
    } else {
      contact_solve(dx, dy, d2, D, c);
    }
  }
}
__device__ __forceinline__ void contacts_finish(float D, Contacts& c) {
#pragma unroll
  for (uint32_t k = 0; k < CONTACT_SLOTS; ++k)
    if (k < c.n) contact_solve(c.dx[k], c.dy[k], c.d2[k], D, c);
}

// particle-Circle (circles are kinematic for particles; index order)
static __device__ float2 particle_circles(const DWorld& W, float2 p) {
  for (uint32_t k = 0; k < W.nc; ++k) {
    const float2 c = W.cpos[k];
    const float dx = fsub(p.x, c.x), dy = fsub(p.y, c.y);
    const float d2 = fadd(fmul(dx, dx), fmul(dy, dy));
    const float R = fadd(W.radius, W.crad[k]);
    if (d2 < fmul(R, R) && d2 > 0.0f) {
      const float dist = fsqrt(d2);
      const float nx = fdiv(dx, dist), ny = fdiv(dy, dist);
      const float m = fsub(R, dist);
      p.x = fadd(p.x, fmul(nx, m));
      p.y = fadd(p.y, fmul(ny, m));
    }
  }
  return p;
}

// particle-Polygon edge projection (one-way)
static __device__ float2 particle_polygon(const DWorld& W, uint32_t k, float2 p) {
  const DPoly P = W.polys[k];
  if (P.nv < 3) return p;
  const float4 bb = W.paabb[k];
  const float r = W.radius;
  if (!(p.x >= fsub(bb.x, r) && p.x <= fadd(bb.z, r) && p.y >= fsub(bb.y, r) &&
        p.y <= fadd(bb.w, r)))
    return p;
  const float2* v = W.vpos + P.v0;
  bool inside = false;
  float best = __int_as_float(0x7f800000);
  float2 bq = p;
  for (uint32_t e = 0; e < P.nv; ++e) {
    const float2 a = v[e];
    const float2 b = v[e + 1 == P.nv ? 0 : e + 1];
    if ((a.y > p.y) != (b.y > p.y)) {
      const float t = fdiv(fsub(p.y, a.y), fsub(b.y, a.y));
      const float xint = fadd(a.x, fmul(t, fsub(b.x, a.x)));
      if (p.x < xint) inside = !inside;
    }
    const float abx = fsub(b.x, a.x), aby = fsub(b.y, a.y);
    const float l2 = fadd(fmul(abx, abx), fmul(aby, aby));
    float t = 0.0f;
    if (l2 > 0.0f) t = fdiv(fadd(fmul(fsub(p.x, a.x), abx), fmul(fsub(p.y, a.y), aby)), l2);
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    const float qx = fadd(a.x, fmul(abx, t)), qy = fadd(a.y, fmul(aby, t));
    const float dqx = fsub(p.x, qx), dqy = fsub(p.y, qy);
    const float d2 = fadd(fmul(dqx, dqx), fmul(dqy, dqy));
    if (d2 < best) { best = d2; bq = make_float2(qx, qy); }
  }
  if (inside) {
    const float dist = fsqrt(best);
    if (dist > 0.0f) {
      const float nx = fdiv(fsub(bq.x, p.x), dist), ny = fdiv(fsub(bq.y, p.y), dist);
      return make_float2(fadd(bq.x, fmul(nx, r)), fadd(bq.y, fmul(ny, r)));
    }
    return bq;
  }
  if (best < fmul(r, r)) {
    const float dist = fsqrt(best);
    if (dist > 0.0f) {
      const float nx = fdiv(fsub(p.x, bq.x), dist), ny = fdiv(fsub(p.y, bq.y), dist);
      return make_float2(fadd(bq.x, fmul(nx, r)), fadd(bq.y, fmul(ny, r)));
    }
  }
  return p;
}

// Contacts of a particle at p with the particles of cell (ncx, ncy), whose
// entries sit in the bucket range [s0, s0 + cnt) among those of other cells
// that share the bucket.  The particle's own entry needs no test: it has
// d2 = 0, which pp_contact never counts as a contact.
__device__ __forceinline__ void visit_cell(const DGrid& G, float2 p, int32_t ncx, int32_t ncy,
                                           uint32_t s0, uint32_t cnt, float D, float D2,
                                           Contacts& c) {
  for (uint32_t k = s0; k < s0 + cnt; ++k) {
    const uint4 e = G.sorted[k];
    if (e.z != (uint32_t)ncx || e.w != (uint32_t)ncy) continue;
    pp_contact(p, make_float2(__uint_as_float(e.x), __uint_as_float(e.y)), D, D2, c);
  }
}

// The collide kernels over either grid form.  grid_head: what a bucket's
// walk starts from (its range in `sorted`, or its cell word); grid_visit:
// the walk of bucket b for cell (ncx, ncy).
__device__ __forceinline__ uint2 grid_head(const DGrid& G, uint32_t, uint32_t b) {
  return G.range[b];
}
__device__ __forceinline__ uint2 grid_head(const DSlots& G, uint32_t sub, uint32_t b) {
  return G.cell[(size_t)(sub & 1u) * G.nbuckets + b];
}
__device__ __forceinline__ void grid_visit(const DGrid& G, float2 p, int32_t ncx, int32_t ncy,
                                           uint32_t, uint2 h, float D, float D2, Contacts& c) {
  visit_cell(G, p, ncx, ncy, h.x, h.y, D, D2, c);
}
// Slots first, then the overflow chain (at most cap links: the chain is
// built acyclic, the bound only keeps a walk finite whatever the words say).
__device__ __forceinline__ void grid_visit(const DSlots& G, float2 p, int32_t ncx, int32_t ncy,
                                           uint32_t b, uint2 h, float D, float D2, Contacts& c) {
  const uint32_t n = h.x < GRID_SLOTS ? h.x : GRID_SLOTS;
  for (uint32_t k = 0; k < n; ++k) {
    const uint4 e = G.slot[slot_index(b, k)];
    if (e.z != (uint32_t)ncx || e.w != (uint32_t)ncy) continue;
    pp_contact(p, make_float2(__uint_as_float(e.x), __uint_as_float(e.y)), D, D2, c);
  }
  uint32_t o = h.y;
  for (uint32_t it = 0; o != 0u && o <= G.cap && it < G.cap; ++it) {
    const uint4 e = G.ovf[o - 1u];
    o = G.ovf_next[o - 1u];
    if (e.z != (uint32_t)ncx || e.w != (uint32_t)ncy) continue;
    pp_contact(p, make_float2(__uint_as_float(e.x), __uint_as_float(e.y)), D, D2, c);
  }
}
// Called by every thread of a collide launch once this sub-step's build is
// complete.  Sorted grid: the scan is done with the cursor; clear it for the
// next sub-step's scan.  Slotted grid: reset the overflow cursor and clear
// the other parity's cell words for the next sub-step's inserts.  Engines
// without particle collisions have no grid (null pointers) but still run the
// collide kernels.
__device__ __forceinline__ void grid_done(const DGrid& G, uint32_t) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && G.cursor != nullptr) *G.cursor = 0u;
}
__device__ __forceinline__ void clear_cells(uint2* cells, uint32_t n) {  // n even
  uint4* c = reinterpret_cast<uint4*>(cells);
  const uint32_t nt = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n / 2u; i += nt)
    c[i] = make_uint4(0u, 0u, 0u, 0u);
}
__device__ __forceinline__ void grid_done(const DSlots& G, uint32_t sub) {
  if (G.cell == nullptr) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) *G.cursor = 0u;
  clear_cells(G.cell + (size_t)((sub & 1u) ^ 1u) * G.nbuckets, G.nbuckets);
}

// True when the interval [lo, hi] cannot reach [cmin, cmax] even allowing
// for float rounding in the exact per-particle test (a relative margin of
// 1e-5 is far above the few-ulp error of the subtractions and squares there).
__device__ __forceinline__ bool separated(float lo, float hi, float cmin, float cmax) {
  const float d = 1e-5f * (fabsf(lo) + fabsf(hi) + 1.0f);
  return cmax < lo - d || cmin > hi + d;
}

// min/max of the warp's particle positions (NaN ignored); all 32 lanes call
__device__ __forceinline__ float4 warp_box(bool act, float2 p) {
  float4 b = act ? make_float4(p.x, p.y, p.x, p.y)
                 : make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    b.x = fminf(b.x, __shfl_xor_sync(0xFFFFFFFFu, b.x, o));
    b.y = fminf(b.y, __shfl_xor_sync(0xFFFFFFFFu, b.y, o));
    b.z = fmaxf(b.z, __shfl_xor_sync(0xFFFFFFFFu, b.z, o));
    b.w = fmaxf(b.w, __shfl_xor_sync(0xFFFFFFFFu, b.w, o));
  }
  return b;
}

// Particle collisions + bounds + integrate of one sub-step of the extension
// pipeline.  Reads positions from buffer cur (the post-link snapshot) and
// writes the new ones to buffer cur^1; prev is updated in place.
//
// Three lanes per particle, ten particles per warp (lanes 30 and 31 idle):
// each lane scans one row of the 3x3 neighbour cells and the owner (the
// first lane of the three) adds their fixed-point sums (integer adds, so the
// split cannot change the result), then runs the circle and polygon tests,
// bounds and integrate.  A CTA of 8 warps covers 80 particles, a quarter of
// one work chunk (grid = 4 x chunks).  Circle and polygon tests are skipped
// for a whole warp when no circle or polygon box reaches the warp's
// particles: then no particle is in contact, nothing moves, and so no later
// test of the sequence can hit either — the skip is exact.
constexpr uint32_t COLLIDE_THREADS = 256;      // 8 warps
constexpr uint32_t COLLIDE_PER_WARP = 10;      // particles per warp, three lanes each
constexpr uint32_t COLLIDE_CTAS = CHUNK / (COLLIDE_THREADS / 32 * COLLIDE_PER_WARP);  // per chunk
static_assert(COLLIDE_CTAS * (COLLIDE_THREADS / 32) * COLLIDE_PER_WARP == CHUNK, "chunk split");
template <class GRID>
__global__ void __launch_bounds__(COLLIDE_THREADS, 5) k_collide_integrate(
    const DWorld* __restrict__ worlds, GRID G, const uint2* __restrict__ chunks,
    uint32_t nchunks, uint32_t cur, uint32_t sub) {
  pdl_trigger();
  // chunk and world records are fixed during a step: read before the wait
  const uint32_t cidx = blockIdx.x / COLLIDE_CTAS;
  const uint2 ch = chunks[cidx < nchunks ? cidx : 0u];
  const DWorld& W = worlds[ch.x];
  pdl_wait();  // the grid's entries (and everything before them)
  grid_done(G, sub);
  if (cidx >= nchunks || sub >= W.S) return;  // uniform over the CTA
  const uint32_t wl = threadIdx.x & 31u, grp = wl / 3u, row = wl - 3u * grp;
  const uint32_t i = ch.y + (blockIdx.x % COLLIDE_CTAS) * (COLLIDE_THREADS / 32 * COLLIDE_PER_WARP) +
                     (threadIdx.x >> 5) * COLLIDE_PER_WARP + grp;
  const bool act = grp < COLLIDE_PER_WARP && i < W.np;
  const bool own = act && row == 0;  // the lane that owns particle i
  const float2* P = W.pos[cur];
  float2 p = act ? P[i] : make_float2(0.f, 0.f);
  float2 q = own ? W.prev[i] : make_float2(0.f, 0.f);  // issued early, used last
  if (W.flags & COLLIDE_PP) {  // uniform over the CTA
    Contacts c;
    c.n = 0;
    c.sx = 0;
    c.sy = 0;
    c.hit = false;
    if (act) {
      const int32_t cx = cell_coord(p.x, W.bx, W.cell, W.icell);
      const int32_t cy = cell_coord(p.y, W.by, W.cell, W.icell) + (int32_t)row - 1;  // this lane's row
      const float D = fadd(W.radius, W.radius);
      const float D2 = fmul(D, D);
      // bucket_of for cells cx - 1, cx, cx + 1 with two hashes: the strip of
      // cx and the neighbouring strip that cx - 1 (first cell of its strip)
      // or cx + 1 (last cell) falls in
      const int32_t st = cx >> 2;
      const uint32_t k = (uint32_t)cx & 3u;
      const uint32_t hm = (cell_hash(st, cy) << 2) & W.gmask;
      const uint32_t ho = (cell_hash(k == 0u ? st - 1 : st + 1, cy) << 2) & W.gmask;
      const uint32_t b0 = W.gb0 + (k == 0u ? (ho | 3u) : (hm | (k - 1u)));
      const uint32_t b1 = W.gb0 + (hm | k);
      const uint32_t b2 = W.gb0 + (k == 3u ? ho : (hm | (k + 1u)));
      const uint2 r0 = grid_head(G, sub, b0), r1 = grid_head(G, sub, b1), r2 = grid_head(G, sub, b2);
      grid_visit(G, p, cx - 1, cy, b0, r0, D, D2, c);
      grid_visit(G, p, cx, cy, b1, r1, D, D2, c);
      grid_visit(G, p, cx + 1, cy, b2, r2, D, D2, c);
      contacts_finish(D, c);
    }
    long long sx = c.sx, sy = c.sy;
    bool hit = c.hit;
    // the owner adds the other two rows' sums (lanes 30, 31 read lanes 31, 0:
    // harmless, they own nothing)
    const uint32_t l1 = (wl + 1u) & 31u, l2 = (wl + 2u) & 31u;
    const long long sx1 = __shfl_sync(0xFFFFFFFFu, sx, l1), sx2 = __shfl_sync(0xFFFFFFFFu, sx, l2);
    const long long sy1 = __shfl_sync(0xFFFFFFFFu, sy, l1), sy2 = __shfl_sync(0xFFFFFFFFu, sy, l2);
    const int h1 = __shfl_sync(0xFFFFFFFFu, (int)hit, l1), h2 = __shfl_sync(0xFFFFFFFFu, (int)hit, l2);
    if (own) {
      sx += sx1 + sx2;
      sy += sy1 + sy2;
      hit = hit || h1 || h2;
      if (hit) { p.x = fadd(p.x, unfix32(sx)); p.y = fadd(p.y, unfix32(sy)); }
    }
  }
  const uint32_t flags = W.flags;
  if (flags & (COLLIDE_PC | COLLIDE_PPOLY)) {
    const float4 box = warp_box(own, p);
    bool near = false;
    if (flags & COLLIDE_PC) {
      for (uint32_t k = wl; k < W.nc; k += 32u) {
        const float2 c = W.cpos[k];
        const float R = W.radius + W.crad[k];
        near |= !(separated(c.x - R, c.x + R, box.x, box.z) ||
                  separated(c.y - R, c.y + R, box.y, box.w));
      }
    }
    if (flags & COLLIDE_PPOLY) {
      for (uint32_t k = wl; k < W.ng; k += 32u) {
        const float4 bb = W.paabb[k];
        const float r = W.radius;
        near |= !(separated(bb.x - r, bb.z + r, box.x, box.z) ||
                  separated(bb.y - r, bb.w + r, box.y, box.w));
      }
    }
    if (__any_sync(0xFFFFFFFFu, near) && own) {
      if (flags & COLLIDE_PC) p = particle_circles(W, p);
      if (flags & COLLIDE_PPOLY) {
        for (uint32_t k = 0; k < W.ng; ++k) p = particle_polygon(W, k, p);
      }
    }
  }
  if (!own) return;
  solve_bounds(p, q, W);
  integrate(p, q, W.gx, W.gy, W.h);
  W.pos[cur ^ 1u][i] = p;
  W.prev[i] = q;
}

// The same sub-step with one thread per particle, which walks all nine
// neighbour cells itself (the nine bucket ranges loaded first, together):
// about half the instructions per particle of the three-lane form, for
// launches with many waves of particles, where the collide pass is bound by
// instruction issue (configuration 5: 2.68 -> 1.98 ms per update); with few
// waves the three-lane form's shorter chains win (configuration 2: 0.17
// against 0.24 ms).  Same contacts and the same fixed-point sums, so the
// same bits.  One CTA per work chunk.
constexpr uint32_t COLLIDE_P_THREADS = CHUNK;
template <class GRID>
__global__ void __launch_bounds__(COLLIDE_P_THREADS, 3) k_collide_particle(
    const DWorld* __restrict__ worlds, GRID G, const uint2* __restrict__ chunks,
    uint32_t nchunks, uint32_t cur, uint32_t sub) {
  pdl_trigger();
  // chunk and world records are fixed during a step: read before the wait
  const uint32_t cidx = blockIdx.x;
  const uint2 ch = chunks[cidx < nchunks ? cidx : 0u];
  const DWorld& W = worlds[ch.x];
  pdl_wait();  // the grid's entries (and everything before them)
  grid_done(G, sub);
  if (cidx >= nchunks || sub >= W.S) return;  // uniform over the CTA
  const uint32_t wl = threadIdx.x & 31u;
  const uint32_t i = ch.y + threadIdx.x;
  const bool own = i < W.np;
  const float2* P = W.pos[cur];
  float2 p = own ? P[i] : make_float2(0.f, 0.f);
  float2 q = own ? W.prev[i] : make_float2(0.f, 0.f);  // issued early, used last
  if (W.flags & COLLIDE_PP) {  // uniform over the CTA
    Contacts c;
    c.n = 0;
    c.sx = 0;
    c.sy = 0;
    c.hit = false;
    if (own) {
      const int32_t cx = cell_coord(p.x, W.bx, W.cell, W.icell);
      const int32_t cy0 = cell_coord(p.y, W.by, W.cell, W.icell);
      const float D = fadd(W.radius, W.radius);
      const float D2 = fmul(D, D);
      // buckets of cells cx - 1 .. cx + 1 in each row, as k_collide_integrate
      const int32_t st = cx >> 2;
      const uint32_t k = (uint32_t)cx & 3u;
      uint32_t bk[9];
      uint2 r[9];
#pragma unroll
      for (int row = 0; row < 3; ++row) {
        const int32_t cy = cy0 + row - 1;
        const uint32_t hm = (cell_hash(st, cy) << 2) & W.gmask;
        const uint32_t ho = (cell_hash(k == 0u ? st - 1 : st + 1, cy) << 2) & W.gmask;
        bk[3 * row] = W.gb0 + (k == 0u ? (ho | 3u) : (hm | (k - 1u)));
        bk[3 * row + 1] = W.gb0 + (hm | k);
        bk[3 * row + 2] = W.gb0 + (k == 3u ? ho : (hm | (k + 1u)));
      }
#pragma unroll
      for (int j = 0; j < 9; ++j) r[j] = grid_head(G, sub, bk[j]);
#pragma unroll
      for (int row = 0; row < 3; ++row)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          grid_visit(G, p, cx + j - 1, cy0 + row - 1, bk[3 * row + j], r[3 * row + j], D, D2, c);
      contacts_finish(D, c);
      if (c.hit) {
        p.x = fadd(p.x, unfix32(c.sx));
        p.y = fadd(p.y, unfix32(c.sy));
      }
    }
  }
  const uint32_t flags = W.flags;
  if (flags & (COLLIDE_PC | COLLIDE_PPOLY)) {  // per-warp filter, as k_collide_integrate
    const float4 box = warp_box(own, p);
    bool near = false;
    if (flags & COLLIDE_PC) {
      for (uint32_t k = wl; k < W.nc; k += 32u) {
        const float2 cc = W.cpos[k];
        const float R = W.radius + W.crad[k];
        near |= !(separated(cc.x - R, cc.x + R, box.x, box.z) ||
                  separated(cc.y - R, cc.y + R, box.y, box.w));
      }
    }
    if (flags & COLLIDE_PPOLY) {
      for (uint32_t k = wl; k < W.ng; k += 32u) {
        const float4 bb = W.paabb[k];
        const float r = W.radius;
        near |= !(separated(bb.x - r, bb.z + r, box.x, box.z) ||
                  separated(bb.y - r, bb.w + r, box.y, box.w));
      }
    }
    if (__any_sync(0xFFFFFFFFu, near) && own) {
      if (flags & COLLIDE_PC) p = particle_circles(W, p);
      if (flags & COLLIDE_PPOLY) {
        for (uint32_t k = 0; k < W.ng; ++k) p = particle_polygon(W, k, p);
      }
    }
  }
  if (!own) return;
  solve_bounds(p, q, W);
  integrate(p, q, W.gx, W.gy, W.h);
  W.pos[cur ^ 1u][i] = p;
  W.prev[i] = q;
}

// positions of worlds whose step ended in buffer 1 go back to buffer 0.
// With an odd number of sub-steps the last collide pass (parity 0) cleared
// parity 1's cell words of the slotted grid; parity 0's, which the first
// sub-step of the next update uses, are cleared here (cells = null: nothing
// to clear).
static __global__ void __launch_bounds__(CHUNK) k_copy_back(const DWorld* __restrict__ worlds,
                                                     const uint2* __restrict__ chunks,
                                                     uint32_t nchunks, uint2* cells,
                                                     uint32_t ncells) {
  if (cells != nullptr) clear_cells(cells, ncells);
  if (blockIdx.x >= nchunks) return;
  const uint2 ch = chunks[blockIdx.x];
  const DWorld& W = worlds[ch.x];
  const uint32_t i = ch.y + threadIdx.x;
  if (i >= W.np || !(W.S & 1u)) return;
  W.pos[0][i] = W.pos[1][i];
}

}  // namespace b2d

// b2d_dev.h — records shared by the host planner and the CUDA kernels.
//
// Device layout: every world (one Solver) is a self-contained block of device
// memory holding all of its arrays; a DWorld record (in a device table) holds
// the world's parameters and pointers into its block.  Work lists name
// (world, item) pairs, so a batch or a serving pool is just a table of worlds.
// Solver particles stay in insertion order, exactly like the reference's
// Vec<Particle> (src/solver.rs:24).
#pragma once
#include <cstdint>

// CUDA's vector types (plain C structs, usable by the host compiler too)
#include <vector_functions.h>
#include <vector_types.h>

#include <cstring>

namespace b2d {

// Collision extension flags (not in the reference; see solve_dynamic_collisions).
enum : uint32_t { COLLIDE_PP = 1u, COLLIDE_PC = 2u, COLLIDE_PPOLY = 4u };
// World flag set by the planner: every solver particle of this world belongs
// to a body that the shared-memory link executor runs, so that executor
// enters each particle into the collision grid (a slot insert, or the
// sorted grid's count) as it stores the body back: no separate insert or
// count kernel for this world.
constexpr uint32_t GRID_IN_LINKS = 8u;

// Schedule op encoding: link ops carry the body-local link index; bounds +
// integrate ops carry the body-local particle index with this bit set.
constexpr uint32_t OP_INTEG = 0x80000000u;
constexpr uint32_t OP_WIDE = 0xFFFFFFFFu;
// Whole-update schedules only: a padding entry {0, OP_NOP} that does
// nothing.  Within a level the link solves come first, padded to a whole
// number of warps, then the bounds+integrate ops, so that no warp runs both
// code paths (the ops of a level are independent, so their order within the
// level cannot change any result).
constexpr uint32_t OP_NOP = 0xFFFFFFFEu;

// A body is a set of solver particles run by one executor unit: a union of
// whole link-connected components, so no link crosses two bodies.
struct DBody {
  uint32_t i0, np;       // particle list bidx[i0 .. i0+np) (world indices, ascending)
  uint32_t l0, nl;       // links lab[l0 .. l0+nl) in insertion order
  uint32_t sched;        // schedule id (group executors), else unused
  uint32_t local;        // 1: link endpoints are body-local; 0: world indices
  uint32_t first;        // bidx[i0 + i] == first + i for every i, else NO_FIRST
  uint32_t pad;
};
constexpr uint32_t NO_FIRST = 0xFFFFFFFFu;

struct DPoly {
  uint32_t v0, nv;       // vertices
  uint32_t l0, nl;       // polygon links (polygon-local indices)
  uint32_t is_static, pad;
};

// A level schedule is stored as a stream of self-describing chunks of at most
// SCHED_CHUNK_WORDS 32-bit words, each 16-byte aligned so that one bulk copy
// (TMA, cp.async.bulk) moves it into shared memory:
//   word 0            nseg
//   words 1..nseg     end of each segment, counted in ops
//   (pad to an even word)
//   then two words per op:
//     link op    {a | b << 16, link index}   (body-local endpoints; bodies
//                                             of up to 65535 particles)
//                {link index, OP_WIDE}       (larger bodies)
//     integrate  {particle, OP_INTEG}
//     padding    {0, OP_NOP}                 (whole-update schedules)
// A segment is a whole level or a piece of one; a group barrier follows
// every segment.
constexpr uint32_t SCHED_CHUNK_WORDS = 4096;
// shared bytes after each executor group's schedule area: two mbarriers and
// two flag words
constexpr uint32_t GROUP_TAIL_BYTES = 32;
struct DSched {
  uint32_t chunk0, nchunks;  // chunk_off / chunk_len entries
  uint32_t nlvl, nops;
  uint32_t off, words;       // the chunks are contiguous: stream[off, off + words)
  uint32_t len0;             // words of the first chunk
  uint32_t maxw;             // most ops in one segment
  uint32_t nop_pad;          // 1: the schedule holds OP_NOP padding entries
};

// 1 / c when c is a positive normal power of two (then x / c == x * (1/c)
// exactly for every x: both round the same real number), else 0.
inline float pow2_reciprocal(float c) {
  uint32_t u;
  std::memcpy(&u, &c, 4);
  const uint32_t e = (u >> 23) & 0xFFu;
  if ((u >> 31) || (u & 0x7FFFFFu) || e == 0u || e == 255u) return 0.0f;
  const int ne = 254 - (int)e;  // 2^(127 - (e - 127)) has exponent field 254 - e
  if (ne < 1 || ne > 254) return 0.0f;
  const uint32_t r = (uint32_t)ne << 23;
  float f;
  std::memcpy(&f, &r, 4);
  return f;
}

struct DWorld {
  // parameters
  float gx, gy;          // 0 + gravity: the acceleration at integrate time
  float bx, by, bw, bh;  // Bounds pos / size (src/solver.rs:13-17)
  float h;               // dt * (1 / sub_steps) (src/solver.rs:107-108)
  float radius, cell;    // extension: particle radius, grid cell
  uint32_t S, I;         // sub_steps, link iterations
  uint32_t flags;        // COLLIDE_* bits
  uint32_t slot;         // stable id (hash salt for the shared grid)
  uint32_t np, nb, nc, ncl, ng;
  uint32_t gb0, gmask;   // extension grid: this world's buckets [gb0, gb0 + gmask]
  uint32_t gp0;          // extension grid: this world's particle scratch offset
  float icell;           // 1 / cell when cell is a power of two (exact), else 0
  // solver particles
  float2* pos[2];        // ping-pong positions; pos[0] holds the state between steps
  float2* prev;
  // bodies and links
  DBody* bodies;
  uint32_t* bidx;
  uint2* lab;
  float* lrest;
  float* lstiff;
  // circles (src/circle.rs:4-8) and circle links
  float2* cpos; float2* cprev; float2* cacc;
  float* crad; uint32_t* cstatic;
  uint2* clab; float* clrest;
  // polygons (src/polygon.rs:7-14)
  DPoly* polys;
  float2* vpos; float2* vprev; float2* vacc;
  float2* pcenter;
  float4* paabb;
  uint2* plab; float* plrest;
  uint32_t* stage_off;   // polygon-pair test offsets, see rigid_phase_a
  uint32_t* stage_pr;    // polygon pair of each stage: self | other << 16
};

// Shared (engine-wide) read-only schedule registry, plus the device error
// word that bounded waits set instead of trapping.
struct DScheds {
  const DSched* scheds;
  const uint32_t* chunk_off;  // word offset of each chunk in `stream`
  const uint32_t* chunk_len;  // words (multiple of 4)
  const uint32_t* stream;
  uint32_t* err;
  uint32_t fault;  // FAULT_BIT_* test switches (0 in normal operation)
};
enum : uint32_t { ERR_BIT_TMA_TIMEOUT = 1u, ERR_BIT_GRID_OVERFLOW = 2u };
// Test switch for failure detection: every executor group treats its first
// bulk-copy wait as timed out (and takes the timeout path: error word, wait
// for the copy in flight to land, leave) without a real timeout.
enum : uint32_t { FAULT_BIT_WAIT = 1u };

// Extension broadphase: hashed uniform grid, sorted form (large grids and
// the allocation-free entry point): built by a counting sort each sub-step.
// Every world with particle collisions owns a power-of-two range of
// buckets; a bucket's entries are contiguous in `sorted`.
// bucket scan tiles: 1,024 buckets (256 threads x 4 each) for grids of up to
// SCAN_SMALL_MAX buckets, else 16,384 (four sub-tiles of 1024 threads x 4)
constexpr uint32_t SCAN_SMALL_TILE = 1024;
constexpr uint32_t SCAN_LARGE_TILE = 16384;
constexpr uint32_t SCAN_SMALL_MAX = 1u << 20;
struct DGrid {
  uint32_t* count;       // nbuckets: entries per bucket (all zero between sub-steps)
  uint2* range;          // nbuckets: {first entry in sorted, count}
  uint32_t* cursor;      // entries of sorted handed out so far this sub-step
  uint2* pbr;            // per particle: (bucket, rank within bucket)
  uint4* sorted;         // cap entries: {pos.x bits, pos.y bits, cell x, cell y}
  uint32_t* err;         // device error word (ERR_BIT_*)
  uint32_t nbuckets;
  uint32_t cap;
};

// The engine's form of the same grid: no sort.  Each particle is inserted
// straight into its bucket, whose first GRID_SLOTS entries sit in fixed
// slots; later ones go to an overflow array, chained per bucket.  A
// sub-step's inserts use the cell words of parity sub & 1; that sub-step's
// collide pass clears the other parity's words for the next sub-step (and
// resets the overflow cursor).  Slots are interleaved by strip (four
// buckets): slot k of the strip's four buckets is one 64-byte run, so the
// first entries of a row of neighbour cells share a cache line.
constexpr uint32_t GRID_SLOTS = 4;
struct DSlots {
  uint2* cell;           // 2 x nbuckets (parity-major): {entries, overflow head + 1 (0: none)}
  uint4* slot;           // nbuckets x GRID_SLOTS entries {pos.x bits, pos.y bits, cell x, cell y}
  uint4* ovf;            // cap overflow entries
  uint32_t* ovf_next;    // cap: the bucket's next overflow entry + 1 (0: end)
  uint32_t* cursor;      // overflow entries handed out this sub-step
  uint32_t* err;         // device error word (ERR_BIT_*)
  uint32_t nbuckets;
  uint32_t cap;
};

}  // namespace b2d

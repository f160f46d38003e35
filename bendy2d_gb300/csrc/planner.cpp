// planner.cpp — turns one world (the reference's Solver contents) into its
// device image: bodies, executor choice, level schedules and the world block.
//
// Level scheduling.  The reference applies links one at a time in insertion
// order (src/solver.rs:143-146), then bounds and integration per particle
// (src/solver.rs:155-158, :118-121).  Give each op the level
//   level(op) = 1 + max(level of the last earlier op touching any of its particles)
// Ops on one level touch disjoint particles, and every particle sees its ops
// in the original order, so executing level by level reproduces the
// sequential loop exactly.  A FULL schedule chains all sub-steps and link
// iterations of one Solver::update, which lets independent regions of a body
// run ahead into later passes (the critical path of a 32x32 cloth step drops
// from 4032 to ~413 levels).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>

#include "engine.hpp"

namespace b2d {

static uint32_t pow2ceil(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}
static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

bool PlanTuning::set(const std::string& k, double v) {
  if (k == "serial_width") serial_width = (float)v;
  else if (k == "t_min") t_min = (uint32_t)v;
  else if (k == "t_max") t_max = (uint32_t)v;
  else if (k == "pack_np") pack_np = (uint32_t)v;
  else if (k == "pack_nl") pack_nl = (uint32_t)v;
  else if (k == "free_chunk") free_chunk = (uint32_t)v;
  else if (k == "smem_max") smem_max = (uint32_t)v;
  else if (k == "warp_groups") warp_groups = (uint32_t)v;
  else if (k == "max_groups") max_groups = (uint32_t)v;
  else if (k == "width_per_thread") width_per_thread = (float)v;
  else if (k == "resident") resident = (uint32_t)v;
  else if (k == "res_max") res_max = (uint32_t)v;
  else if (k == "stage_frac") stage_frac = (float)v;
  else if (k == "bucket_factor") bucket_factor = (float)v;
  else if (k == "collide_thread_min") collide_thread_min = (uint32_t)v;
  else if (k == "large_max") large_max = (uint32_t)v;
  else if (k == "grid_slot_max") grid_slot_max = (uint32_t)std::min(v, 4294967295.0);
  else return false;
  return true;
}

uint32_t SchedRegistry::get(const uint2* links, uint32_t nl, uint32_t np, uint32_t S, uint32_t I,
                            bool full, bool wide) {
  std::string key;
  key.resize(20 + (size_t)nl * 8);
  const uint32_t hdr[5] = {np, nl, S, I, (full ? 1u : 0u) | (full && wide ? 2u : 0u)};
  std::memcpy(&key[0], hdr, 20);
  if (nl) std::memcpy(&key[20], links, (size_t)nl * 8);
  auto it = index.find(key);
  if (it != index.end()) return it->second;

  const uint32_t nsub = full ? S : 1u;
  const size_t total = (size_t)nsub * ((size_t)I * nl + (full ? np : 0));
  std::vector<uint32_t> last(np, 0), lvl_of, op_of;
  lvl_of.reserve(total);
  op_of.reserve(total);
  uint32_t maxl = 0;
  for (uint32_t s = 0; s < nsub; ++s) {
    for (uint32_t it2 = 0; it2 < I; ++it2) {
      for (uint32_t k = 0; k < nl; ++k) {
        const uint32_t a = links[k].x, b = links[k].y;
        const uint32_t l = std::max(last[a], last[b]) + 1;
        last[a] = l;
        last[b] = l;
        lvl_of.push_back(l);
        op_of.push_back(k);
        maxl = std::max(maxl, l);
      }
    }
    if (full) {
      for (uint32_t p = 0; p < np; ++p) {
        const uint32_t l = last[p] + 1;
        last[p] = l;
        lvl_of.push_back(l);
        op_of.push_back(OP_INTEG | p);
        maxl = std::max(maxl, l);
      }
    }
  }
  // stable counting sort by level
  std::vector<uint32_t> start(maxl + 2, 0);
  for (uint32_t l : lvl_of) start[l + 1]++;
  for (uint32_t l = 1; l <= maxl + 1; ++l) start[l] += start[l - 1];
  std::vector<uint32_t> sorted(total);
  {
    std::vector<uint32_t> fill(start.begin(), start.end());
    for (size_t i = 0; i < total; ++i) sorted[fill[lvl_of[i]]++] = op_of[i];
  }
  // Whole-update schedules whose levels fit one op per thread of a group of
  // up to 512: within each level the link solves first, then the
  // bounds+integrate ops, the links padded with OP_NOP entries to a whole
  // number of warps (a level's ops are independent, so this order gives the
  // same results).  A warp then runs one kind only (configuration 1 in
  // reference order: 378 of 413 levels had a warp running both).  Padding
  // stays within the power of two above the widest level, so a group that
  // ran every level with one op per thread still does.  Wider schedules
  // (fast order: levels of up to ~930 ops, several per thread, and hardly
  // any mixed warps) keep their order.
  constexpr uint32_t NOP_ID = 0xFFFFFFFFu;
  bool padded = false;
  uint32_t maxw0 = 0;
  for (uint32_t l = 1; l <= maxl; ++l) maxw0 = std::max(maxw0, start[l + 1] - start[l]);
  uint32_t cap = 1;
  while (cap < maxw0) cap <<= 1;
  if (full && (cap <= 512u || wide)) {
    std::vector<uint32_t> out, nstart(maxl + 2, 0);
    out.reserve(total + 32 * (size_t)maxl);
    for (uint32_t l = 1; l <= maxl; ++l) {
      nstart[l] = (uint32_t)out.size();
      const uint32_t b = start[l], e = start[l + 1];
      uint32_t nlink = 0;
      for (uint32_t i = b; i < e; ++i)
        if (!(sorted[i] & OP_INTEG)) {
          out.push_back(sorted[i]);
          ++nlink;
        }
      const uint32_t ninteg = (e - b) - nlink;
      const uint32_t pad = (32u - nlink % 32u) % 32u;
      if (nlink && ninteg && pad && (wide || nlink + pad + ninteg <= cap)) {
        out.insert(out.end(), pad, NOP_ID);
        padded = true;
      }
      for (uint32_t i = b; i < e; ++i)
        if (sorted[i] & OP_INTEG) out.push_back(sorted[i]);
    }
    nstart[maxl + 1] = (uint32_t)out.size();
    sorted.swap(out);
    start.swap(nstart);
  }
  for (uint32_t op : sorted) {  // self-check: ops name the body's links/particles
    if (op == NOP_ID) continue;
    if ((op & OP_INTEG) ? (op & ~OP_INTEG) >= np : op >= nl) std::abort();
  }
  // cut the level sequence into chunks (a level may span chunks)
  DSched d;
  d.chunk0 = (uint32_t)chunk_off.size();
  d.nlvl = maxl;
  d.nops = (uint32_t)total;
  const bool narrow = np <= 65535u;
  std::vector<uint32_t> seg_end, chunk_ops;  // chunk_ops: op ids
  auto flush = [&]() {
    if (seg_end.empty()) return;
    while (stream.size() % 4) stream.push_back(0);
    chunk_off.push_back((uint32_t)stream.size());
    const size_t at = stream.size();
    stream.push_back((uint32_t)seg_end.size());
    stream.insert(stream.end(), seg_end.begin(), seg_end.end());
    if ((stream.size() - at) % 2) stream.push_back(0);
    for (uint32_t op : chunk_ops) {
      if (op == NOP_ID) {
        stream.push_back(0);
        stream.push_back(OP_NOP);
      } else if (op & OP_INTEG) {
        stream.push_back(op & ~OP_INTEG);
        stream.push_back(OP_INTEG);
      } else if (narrow) {
        stream.push_back(links[op].x | (links[op].y << 16));
        stream.push_back(op);
      } else {
        stream.push_back(op);
        stream.push_back(OP_WIDE);
      }
    }
    while ((stream.size() - at) % 4) stream.push_back(0);
    chunk_len.push_back((uint32_t)(stream.size() - at));
    if (chunk_len.back() > SCHED_CHUNK_WORDS) std::abort();
    seg_end.clear();
    chunk_ops.clear();
  };
  for (uint32_t l = 1; l <= maxl; ++l) {
    uint32_t b = start[l];
    const uint32_t e = start[l + 1];
    while (b < e) {
      // words: 1 (nseg) + segments (+1 for this one) + 1 pad + 2 per op + 3 pad
      const size_t fixed = 1 + (seg_end.size() + 1) + 1 + 3;
      const size_t used = fixed + 2 * chunk_ops.size();
      if (used + 2 > SCHED_CHUNK_WORDS) {
        flush();
        continue;
      }
      const size_t room = (SCHED_CHUNK_WORDS - used) / 2;
      const uint32_t take = (uint32_t)std::min<size_t>(room, e - b);
      chunk_ops.insert(chunk_ops.end(), sorted.begin() + b, sorted.begin() + b + take);
      seg_end.push_back((uint32_t)chunk_ops.size());
      b += take;
    }
  }
  flush();
  d.nchunks = (uint32_t)chunk_off.size() - d.chunk0;
  d.off = d.words = d.len0 = d.maxw = 0;
  d.nop_pad = padded ? 1u : 0u;
  for (uint32_t l = 1; l <= maxl; ++l) d.maxw = std::max(d.maxw, start[l + 1] - start[l]);
  if (d.nchunks) {
    d.off = chunk_off[d.chunk0];
    d.len0 = chunk_len[d.chunk0];
    for (uint32_t c = d.chunk0; c + 1 < d.chunk0 + d.nchunks; ++c)  // self-check: contiguous
      if (chunk_off[c] + chunk_len[c] != chunk_off[c + 1]) std::abort();
    d.words = chunk_off.back() + chunk_len.back() - d.off;
  }
  const uint32_t id = (uint32_t)scheds.size();
  scheds.push_back(d);
  index.emplace(std::move(key), id);
  return id;
}

// Bounds check of a finished image: every index a kernel dereferences must
// land inside the world's arrays.  Runs on every plan (linear in the size of
// the world); a failure is a planner bug and stops the world from reaching
// the GPU.
static bool check_image(const WorldImage& im, const SchedRegistry& reg, std::string* why) {
  auto bad = [&](const std::string& m) {
    if (why) *why = "internal planner check failed: " + m;
    return false;
  };
  const DWorld& P = im.params;
  if (im.pos.size() != P.np || im.prev.size() != P.np) return bad("particle arrays");
  if (im.bodies.size() != P.nb) return bad("body count");
  for (const DBody& B : im.bodies) {
    if ((size_t)B.i0 + B.np > im.bidx.size()) return bad("body particle range");
    if ((size_t)B.l0 + B.nl > im.lab.size() || im.lab.size() != im.lrest.size() ||
        im.lab.size() != im.lstiff.size())
      return bad("body link range");
    for (uint32_t i = 0; i < B.np; ++i)
      if (im.bidx[B.i0 + i] >= P.np) return bad("body particle index");
    if (B.first != NO_FIRST &&
        ((size_t)B.first + B.np > P.np || (B.np && im.bidx[B.i0] != B.first)))
      return bad("body first particle");
    const uint32_t lim = B.local ? B.np : P.np;
    for (uint32_t k = 0; k < B.nl; ++k) {
      const uint2 e = im.lab[B.l0 + k];
      if (e.x >= lim || e.y >= lim || e.x == e.y) return bad("link endpoint");
    }
  }
  for (const GroupBody& g : im.groups) {
    if (g.body >= im.bodies.size()) return bad("group body id");
    const DBody& B = im.bodies[g.body];
    if (B.sched >= reg.scheds.size()) return bad("schedule id");
    const DSched& S = reg.scheds[B.sched];
    if ((size_t)S.chunk0 + S.nchunks > reg.chunk_off.size() ||
        (size_t)S.off + S.words > reg.stream.size())
      return bad("schedule range");
    if (g.smem && (!B.local || B.np > 65535u)) return bad("shared-memory body needs local links");
    if (g.large_c && (g.smem || !B.local || g.large_c > 16u || g.log2per > 14u ||
                      (size_t)g.large_c << g.log2per < B.np || g.T > 1024u))
      return bad("large-body executor layout");
    if (g.res && (!g.smem || g.res != S.words * 4u)) return bad("resident schedule size");
    if (g.T < 32 || g.T % 32) return bad("group size");
  }
  for (uint32_t b : im.serials)
    if (b >= im.bodies.size() || !im.bodies[b].local) return bad("serial body");
  if (im.cpos.size() != P.nc || im.crad.size() != P.nc) return bad("circle arrays");
  for (const uint2& e : im.clab)
    if (e.x >= P.nc || e.y >= P.nc) return bad("circle link");
  if (im.polys.size() != P.ng || im.pcenter.size() != P.ng) return bad("polygon arrays");
  for (const DPoly& g : im.polys) {
    if ((size_t)g.v0 + g.nv > im.vpos.size()) return bad("polygon vertex range");
    if ((size_t)g.l0 + g.nl > im.plab.size()) return bad("polygon link range");
    for (uint32_t k = 0; k < g.nl; ++k) {
      const uint2 e = im.plab[g.l0 + k];
      if (e.x >= g.nv || e.y >= g.nv) return bad("polygon link endpoint");
    }
  }
  const size_t nst = P.ng >= 2 ? (size_t)P.ng * (P.ng - 1) + 1 : 0;
  if (im.stage_off.size() != nst) return bad("polygon stage table");
  if (im.stage_pr.size() != (nst ? nst - 1 : 0)) return bad("polygon stage pairs");
  for (uint32_t v : im.stage_pr)
    if ((v & 0xFFFFu) >= P.ng || (v >> 16) >= P.ng) return bad("polygon stage pair");
  for (size_t i = 1; i < nst; ++i)
    if (im.stage_off[i] < im.stage_off[i - 1]) return bad("polygon stage order");
  return true;
}

namespace {
struct Comp {
  std::vector<uint32_t> parts;  // ascending world indices
  std::vector<uint32_t> links;  // world link ids in execution order
};

uint32_t single_pass_depth(const WorldHost& w, const Comp& c, std::vector<uint32_t>& last) {
  uint32_t depth = 0;
  for (uint32_t k : c.links) {
    const uint32_t a = (uint32_t)w.particle_links[k].particle_a;
    const uint32_t b = (uint32_t)w.particle_links[k].particle_b;
    const uint32_t l = std::max(last[a], last[b]) + 1;
    last[a] = l;
    last[b] = l;
    depth = std::max(depth, l);
  }
  for (uint32_t k : c.links) {
    last[w.particle_links[k].particle_a] = 0;
    last[w.particle_links[k].particle_b] = 0;
  }
  return depth;
}
}  // namespace

int plan_world(const WorldHost& w, const PlanTuning& tune, SchedRegistry& reg, WorldImage& im,
               std::string* why) {
  int st = validate_world(w, why);
  if (st != OK) return st;
  const size_t np64 = w.particles.size();
  if (np64 >= 0x7FFFFFFFull || w.particle_links.size() >= 0x7FFFFFFFull) {
    if (why) *why = "world too large for 32-bit indices";
    return ERR_ARG;
  }
  const uint32_t np = (uint32_t)np64;
  const uint32_t nl = (uint32_t)w.particle_links.size();
  im = WorldImage();
  DWorld& P = im.params;
  std::memset(&P, 0, sizeof(P));
  P.gx = 0.0f + w.gravity.x;  // acc = 0 + g at integrate time (src/particle.rs:52-54)
  P.gy = 0.0f + w.gravity.y;
  P.bx = w.bounds.pos.x;
  P.by = w.bounds.pos.y;
  P.bw = w.bounds.size.x;
  P.bh = w.bounds.size.y;
  P.radius = w.particle_radius;
  P.cell = w.grid_cell;
  P.icell = pow2_reciprocal(w.grid_cell);
  P.S = w.sub_steps;
  P.I = w.link_iters;
  P.flags = w.collide & (COLLIDE_PP | COLLIDE_PC | COLLIDE_PPOLY);
  P.np = np;
  P.nc = (uint32_t)w.circles.size();
  P.ncl = (uint32_t)w.circle_links.size();
  P.ng = (uint32_t)w.polygons.size();
  im.ext = P.flags != 0;
  const bool full = !im.ext;

  im.pos.resize(np);
  im.prev.resize(np);
  for (uint32_t i = 0; i < np; ++i) {
    im.pos[i] = make_float2(w.particles[i].pos.x, w.particles[i].pos.y);
    im.prev[i] = make_float2(w.particles[i].prev_pos.x, w.particles[i].prev_pos.y);
  }

  // link execution order: insertion order, or colour-major in fast mode
  std::vector<uint32_t> order(nl);
  std::iota(order.begin(), order.end(), 0u);
  if (w.mode == MODE_FAST) {
    order = colour_link_order(w, &im.stats.colours);
    im.link_order = order;
  }

  // connected components (union-find over links)
  std::vector<uint32_t> parent(np);
  std::iota(parent.begin(), parent.end(), 0u);
  auto find = [&](uint32_t x) {
    while (parent[x] != x) {
      parent[x] = parent[parent[x]];
      x = parent[x];
    }
    return x;
  };
  for (uint32_t k = 0; k < nl; ++k) {
    uint32_t a = find((uint32_t)w.particle_links[k].particle_a);
    uint32_t b = find((uint32_t)w.particle_links[k].particle_b);
    if (a != b) parent[std::max(a, b)] = std::min(a, b);
  }
  std::vector<int64_t> comp_of_root(np, -1);
  std::vector<Comp> comps;
  std::vector<uint32_t> comp_of(np);
  for (uint32_t i = 0; i < np; ++i) {
    const uint32_t r = find(i);
    if (comp_of_root[r] < 0) {
      comp_of_root[r] = (int64_t)comps.size();
      comps.emplace_back();
    }
    comp_of[i] = (uint32_t)comp_of_root[r];
    comps[comp_of[i]].parts.push_back(i);
  }
  for (uint32_t k : order) comps[comp_of[w.particle_links[k].particle_a]].links.push_back(k);

  std::vector<uint32_t> last(np, 0), local(np, 0);
  std::vector<uint32_t> free_parts;
  std::vector<const Comp*> pack;
  uint32_t pack_np = 0, pack_nl = 0;

  auto emit_group = [&](const std::vector<const Comp*>& cs) {
    DBody B{};
    B.i0 = (uint32_t)im.bidx.size();
    B.l0 = (uint32_t)im.lab.size();
    uint32_t n = 0;
    for (const Comp* c : cs)
      for (uint32_t p : c->parts) {
        local[p] = n++;
        im.bidx.push_back(p);
      }
    B.np = n;
    std::vector<uint2> loc;
    for (const Comp* c : cs)
      for (uint32_t k : c->links) {
        const Link& L = w.particle_links[k];
        loc.push_back(make_uint2(local[L.particle_a], local[L.particle_b]));
        im.lrest.push_back(L.target_distance);
        im.lstiff.push_back(L.stiffness);
      }
    B.nl = (uint32_t)loc.size();
    const size_t region = align16((full ? 16u : 8u) * (size_t)B.np + 8u * (size_t)B.nl);
    const bool smem = region <= tune.smem_max && B.np <= 65535u;
    // whether the large-body executor (below) will run it
    const bool to_large = !smem && tune.large_max > 0 && B.np > 0 &&
                          (B.np + (1u << (full ? 13u : 14u)) - 1u) >> (full ? 13u : 14u) <=
                              tune.large_max;
    B.sched = reg.get(loc.data(), B.nl, B.np, P.S, P.I, full, to_large);
    const DSched& S = reg.scheds[B.sched];
    const float avg = S.nlvl ? (float)S.nops / (float)S.nlvl : 1.0f;
    uint32_t T = pow2ceil((uint32_t)(avg / tune.width_per_thread + 0.999f));
    T = std::min(std::max(T, tune.t_min), tune.t_max);
    // the whole schedule resident in shared memory when it fits beside the body
    uint32_t res = 0;
    if (smem && tune.resident) {
      const size_t sb = (size_t)S.words * 4u;
      if (region + sb + GROUP_TAIL_BYTES <= tune.res_max)
        res = (uint32_t)sb;
    }
    // A body over one CTA's shared memory: the large-body executor keeps its
    // positions (and prev) in the shared memory of a cluster of up to
    // large_max CTAs, at most 128 KB each (8,192 particles whole-step,
    // 16,384 for link passes), with link parameters and schedule read
    // through the caches; beyond that the group executor runs it from
    // global memory.
    uint32_t large_c = 0, log2per = 0, TL = T;
    if (!smem && tune.large_max > 0 && B.np > 0) {
      const uint32_t cap_log2 = full ? 13u : 14u;
      uint32_t l2 = 0;
      while (l2 < cap_log2 && (1u << l2) < B.np) ++l2;
      const uint32_t c = (B.np + (1u << l2) - 1u) >> l2;
      if (c <= tune.large_max) {
        large_c = c;
        log2per = l2;
        const float w = avg / (tune.width_per_thread * (float)c);
        TL = std::min<uint32_t>(1024u, std::max<uint32_t>(64u, pow2ceil((uint32_t)(w + 0.999f))));
      }
    }
    const bool local = smem || large_c > 0;
    B.local = local ? 1u : 0u;
    for (size_t i = 0; i < loc.size(); ++i) {
      if (local) im.lab.push_back(loc[i]);
      else im.lab.push_back(make_uint2(im.bidx[B.i0 + loc[i].x], im.bidx[B.i0 + loc[i].y]));
    }
    const uint32_t id = (uint32_t)im.bodies.size();
    im.bodies.push_back(B);
    GroupBody gbody{id, large_c ? TL : T, smem ? (uint32_t)region : 0u, res, smem};
    gbody.large_c = large_c;
    gbody.log2per = log2per;
    im.groups.push_back(gbody);
    im.stats.group_bodies++;
    if (large_c) im.stats.large_bodies++;
    else if (!smem) im.stats.global_bodies++;
    im.stats.levels += S.nlvl;
    im.stats.ops += S.nops;
  };
  auto flush_pack = [&]() {
    if (!pack.empty()) emit_group(pack);
    pack.clear();
    pack_np = pack_nl = 0;
  };

  for (const Comp& c : comps) {
    if (c.links.empty()) {
      free_parts.push_back(c.parts[0]);
      continue;
    }
    const uint32_t depth = single_pass_depth(w, c, last);
    const float width = (float)c.links.size() / (float)std::max(depth, 1u);
    if (width < tune.serial_width) {
      DBody B{};
      B.i0 = (uint32_t)im.bidx.size();
      B.np = (uint32_t)c.parts.size();
      B.l0 = (uint32_t)im.lab.size();
      B.nl = (uint32_t)c.links.size();
      B.local = 1;  // body-local endpoints: index into the body's particle list
      uint32_t nloc = 0;
      for (uint32_t p : c.parts) {
        local[p] = nloc++;
        im.bidx.push_back(p);
      }
      for (uint32_t k : c.links) {
        const Link& L = w.particle_links[k];
        im.lab.push_back(make_uint2(local[L.particle_a], local[L.particle_b]));
        im.lrest.push_back(L.target_distance);
        im.lstiff.push_back(L.stiffness);
      }
      im.serials.push_back((uint32_t)im.bodies.size());
      im.bodies.push_back(B);
      im.stats.serial_bodies++;
      continue;
    }
    const uint32_t cn = (uint32_t)c.parts.size(), cl = (uint32_t)c.links.size();
    if (!pack.empty() && (pack_np + cn > tune.pack_np || pack_nl + cl > tune.pack_nl)) flush_pack();
    pack.push_back(&c);
    pack_np += cn;
    pack_nl += cl;
  }
  flush_pack();
  // link-free particles: integrate-only bodies (the extension pipeline
  // integrates every particle in its collide pass instead)
  if (full) {
    for (size_t i = 0; i < free_parts.size(); i += tune.free_chunk) {
      std::vector<Comp> chunk(1);
      const size_t e = std::min(free_parts.size(), i + tune.free_chunk);
      chunk[0].parts.assign(free_parts.begin() + i, free_parts.begin() + e);
      std::vector<const Comp*> cs{&chunk[0]};
      emit_group(cs);
    }
  }
  P.nb = (uint32_t)im.bodies.size();
  im.stats.bodies = P.nb;
  // particle collisions with every particle in a shared-memory group body:
  // the link executor counts them into the grid (GRID_IN_LINKS)
  if ((P.flags & COLLIDE_PP) && free_parts.empty() && im.serials.empty() && np > 0) {
    bool all_smem = true;
    for (const GroupBody& gb : im.groups) all_smem = all_smem && gb.smem;
    if (all_smem) P.flags |= GRID_IN_LINKS;
  }

  // circles (src/circle.rs:4-8) and circle links
  for (const Circle& c : w.circles) {
    im.cpos.push_back(make_float2(c.point.pos.x, c.point.pos.y));
    im.cprev.push_back(make_float2(c.point.prev_pos.x, c.point.prev_pos.y));
    im.cacc.push_back(make_float2(c.point.acc.x, c.point.acc.y));
    im.crad.push_back(c.radius);
    im.cstatic.push_back(c.is_static ? 1u : 0u);
  }
  for (const Link& l : w.circle_links) {
    im.clab.push_back(make_uint2((uint32_t)l.particle_a, (uint32_t)l.particle_b));
    im.clrest.push_back(l.target_distance);
  }
  // polygons (src/polygon.rs:7-14)
  for (const Polygon& g : w.polygons) {
    DPoly d{};
    d.v0 = (uint32_t)im.vpos.size();
    d.nv = (uint32_t)g.particles.size();
    d.l0 = (uint32_t)im.plab.size();
    d.nl = (uint32_t)g.particle_links.size();
    d.is_static = g.is_static ? 1u : 0u;
    for (const Particle& v : g.particles) {
      im.vpos.push_back(make_float2(v.pos.x, v.pos.y));
      im.vprev.push_back(make_float2(v.prev_pos.x, v.prev_pos.y));
      im.vacc.push_back(make_float2(v.acc.x, v.acc.y));
    }
    for (const Link& l : g.particle_links) {
      im.plab.push_back(make_uint2((uint32_t)l.particle_a, (uint32_t)l.particle_b));
      im.plrest.push_back(l.target_distance);
    }
    im.pcenter.push_back(make_float2(g.center.x, g.center.y));
    im.polys.push_back(d);
  }
  // polygon pair stages: (i,j) then (j,i) for pairs i<j in row-major order
  if (P.ng >= 2) {
    uint32_t acc = 0;
    if (P.ng > 65535u) {
      if (why) *why = "at most 65535 polygons per world";
      return ERR_ARG;
    }
    for (uint32_t i = 0; i < P.ng; ++i)
      for (uint32_t j = i + 1; j < P.ng; ++j) {
        im.stage_off.push_back(acc);
        im.stage_pr.push_back(i | (j << 16));
        acc += im.polys[i].nv * im.polys[j].nv;
        im.stage_off.push_back(acc);
        im.stage_pr.push_back(j | (i << 16));
        acc += im.polys[j].nv * im.polys[i].nv;
      }
    im.stage_off.push_back(acc);
  }
  for (DBody& B : im.bodies) {  // contiguous particle lists load without bidx
    B.first = B.np ? im.bidx[B.i0] : NO_FIRST;
    for (uint32_t i = 1; i < B.np && B.first != NO_FIRST; ++i)
      if (im.bidx[B.i0 + i] != B.first + i) B.first = NO_FIRST;
  }
  if (!check_image(im, reg, why)) return ERR_STATE;
  return OK;
}

BlockLayout layout_of(const WorldImage& im) {
  BlockLayout L;
  size_t o = 0;
  auto seg = [&](size_t bytes) {
    size_t at = o;
    o = align16(o + bytes);
    return at;
  };
  const size_t np = im.pos.size(), nc = im.cpos.size(), nv = im.vpos.size(),
               ng = im.polys.size();
  // the state prefix is one contiguous run of float2
  L.o_pos = 0;
  L.o_prev = L.o_pos + 8 * np;
  L.o_cpos = L.o_prev + 8 * np;
  L.o_cprev = L.o_cpos + 8 * nc;
  L.o_cacc = L.o_cprev + 8 * nc;
  L.o_vpos = L.o_cacc + 8 * nc;
  L.o_vprev = L.o_vpos + 8 * nv;
  L.o_vacc = L.o_vprev + 8 * nv;
  L.o_pcenter = L.o_vacc + 8 * nv;
  L.state_bytes = L.o_pcenter + 8 * ng;
  o = align16(L.state_bytes);
  L.o_pos1 = seg(8 * np);
  L.o_bidx = seg(4 * im.bidx.size());
  L.o_bodies = seg(sizeof(DBody) * im.bodies.size());
  L.o_lab = seg(8 * im.lab.size());
  L.o_lrest = seg(4 * im.lrest.size());
  L.o_lstiff = seg(4 * im.lstiff.size());
  L.o_crad = seg(4 * nc);
  L.o_cstatic = seg(4 * nc);
  L.o_clab = seg(8 * im.clab.size());
  L.o_clrest = seg(4 * im.clrest.size());
  L.o_polys = seg(sizeof(DPoly) * ng);
  L.o_paabb = seg(16 * ng);
  L.o_plab = seg(8 * im.plab.size());
  L.o_plrest = seg(4 * im.plrest.size());
  L.o_stage = seg(4 * im.stage_off.size());
  L.o_stage_pr = seg(4 * im.stage_pr.size());
  L.total = std::max<size_t>(o, 16);
  return L;
}

void write_block(const WorldImage& im, const BlockLayout& L, unsigned char* dst) {
  std::memset(dst, 0, L.total);
  auto put = [&](size_t off, const void* src, size_t bytes) {
    if (bytes) std::memcpy(dst + off, src, bytes);
  };
  put(L.o_pos, im.pos.data(), 8 * im.pos.size());
  put(L.o_prev, im.prev.data(), 8 * im.prev.size());
  put(L.o_cpos, im.cpos.data(), 8 * im.cpos.size());
  put(L.o_cprev, im.cprev.data(), 8 * im.cprev.size());
  put(L.o_cacc, im.cacc.data(), 8 * im.cacc.size());
  put(L.o_vpos, im.vpos.data(), 8 * im.vpos.size());
  put(L.o_vprev, im.vprev.data(), 8 * im.vprev.size());
  put(L.o_vacc, im.vacc.data(), 8 * im.vacc.size());
  put(L.o_pcenter, im.pcenter.data(), 8 * im.pcenter.size());
  put(L.o_pos1, im.pos.data(), 8 * im.pos.size());
  put(L.o_bidx, im.bidx.data(), 4 * im.bidx.size());
  put(L.o_bodies, im.bodies.data(), sizeof(DBody) * im.bodies.size());
  put(L.o_lab, im.lab.data(), 8 * im.lab.size());
  put(L.o_lrest, im.lrest.data(), 4 * im.lrest.size());
  put(L.o_lstiff, im.lstiff.data(), 4 * im.lstiff.size());
  put(L.o_crad, im.crad.data(), 4 * im.crad.size());
  put(L.o_cstatic, im.cstatic.data(), 4 * im.cstatic.size());
  put(L.o_clab, im.clab.data(), 8 * im.clab.size());
  put(L.o_clrest, im.clrest.data(), 4 * im.clrest.size());
  put(L.o_polys, im.polys.data(), sizeof(DPoly) * im.polys.size());
  put(L.o_plab, im.plab.data(), 8 * im.plab.size());
  put(L.o_plrest, im.plrest.data(), 4 * im.plrest.size());
  put(L.o_stage, im.stage_off.data(), 4 * im.stage_off.size());
  put(L.o_stage_pr, im.stage_pr.data(), 4 * im.stage_pr.size());
}

}  // namespace b2d

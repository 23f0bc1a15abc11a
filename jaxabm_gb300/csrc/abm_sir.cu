// SIR contagion on a Network (CSR), batched over any number of model instances.
//
// Agent semantics (partitionable jax.random; agent i of an instance holds
// agent_key = split(coll_key, n)[i], jaxabm/agent.py:156; k_inf, k_rec = split(agent_key)):
//   S: infected if any neighbour slot k (CSR position row_ptr[i] + k) whose neighbour is I
//      has uniform(k_inf, (deg,))[k] < beta           (bernoulli(beta) per I-edge)
//   I: recovers if uniform(k_rec) < gamma
//   R: stays R
// All agents read the pre-step states (synchronous update, jaxabm/agent.py:168-177); the
// S/I/R counts after each step are the metrics (jaxabm/model.py:193-200).
//
// Work-efficient ("frontier") formulation over one byte per agent:
//     word = (number of infected neighbours << 2) | compartment      (degree < 63)
//     word = (63 << 2) | compartment, count in hub_counts[i]          (hubs: degree >= 63)
// A second copy of the compartments, 2 bits per agent (16 agents per 32-bit word of
// `comp`, ~22 MB for a 4,096-instance ensemble), serves the random neighbour reads of the
// decisions from L2; the bytes (~87 MB) serve the sweep and the count updates;
// CSR columns, row offsets and list entries are read with the streaming (evict-first)
// policy so that they do not displace the words.  Column entries that point at a hub carry
// bit 31 (set by abm_sir_pack), so a count update knows where its target's count lives
// without a further read.  A count update is a 32-bit reduction (red.global.add) on the
// aligned word holding the target byte: the byte never borrows or carries into its
// neighbours, because a count never drops below the number of its pre-step infected
// neighbours that are still to recover, and never exceeds the degree (< 63).
//
// A step is four launches:
//   sweep      over (instance, 8192-agent tile) work items, 32 agents per lane read with
//              two 128-bit loads.  Infected agents draw their recovery right there (each
//              warp queues its infected agents in shared memory and draws them one lane
//              each); susceptible agents with infected neighbours are appended to a
//              candidate list in agent order (8-byte entries; one counter atomic per CTA
//              and tile).  Everyone else (most agents) costs one byte.
//   candidates one lane per candidate (entries and row offsets loaded a pass ahead): it
//              reads its CSR row, eight column/compartment loads in flight per pass, until
//              all its infected neighbours were seen, then draws for those slots in order
//              with the lanes of the warp drawing together, stopping at the first firing
//              draw (rows longer than 32 slots are scanned by the whole warp, 128 slots per
//              pass, with warp votes).  Decisions read only the 2-bit compartment copy,
//              which no kernel writes before the push, so every decision sees the pre-step
//              states.  A newly infected agent's own word and its neighbours' counts are
//              updated right away (+1; counts only grow during the kernel, so a hub's count
//              is not read: its row is scanned to the end).  Changes of both kernels are
//              buffered per warp in shared memory and appended to the change list 32 at a
//              time.
//   push       +1 on the compartment copy of every changed agent; for recoveries also +1
//              on the agent's own word and -1 on its neighbours' counts (one warp per 32
//              changes, walking the concatenation of their rows one slot per lane).
//   finalize   one thread per instance: S/I/R counts of the step from the transitions,
//              rng = split(rng)[0], t += 1, the next step's collection key, done flag after
//              the last step; clears the lists.
// Integer atomics commute, so every result is exact and independent of scheduling.  No
// kernel waits on anything.

#include <algorithm>

#include "abm_common.cuh"

namespace {

constexpr int kSirThreads = 256;
constexpr int kWarpsPerCta = kSirThreads / 32;
constexpr int kVecs = 2;                           // 128-bit loads per lane and tile
constexpr int kPerThread = 16 * kVecs;             // agents (bytes) per lane: 32
constexpr int kSub = 32 * kPerThread;              // 1024 agents per warp and tile
constexpr int kTile = kSirThreads * kPerThread;    // 8192 agents per work item
constexpr int kHeavyDeg = 32;
constexpr int kHeavyUnroll = 4;                    // slots per lane per pass of a warp row scan
constexpr int kResHeavyUnroll = 2;                 // the same on the resident path
constexpr int kDrawFirstDeg = 96;                  // rows longer than this draw before reading
constexpr int kChunk = 8;                          // row slots per scan pass (grid path)
constexpr int kResScan = 5;                        // row slots per scan pass (resident path)
constexpr int kHubDeg = 63;                        // degree from which a count is a hub count
constexpr uint32_t kHubMark = 63;                  // count field of a hub's word
constexpr uint32_t kTag = 0x80000000u;             // column entry of a hub neighbour
constexpr uint32_t kIdx = 0x7FFFFFFFu;
constexpr int kInstBits = 26;                      // instance bits of a candidate entry
constexpr int kCompactEvery = 8;                   // steps between work-list compactions
constexpr int kFusedFinalizeMax = 256;             // instances finalized by the last push CTA
constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kS = 0, kI = 1;

static_assert(sizeof(abm_sir_instance) == 152, "abm_sir_instance layout");
static_assert(sizeof(abm_work_item) == 16, "abm_work_item layout");

// List workspace: this header, then `capacity` change entries (int2 {inst, agent << 2 |
// new compartment}), then `capacity` candidate entries of susceptible agents (int2
// {inst | min(count, 63) << kInstBits, agent}), then the compacted work list.
struct ListHeader {
  int32_t changes;
  int32_t overflow;
  int32_t cand_s;
  int32_t live_tiles;   // length of the compacted work list
  uint32_t push_done;   // CTAs of the push kernel that finished (fused finalize)
  int32_t reserved[3];
};
static_assert(sizeof(ListHeader) == 32, "list header layout");

// The compacted work list (tiles of live instances, `max_tiles` int4 entries) sits at the
// end of the workspace.
struct Lists {
  ListHeader* hdr;
  int2* changes;
  int2* cands;
  int4* live_work;
  int capacity;
};

__device__ __forceinline__ uint2 step_key_of(const abm_sir_instance* I, int t, uint2 rng) {
  // collection key of step t: given per step, or from the instance's key chain
  // (step_key = split(rng)[1]; coll_key = split(step_key)[1], jaxabm/model.py:156,164)
  return I->coll_keys != nullptr ? abm::load_key(I->coll_keys + 2 * (size_t)t)
                                 : abm::split_at(abm::split_at(rng, 1), 1);
}

__device__ __forceinline__ int live_count(const int32_t* live, int nwork) {
  return live != nullptr ? min(*live, nwork) : nwork;
}

// Column entry k of a row, read once (streaming policy: evict first from L1 and L2).
__device__ __forceinline__ uint32_t ld_col(const int32_t* __restrict__ adj, int k) {
  return static_cast<uint32_t>(__ldcs(adj + k));
}

// Compartment of agent t from the 2-bit compartment array (16 agents per 32-bit word).
__device__ __forceinline__ uint32_t comp_of(const uint32_t* __restrict__ comp, uint32_t t) {
  return (comp[t >> 4] >> (2u * (t & 15u))) & 3u;
}

// Fire-and-forget global reduction (no value returned, so the issuing warp never waits
// for it).
__device__ __forceinline__ void red_add(uint32_t* p, uint32_t v) {
  asm volatile("red.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void red_add(int32_t* p, int32_t v) {
  asm volatile("red.relaxed.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void red_add(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Adds d to the infected-neighbour count of the agent that column entry v points at.
__device__ __forceinline__ void add_count(uint8_t* words, int32_t* hubs, uint32_t v, int d) {
  const uint32_t t = v & kIdx;
  if (v & kTag) {
    red_add(reinterpret_cast<uint32_t*>(hubs + t), static_cast<uint32_t>(d));
  } else {
    const uintptr_t a = reinterpret_cast<uintptr_t>(words + t);
    red_add(reinterpret_cast<uint32_t*>(a & ~static_cast<uintptr_t>(3)),
            static_cast<uint32_t>(4 * d) << (8u * static_cast<uint32_t>(a & 3)));
  }
}

// Warp-aggregated append: lanes with `want` get consecutive slots of *counter.
__device__ __forceinline__ int warp_append(bool want, int32_t* counter, int lane) {
  const unsigned m = __ballot_sync(kFull, want);
  if (!m) return -1;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(kFull, base, leader);
  return want ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

// Collection key of each live instance's current step.
__global__ void sir_prepare_kernel(abm_sir_instance* __restrict__ insts, int ninst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ninst) return;
  abm_sir_instance* I = insts + k;
  if (I->t >= I->steps) return;
  const uint2 c = step_key_of(I, I->t, make_uint2(I->rng[0], I->rng[1]));
  I->coll[0] = c.x;
  I->coll[1] = c.y;
}

__device__ __forceinline__ uint32_t byte_of(const uint32_t (&q)[4 * kVecs], int j) {
  return (q[j >> 2] >> (8 * (j & 3))) & 0xFFu;
}

// Flags of 32 agents' words (8 x 32 bits, agent j in byte j): bit j of need_s = susceptible
// with a non-zero count (hubs included), need_i = infected, hub_s = susceptible hub.
// Four agents per word at once: per byte, the compartment bits (S = 0, I = 1), count > 0
// (adding 0x7F sets bit 7 iff the 6-bit count is non-zero) and the hub mark (count + 1
// reaches 64 only for 63); bit 0 of each byte becomes one mask bit by one multiply (the
// partial products land on distinct bits, so nothing carries).
__device__ __forceinline__ void sweep_flags(const uint32_t (&q)[4 * kVecs], unsigned& need_s,
                                            unsigned& need_i, unsigned& hub_s) {
  need_s = need_i = hub_s = 0;
#pragma unroll
  for (int k = 0; k < 4 * kVecs; ++k) {
    const uint32_t w = q[k];
    const uint32_t lo = w & 0x01010101u, hi = (w >> 1) & 0x01010101u;
    const uint32_t cnt = (w >> 2) & 0x3F3F3F3Fu;
    const uint32_t is_s = ~(lo | hi) & 0x01010101u;
    const uint32_t is_i = lo & ~hi;
    const uint32_t nz = ((cnt + 0x7F7F7F7Fu) >> 7) & 0x01010101u;
    const uint32_t hub = ((cnt + 0x01010101u) >> 6) & 0x01010101u;
    need_s |= (((is_s & nz) * 0x01020408u) >> 24 & 0xFu) << (4 * k);
    need_i |= ((is_i * 0x01020408u) >> 24 & 0xFu) << (4 * k);
    hub_s |= (((is_s & hub) * 0x01020408u) >> 24 & 0xFu) << (4 * k);
  }
}

// Clears from need_s the susceptible hubs (bits of hub_s) whose count in hubs[] (agent j at
// hubs[j]) is not positive: a hub needs a decision only with infected neighbours (the grid
// path's sweep; its candidates kernel draws at every slot of a long row first, so an idle
// hub would cost a whole row of draws there).  Four counts are read at a time, through L2.
__device__ __forceinline__ unsigned drop_idle_hubs(unsigned need_s, unsigned hub_s,
                                                   const int32_t* hubs) {
  while (hub_s) {
    int jj[4];
    int32_t hc[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      jj[u] = hub_s ? __ffs(hub_s) - 1 : -1;
      hub_s &= hub_s - 1;
      hc[u] = jj[u] >= 0 ? __ldcg(hubs + jj[u]) : 1;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (jj[u] >= 0 && hc[u] <= 0) need_s &= ~(1u << jj[u]);
  }
  return need_s;
}

// Changes buffered per warp in shared memory and appended to the change list 32 at a time
// (one counter atomic per 32 changes instead of one per pass).
constexpr int kBuf = 64;

__device__ __forceinline__ void flush_changes(int2* buf, int k, Lists& L, int lane) {
  if (k == 0) return;  // uniform over the warp
  int base = 0;
  if (lane == 0) base = atomicAdd(&L.hdr->changes, k);
  base = __shfl_sync(kFull, base, 0);
  if (lane < k) {
    const int pos = base + lane;
    if (pos < L.capacity) L.changes[pos] = buf[lane];
    else L.hdr->overflow = 1;
  }
}

__device__ __forceinline__ void buffer_change(bool changed, int2 entry, int2* buf, int& count,
                                              Lists& L, int lane) {
  const unsigned m = __ballot_sync(kFull, changed);
  if (!m) return;
  if (changed) buf[count + __popc(m & ((1u << lane) - 1u))] = entry;
  count += __popc(m);
  __syncwarp();
  if (count >= 32) {
    flush_changes(buf, 32, L, lane);
    const int rest = count - 32;
    int2 v = make_int2(0, 0);
    if (lane < rest) v = buf[32 + lane];
    __syncwarp();
    if (lane < rest) buf[lane] = v;
    __syncwarp();
    count = rest;
  }
}

// Count updates of up to 32 CSR rows, one per lane (len 0: none), by the whole warp: the
// warp walks the concatenation of the rows 32 slots per pass, slot f belonging to the first
// lane whose inclusive prefix sum of row lengths exceeds f (a five-step binary search over
// the lanes' prefix sums), so every lane pushes one slot per pass whatever the row lengths
// and consecutive lanes read consecutive column entries; kPushPasses passes are in flight.
// tag = instance << 1 | (1: +1, 0: -1).  Called by all lanes of the warp.
constexpr int kPushPasses = 4;

__device__ __forceinline__ void push_rows(const abm_sir_instance* __restrict__ insts, int tag,
                                          int row0, int len, int lane) {
  int incl = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(kFull, incl, 31);
  const int shift = row0 - (incl - len);  // column index of concatenated slot f: f + shift
  for (int base = 0; base < total; base += 32 * kPushPasses) {
    uint32_t v[kPushPasses];
    int owner[kPushPasses];
#pragma unroll
    for (int u = 0; u < kPushPasses; ++u) {
      const int f = base + 32 * u + lane;
      int lo = 0;
#pragma unroll
      for (int st = 16; st > 0; st >>= 1) {
        const int p = __shfl_sync(kFull, incl, lo + st - 1);
        if (p <= f) lo += st;
      }
      const int sh = __shfl_sync(kFull, shift, lo);
      owner[u] = __shfl_sync(kFull, tag, lo);
      v[u] = f < total ? ld_col(insts[owner[u] >> 1].adj, f + sh) : 0u;
    }
#pragma unroll
    for (int u = 0; u < kPushPasses; ++u) {
      if (base + 32 * u + lane < total) {
        const abm_sir_instance* J = insts + (owner[u] >> 1);
        add_count(J->words, J->hub_counts, v[u], (owner[u] & 1) ? 1 : -1);
      }
    }
  }
}

// Adds 1 to the compartment field of agent i's word (S -> I, I -> R).
__device__ __forceinline__ void bump_word(uint8_t* words, int i) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(words + i);
  red_add(reinterpret_cast<uint32_t*>(a & ~static_cast<uintptr_t>(3)),
          1u << (8u * static_cast<uint32_t>(a & 3)));
}

// Per-instance sums over the lanes of a warp (lanes grouped by instance), added to the
// group's instance by the group's lowest lane: CSR slots scanned, infections, slots pushed,
// infection draws.
__device__ __forceinline__ void add_decided(bool valid, int inst, int scanned, int infected,
                                            int pushed, int draws, abm_sir_instance* insts,
                                            int lane) {
  if (!__any_sync(kFull, scanned != 0 || infected != 0 || draws != 0)) return;
  const unsigned group = __match_any_sync(kFull, valid ? inst : -1);
  const int s = __reduce_add_sync(group, scanned);
  const int f = __reduce_add_sync(group, infected);
  const int p = __reduce_add_sync(group, pushed);
  const int d = __reduce_add_sync(group, draws);
  if (valid && lane == __ffs(group) - 1) {
    if (s) red_add(&insts[inst].edges_scanned, static_cast<unsigned long long>(s));
    if (f) red_add(&insts[inst].step_si, f);
    if (p) red_add(&insts[inst].edges_pushed, static_cast<unsigned long long>(p));
    if (d) red_add(&insts[inst].draws, static_cast<unsigned long long>(d));
  }
}

// One step's sweep over (instance, 8192-agent tile) work items: lane l of warp w reads
// agents 1024w + 32l .. 1024w + 32l + 31 of the tile with two 128-bit loads.
//  * Infected agents draw their recovery here: each warp queues its infected agents in
//    shared memory and draws them 32 at a time, one lane each (no list entry).
//  * Susceptible agents with infected neighbours are appended to the candidate list in
//    agent order (block scan; one counter atomic per CTA and tile), so that consecutive
//    entries read nearby row offsets and CSR rows.
// Everyone else (most agents) costs one byte.
__global__ void __launch_bounds__(kSirThreads)
sir_sweep_kernel(abm_sir_instance* __restrict__ insts, const int4* __restrict__ work,
                 int nwork_max, const int32_t* __restrict__ live, Lists L) {
  __shared__ int swarp[kWarpsPerCta];
  __shared__ int sbase;
  __shared__ uint16_t squeue[kWarpsPerCta][kSub];
  __shared__ int2 sbuf[kWarpsPerCta][kBuf];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint16_t* __restrict__ queue = squeue[warp];
  int2* buf = sbuf[warp];
  int nbuf = 0;
  const int nwork = live_count(live, nwork_max);
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int4 item = work[w];
    abm_sir_instance* I = insts + item.x;
    // finished instances, and instances without an infected agent (nothing can change in
    // them any more: no infection source, no recovery), need no decisions
    if (I->t >= I->steps || I->num_i == 0) continue;  // uniform over the CTA
    const uint8_t* __restrict__ words = I->words;
    const int32_t* __restrict__ hubs = I->hub_counts;
    const int off = kSub * warp + kPerThread * lane;  // offset in the tile
    const int base = item.y + off;
    uint32_t q[4 * kVecs];
    const bool vec_ok = (reinterpret_cast<uintptr_t>(words + base) & 15) == 0;
#pragma unroll
    for (int v = 0; v < kVecs; ++v) {
      const int b16 = base + 16 * v;
      if (vec_ok && b16 + 16 <= item.z) {
        const uint4 x = *reinterpret_cast<const uint4*>(words + b16);
        q[4 * v] = x.x;
        q[4 * v + 1] = x.y;
        q[4 * v + 2] = x.z;
        q[4 * v + 3] = x.w;
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          uint32_t r = 0;
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int i = b16 + 4 * c + b;
            r |= (i < item.z ? static_cast<uint32_t>(words[i]) : 2u) << (8 * b);
          }
          q[4 * v + c] = r;
        }
      }
    }
    unsigned need_s, need_i, hub_s;
    sweep_flags(q, need_s, need_i, hub_s);
    need_s = drop_idle_hubs(need_s, hub_s, hubs + base);
    // both counts scanned at once (16 bits each): warp scan, then block totals
    const int mine = __popc(need_s) | (__popc(need_i) << 16);
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += u;
    }
    const int wtotal = __shfl_sync(kFull, incl, 31);
    if (lane == 31) swarp[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      int total = 0;
      for (int x = 0; x < kWarpsPerCta; ++x) total += swarp[x];
      const int ts = total & 0xFFFF, ti = total >> 16;
      sbase = ts ? atomicAdd(&L.hdr->cand_s, ts) : 0;
      if (ts + ti) red_add(&I->candidates, static_cast<unsigned long long>(ts + ti));
    }
    __syncthreads();
    int pos_s = (incl - mine) & 0xFFFF;
    for (int x = 0; x < warp; ++x) pos_s += swarp[x] & 0xFFFF;
    pos_s += sbase;
    int pos_i = (incl - mine) >> 16;  // within the warp's queue
    for (unsigned m = need_s; m; m &= m - 1) {
      const int j = __ffs(m) - 1;
      // {inst | min(count, 63) << 26, agent}: 63 is a hub's mark (count in hub_counts)
      const int c = static_cast<int>(words[base + j] >> 2);  // just loaded: an L1 hit
      if (pos_s < L.capacity) L.cands[pos_s] = make_int2(item.x | (c << kInstBits), base + j);
      else L.hdr->overflow = 1;
      ++pos_s;
    }
    for (unsigned m = need_i; m; m &= m - 1) queue[pos_i++] = static_cast<uint16_t>(off + __ffs(m) - 1);
    __syncwarp();
    // recovery draws of the warp's infected agents
    const int ni = wtotal >> 16;
    if (ni) {
      const uint2 coll = make_uint2(I->coll[0], I->coll[1]);
      const float gamma = I->gamma;
      int ir = 0;
      for (int k0 = 0; k0 < ni; k0 += 32) {
        const int k = k0 + lane;
        const bool valid = k < ni;
        const int i = item.y + (valid ? queue[k] : 0);
        bool changed = false;
        if (valid) {
          const uint2 krec = abm::split_at(abm::split_at(coll, (uint64_t)i), 1);
          changed = abm::unit_float(abm::bits_at(krec, 0)) < gamma;
        }
        ir += changed;
        buffer_change(changed, make_int2(item.x, (i << 2) | 2), buf, nbuf, L, lane);
      }
      ir = __reduce_add_sync(kFull, ir);
      if (lane == 0 && ir) red_add(&I->step_ir, ir);
    }
    __syncthreads();  // swarp, sbase and the queues are rewritten by the next tile
  }
  flush_changes(buf, nbuf, L, lane);
}

// Susceptible candidates: one lane each scans its CSR row, eight slots per pass (the eight
// column loads, then the eight neighbour-compartment loads, issued together), stopping at
// the first firing draw or once all its infected neighbours were seen; rows longer than 32
// slots are scanned by the whole warp, 128 slots per pass, with warp votes.  Decisions read
// only the 2-bit compartment copy (unchanged until the push kernel), so every decision sees
// the pre-step states; the rows of the newly infected agents are pushed (+1) by the warp
// at the end of each pass, and the changes go to the change list.
__global__ void __launch_bounds__(kSirThreads, 5)
sir_candidates_kernel(abm_sir_instance* __restrict__ insts, Lists L) {
  __shared__ int2 sbuf[kWarpsPerCta][kBuf];
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * kWarpsPerCta;
  const int wid = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  int2* buf = sbuf[threadIdx.x >> 5];
  int nbuf = 0;
  const int ns_count = min(L.hdr->cand_s, L.capacity);
  const int stride = warps * 32;
  // a lane's list entries are loaded two passes ahead and their row offsets one pass
  // ahead, so a pass starts with both in registers
  int2 e_next = make_int2(0, 0), e_next2 = make_int2(0, 0);
  int r0_next = 0, r1_next = 0;
  {
    const int k = wid * 32 + lane;
    if (k < ns_count) {
      e_next = __ldcs(&L.cands[k]);
      const int32_t* rp = insts[e_next.x & ((1 << kInstBits) - 1)].row_ptr;
      r0_next = __ldcs(rp + e_next.y);
      r1_next = __ldcs(rp + e_next.y + 1);
    }
    if (k + stride < ns_count) e_next2 = __ldcs(&L.cands[k + stride]);
  }
  for (int b = wid * 32; b < ns_count; b += stride) {
    const int k = b + lane;
    const bool valid = k < ns_count;
    const int2 e = e_next;
    const int r0_cur = r0_next, r1_cur = r1_next;
    e_next = e_next2;
    if (k + stride < ns_count) {
      const int32_t* rp = insts[e_next.x & ((1 << kInstBits) - 1)].row_ptr;
      r0_next = __ldcs(rp + e_next.y);
      r1_next = __ldcs(rp + e_next.y + 1);
    }
    if (k + 2 * stride < ns_count) e_next2 = __ldcs(&L.cands[k + 2 * stride]);
    const int inst = e.x & ((1 << kInstBits) - 1), i = e.y;
    const abm_sir_instance* I = insts + inst;
    int cnt = static_cast<int>(static_cast<uint32_t>(e.x) >> kInstBits);
    bool infected = false, heavy = false;
    int row0 = 0, deg = 0, scanned = 0, draws = 0;
    unsigned imask = 0;
    uint2 coll = make_uint2(0, 0);
    const int32_t* __restrict__ adj = nullptr;
    const uint32_t* __restrict__ comp = nullptr;
    float beta = 0.f;
    if (valid) {
      coll = make_uint2(I->coll[0], I->coll[1]);
      adj = I->adj;
      comp = I->comp;
      beta = I->beta;
      row0 = r0_cur;
      deg = r1_cur - r0_cur;
      // a hub's count is not read here (infections of this step are already being added
      // to it): its row is scanned to the end
      if (cnt == static_cast<int>(kHubMark)) cnt = deg;
      heavy = deg > kHeavyDeg;
      if (!heavy) {
        // slots of infected neighbours (bit k: slot k), read until all `cnt` were seen;
        // eight column loads, then eight neighbour loads, in flight per pass
        int seen = 0, k1 = 0;
        for (; k1 < deg && seen < cnt; k1 += kChunk) {
          int nb[kChunk];
          uint32_t wn[kChunk];
#pragma unroll
          for (int c = 0; c < kChunk; ++c)
            nb[c] = k1 + c < deg ? static_cast<int>(ld_col(adj, row0 + k1 + c) & kIdx) : -1;
#pragma unroll
          for (int c = 0; c < kChunk; ++c) wn[c] = nb[c] >= 0 ? comp_of(comp, nb[c]) : 0u;
#pragma unroll
          for (int c = 0; c < kChunk; ++c) {
            const bool inf = nb[c] >= 0 && (wn[c] & 3u) == kI;
            imask |= static_cast<unsigned>(inf) << (k1 + c);
            seen += inf;
          }
        }
        scanned = min(k1, deg);
      }
    }
    // infection draws in slot order, one per lane and pass, so that the lanes of the warp
    // draw together: a susceptible agent is infected iff some infected slot fires
    if (__any_sync(kFull, imask != 0)) {
      const uint2 kinf = abm::split_at(abm::split_at(coll, (uint64_t)i), 0);
      while (__any_sync(kFull, imask != 0)) {
        if (imask) {
          const int slot = __ffs(imask) - 1;
          imask &= imask - 1;
          ++draws;
          if (abm::unit_float(abm::bits_at(kinf, (uint64_t)slot)) < beta) {
            infected = true;
            imask = 0;
          }
        }
      }
    }

    // rows longer than kHeavyDeg: the whole warp scans them, one at a time
    unsigned hmask = __ballot_sync(kFull, heavy);
    while (hmask) {
      const int src = __ffs(hmask) - 1;
      hmask &= hmask - 1;
      const int hi = __shfl_sync(kFull, i, src);
      const int hrow = __shfl_sync(kFull, row0, src);
      const int hdeg = __shfl_sync(kFull, deg, src);
      int remaining = __shfl_sync(kFull, cnt, src);
      const uint2 hcoll = make_uint2(__shfl_sync(kFull, coll.x, src), __shfl_sync(kFull, coll.y, src));
      const float hbeta = __shfl_sync(kFull, beta, src);
      const int32_t* __restrict__ hadj = reinterpret_cast<const int32_t*>(
          __shfl_sync(kFull, reinterpret_cast<unsigned long long>(adj), src));
      const uint32_t* __restrict__ hcomp = reinterpret_cast<const uint32_t*>(
          __shfl_sync(kFull, reinterpret_cast<unsigned long long>(comp), src));
      const uint2 kinf = abm::split_at(abm::split_at(hcoll, (uint64_t)hi), 0);
      bool fired = false;
      int c = 0, hdraws = 0;
      if (hdeg > kDrawFirstDeg) {
        // long rows: the draws first (ALU only), the neighbour's compartment read only
        // where a draw fires -- a fraction beta of the slots -- in slot order, so the
        // first firing slot with an infected neighbour decides as in the scan below
        int loaded = 0;
        for (; c < hdeg && !fired; c += 32 * kHeavyUnroll) {
          unsigned fire = 0;
#pragma unroll
          for (int u = 0; u < kHeavyUnroll; ++u) {
            const int slot = c + 32 * u + lane;
            hdraws += slot < hdeg;
            if (slot < hdeg && abm::unit_float(abm::bits_at(kinf, (uint64_t)slot)) < hbeta)
              fire |= 1u << u;
          }
          uint32_t wv[kHeavyUnroll];
#pragma unroll
          for (int u = 0; u < kHeavyUnroll; ++u)
            wv[u] = (fire >> u) & 1u ? ld_col(hadj, hrow + c + 32 * u + lane) : 0u;
          bool f = false;
#pragma unroll
          for (int u = 0; u < kHeavyUnroll; ++u)
            if ((fire >> u) & 1u) f |= comp_of(hcomp, wv[u] & kIdx) == kI;
          loaded += __popc(fire);
          fired = __any_sync(kFull, f);
        }
        loaded = __reduce_add_sync(kFull, loaded);
        hdraws = __reduce_add_sync(kFull, hdraws);
        if (lane == src) {
          infected = fired;
          scanned = loaded;
          draws = hdraws;
        }
        continue;
      }
      for (; c < hdeg && !fired && remaining > 0; c += 32 * kHeavyUnroll) {
        uint32_t wv[kHeavyUnroll];
#pragma unroll
        for (int u = 0; u < kHeavyUnroll; ++u) {
          const int slot = c + 32 * u + lane;
          wv[u] = slot < hdeg ? ld_col(hadj, hrow + slot) : kTag;
        }
#pragma unroll
        for (int u = 0; u < kHeavyUnroll; ++u) {
          const int slot = c + 32 * u + lane;
          wv[u] = slot < hdeg ? comp_of(hcomp, wv[u] & kIdx) : 0u;
        }
        bool f = false;
        int seen = 0;
#pragma unroll
        for (int u = 0; u < kHeavyUnroll; ++u) {
          const int slot = c + 32 * u + lane;
          if (slot < hdeg && (wv[u] & 3u) == kI) {
            ++seen;
            if (!f) {
              ++hdraws;
              f = abm::unit_float(abm::bits_at(kinf, (uint64_t)slot)) < hbeta;
            }
          }
        }
        fired = __any_sync(kFull, f);
        remaining -= __reduce_add_sync(kFull, seen);
      }
      hdraws = __reduce_add_sync(kFull, hdraws);
      if (lane == src) {
        infected = fired;
        scanned = min(c, hdeg);
        draws = hdraws;
      }
    }

    // newly infected agents: their own compartment field and their neighbours' counts are
    // updated right away (no decision of this step reads the words or the hub counts); the
    // 2-bit compartment copy, which the decisions read, changes in the push kernel
    if (infected) bump_word(insts[inst].words, i);
    push_rows(insts, inst << 1 | 1, row0, infected ? deg : 0, lane);
    buffer_change(infected, make_int2(inst, (i << 2) | static_cast<int>(kI)), buf, nbuf, L, lane);
    add_decided(valid, inst, scanned, infected ? 1 : 0, infected ? deg : 0, draws, insts, lane);
  }
  flush_changes(buf, nbuf, L, lane);
}

// Counts after the step, key chain, step counter, next step's key, done flag of one
// instance.
__device__ __forceinline__ void finalize_one(abm_sir_instance* __restrict__ I) {
  const int t = I->t;
  if (t >= I->steps) return;
  const int si = I->step_si, ir = I->step_ir;
  I->num_s -= si;
  I->num_i += si - ir;
  I->num_r += ir;
  I->step_si = 0;
  I->step_ir = 0;
  I->counts[3 * t] = I->num_s;
  I->counts[3 * t + 1] = I->num_i;
  I->counts[3 * t + 2] = I->num_r;
  const uint2 r = abm::split_at(make_uint2(I->rng[0], I->rng[1]), 0);
  I->rng[0] = r.x;
  I->rng[1] = r.y;
  I->t = t + 1;
  if (t + 1 < I->steps) {
    const uint2 c = step_key_of(I, t + 1, r);
    I->coll[0] = c.x;
    I->coll[1] = c.y;
  }
  if (t + 1 == I->steps && I->done_flag) {
    __threadfence_system();
    *reinterpret_cast<volatile int32_t*>(I->done_flag) = 1;
  }
}

// The step's finalization of every instance; clears the lists.
__global__ void sir_finalize_kernel(abm_sir_instance* __restrict__ insts, int ninst,
                                    ListHeader* __restrict__ hdr) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0) {
    hdr->changes = 0;
    hdr->cand_s = 0;
  }
  if (k < ninst) finalize_one(insts + k);
}

// Changes of the step after every decision was made: +1 on the 2-bit compartment copy of
// every changed agent; for recoveries (I -> R) also +1 on the agent's own word and -1 on
// its neighbours' infected counts (push_rows, one warp per 32 changes).  Infections were
// pushed by the candidates kernel.
// With few instances (ninst_fused > 0) the last push CTA to finish also finalizes the
// step: each CTA takes a ticket when done, and the CTA holding the last one runs after
// every change was pushed.
__global__ void __launch_bounds__(kSirThreads)
sir_push_kernel(abm_sir_instance* __restrict__ insts, Lists L, int ninst_fused) {
  const int lane = threadIdx.x & 31;
  const int count = min(L.hdr->changes, L.capacity);
  const int threads = gridDim.x * kSirThreads;
  for (int b = (blockIdx.x * kSirThreads + threadIdx.x) & ~31; b < count; b += threads) {
    const int k = b + lane;
    int inst = -1, r0 = 0, len = 0;
    abm_sir_instance* I = insts;
    if (k < count) {
      const int2 ent = __ldcs(&L.changes[k]);
      inst = ent.x;
      const int agent = ent.y >> 2;
      I = insts + inst;
      red_add(I->comp + (agent >> 4), 1u << (2u * static_cast<uint32_t>(agent & 15)));
      if ((ent.y & 3) != static_cast<int>(kI)) {  // a recovery
        bump_word(I->words, agent);
        r0 = __ldcs(I->row_ptr + agent);
        len = __ldcs(I->row_ptr + agent + 1) - r0;
      }
    }
    // slots pushed, summed per instance over the warp's lanes
    if (__any_sync(kFull, len != 0)) {
      const unsigned group = __match_any_sync(kFull, inst);
      const int sum = __reduce_add_sync(group, len);
      if (inst >= 0 && lane == __ffs(group) - 1 && sum)
        red_add(&I->edges_pushed, static_cast<unsigned long long>(sum));
    }
    push_rows(insts, inst >= 0 ? inst << 1 : 0, r0, len, lane);
  }
  if (ninst_fused <= 0) return;
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&L.hdr->push_done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int k = threadIdx.x; k < ninst_fused; k += blockDim.x) finalize_one(insts + k);
  if (threadIdx.x == 0) {
    L.hdr->push_done = 0;
    L.hdr->changes = 0;
    L.hdr->cand_s = 0;
  }
}

// Work items of instances that can still change (t < steps and an infected agent) into the
// compacted work list; instances never come back once they stop, so the list may be
// rebuilt every few steps.  The count is zeroed by the caller.
__global__ void sir_compact_kernel(const abm_sir_instance* __restrict__ insts,
                                   const int4* __restrict__ work, int nwork_max,
                                   const int32_t* __restrict__ live, Lists L) {
  const int lane = threadIdx.x & 31;
  const int nwork = live_count(live, nwork_max);
  const int stride = gridDim.x * blockDim.x;
  for (int b = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; b < nwork; b += stride) {
    const int k = b + lane;
    int4 item = make_int4(0, 0, 0, 0);
    bool keep = false;
    if (k < nwork) {
      item = work[k];
      const abm_sir_instance* I = insts + item.x;
      keep = I->t < I->steps && I->num_i > 0 && item.y < item.z;
    }
    const int pos = warp_append(keep, &L.hdr->live_tiles, lane);
    if (keep) L.live_work[pos] = item;
  }
}

// ---- packing: int8 compartments -> words ---------------------------------------------

__host__ __device__ constexpr int64_t round16(int64_t n) { return (n + 15) & ~static_cast<int64_t>(15); }

// Pass 1, agent (or padding byte) i: compartment and hub mark; padding bytes read as R.
__device__ __forceinline__ int pack_mark(const int8_t* __restrict__ st,
                                         const int32_t* __restrict__ rp, int n,
                                         uint8_t* __restrict__ words, int i,
                                         int32_t* __restrict__ bad) {
  if (i >= n) {
    words[i] = 2;
    return -1;
  }
  const int s = st[i];
  if (s < 0 || s > 2) {
    atomicOr(bad, ABM_SIR_STATUS_BAD_COMPARTMENT);
    words[i] = 2;
    return -1;
  }
  const int deg = rp[i + 1] - rp[i];
  words[i] = static_cast<uint8_t>((deg >= kHubDeg ? (kHubMark << 2) : 0u) | static_cast<uint32_t>(s));
  return s;
}

// Pass 2, agent i: counts its infected neighbours and writes its column entries with the
// hub tag of their target (adj may be col itself; col entries may already carry tags).
// Other threads read this agent's byte meanwhile: only its count bits change, never its
// compartment or hub mark, so every reader sees the same compartment and mark.
__device__ __forceinline__ void pack_count(const int32_t* __restrict__ rp, const int32_t* col,
                                           int32_t* adj, int n, uint8_t* words,
                                           int32_t* __restrict__ hubs, int i,
                                           int32_t* __restrict__ bad) {
  int c = 0;
  for (int k = rp[i]; k < rp[i + 1]; ++k) {
    const uint32_t v = static_cast<uint32_t>(col[k]);
    const uint32_t t = v & kIdx;
    if (t >= static_cast<uint32_t>(n)) {
      // out-of-range column: flagged, and replaced by a self-loop so that no step kernel
      // reads outside the instance
      atomicOr(bad, ABM_SIR_STATUS_BAD_COLUMN);
      adj[k] = static_cast<int32_t>((words[i] >> 2) == kHubMark ? (static_cast<uint32_t>(i) | kTag)
                                                                : static_cast<uint32_t>(i));
      continue;
    }
    const uint32_t w = words[t];
    const uint32_t tagged = (w >> 2) == kHubMark ? (t | kTag) : t;
    if (tagged != v || adj != col) adj[k] = static_cast<int32_t>(tagged);
    c += (w & 3u) == kI;
  }
  const uint32_t own = words[i];
  if ((own >> 2) == kHubMark) hubs[i] = c;
  else words[i] = static_cast<uint8_t>(own | (static_cast<uint32_t>(c) << 2));
}

__global__ void sir_pack_mark_kernel(const int8_t* __restrict__ state,
                                     const int32_t* __restrict__ rp, int n, int npad,
                                     uint8_t* __restrict__ words, int32_t* __restrict__ sizes,
                                     int32_t* __restrict__ bad) {
  __shared__ int sc[3];
  if (threadIdx.x < 3) sc[threadIdx.x] = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < npad) {
    const int s = pack_mark(state, rp, n, words, i, bad);
    if (s >= 0) atomicAdd(&sc[s], 1);
  }
  __syncthreads();
  if (threadIdx.x < 3 && sc[threadIdx.x]) atomicAdd(&sizes[threadIdx.x], sc[threadIdx.x]);
}

__global__ void sir_pack_count_kernel(const int32_t* __restrict__ rp, const int32_t* col,
                                      int32_t* adj, int n, uint8_t* words,
                                      int32_t* __restrict__ hubs, int32_t* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pack_count(rp, col, adj, n, words, hubs, i, bad);
}

// The same over the tiles of many instances (in place: each descriptor's adj holds its
// columns).  The int8 compartments of an instance sit in states8 at the same byte offset
// as its words from words_base.
__global__ void sir_pack_mark_tiles_kernel(const abm_sir_instance* __restrict__ insts,
                                           const int4* __restrict__ work, int nwork,
                                           const int8_t* __restrict__ states8,
                                           const uint8_t* __restrict__ words_base,
                                           int32_t* __restrict__ bad) {
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int4 item = work[w];
    const abm_sir_instance* I = insts + item.x;
    uint8_t* words = I->words;
    const int8_t* st = states8 + (words - words_base);
    const int end = item.z == I->n ? static_cast<int>(round16(I->n)) : item.z;
    for (int i = item.y + threadIdx.x; i < end; i += blockDim.x)
      pack_mark(st, I->row_ptr, I->n, words, i, bad);
  }
}

__global__ void sir_pack_count_tiles_kernel(const abm_sir_instance* __restrict__ insts,
                                            const int4* __restrict__ work, int nwork,
                                            int32_t* __restrict__ bad) {
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int4 item = work[w];
    const abm_sir_instance* I = insts + item.x;
    for (int i = item.y + threadIdx.x; i < item.z; i += blockDim.x)
      pack_count(I->row_ptr, I->adj, I->adj, I->n, I->words, I->hub_counts, i, bad);
  }
}

// Pass 1b, group g of 16 agents: their compartments as 2-bit fields of comp[g] (from the
// bytes of pass 1; padding bytes read as R).
__device__ __forceinline__ void pack_comp_group(const uint8_t* __restrict__ words,
                                                uint32_t* __restrict__ comp, int g) {
  const uint4 v = *reinterpret_cast<const uint4*>(words + 16 * g);
  const uint32_t q[4] = {v.x, v.y, v.z, v.w};
  uint32_t w = 0;
#pragma unroll
  for (int j = 0; j < 16; ++j) w |= ((q[j >> 2] >> (8 * (j & 3))) & 3u) << (2 * j);
  comp[g] = w;
}

__global__ void sir_pack_comp_kernel(const uint8_t* __restrict__ words, int ngroups,
                                     uint32_t* __restrict__ comp) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < ngroups) pack_comp_group(words, comp, g);
}

__global__ void sir_pack_comp_tiles_kernel(const abm_sir_instance* __restrict__ insts,
                                           const int4* __restrict__ work, int nwork) {
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int4 item = work[w];
    const abm_sir_instance* I = insts + item.x;
    const int end = item.z == I->n ? static_cast<int>(round16(I->n)) : item.z;
    for (int g = item.y / 16 + threadIdx.x; g < (end + 15) / 16; g += blockDim.x)
      pack_comp_group(I->words, I->comp, g);
  }
}

// S, I and R totals of every instance from its int8 compartments (the descriptors'
// num_s/num_i/num_r, zeroed by the caller): per tile and CTA in shared memory, then one
// atomic add per compartment.  Compartments outside 0..2 are not counted (the pack reports
// them).
__global__ void sir_count_tiles_kernel(abm_sir_instance* __restrict__ insts,
                                       const int4* __restrict__ work, int nwork,
                                       const int8_t* __restrict__ states8,
                                       const uint8_t* __restrict__ words_base) {
  __shared__ int sc[3];
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    if (threadIdx.x < 3) sc[threadIdx.x] = 0;
    __syncthreads();
    const int4 item = work[w];
    abm_sir_instance* I = insts + item.x;
    const int8_t* st = states8 + (I->words - words_base);
    int c[3] = {0, 0, 0};
    for (int i = item.y + threadIdx.x; i < item.z; i += blockDim.x) {
      const int v = st[i];
      if (v >= 0 && v <= 2) ++c[v];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int tot = __reduce_add_sync(kFull, c[q]);
      if ((threadIdx.x & 31) == 0 && tot) atomicAdd(&sc[q], tot);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (sc[0]) atomicAdd(&I->num_s, sc[0]);
      if (sc[1]) atomicAdd(&I->num_i, sc[1]);
      if (sc[2]) atomicAdd(&I->num_r, sc[2]);
    }
    __syncthreads();  // sc is reset for the next tile
  }
}

__global__ void sir_unpack_kernel(const uint8_t* __restrict__ words, int n,
                                  int8_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = static_cast<int8_t>(words[i] & 3u);
}

// Single-instance descriptor and tile list written on the device, so abm_sir_run makes
// no host-to-device copy and can be captured in a CUDA graph.
__global__ void sir_setup_single_kernel(abm_sir_instance* d, int4* work, int ntiles,
                                        const int32_t* row_ptr, int32_t* adj, uint8_t* words,
                                        int32_t* hubs, uint32_t* comp, int32_t* counts,
                                        const uint32_t* coll_keys, int32_t n, int32_t steps,
                                        float beta, float gamma, const int32_t* sizes) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g == 0) {
    d->row_ptr = row_ptr;
    d->adj = adj;
    d->words = words;
    d->hub_counts = hubs;
    d->comp = comp;
    d->counts = counts;
    d->done_flag = nullptr;
    d->coll_keys = coll_keys;
    d->rng[0] = 0;
    d->rng[1] = 0;
    d->n = n;
    d->t = 0;
    d->steps = steps;
    d->beta = beta;
    d->gamma = gamma;
    d->num_s = sizes[0];
    d->num_i = sizes[1];
    d->num_r = sizes[2];
    d->step_si = 0;
    d->step_ir = 0;
    d->edges_scanned = 0;
    d->edges_pushed = 0;
    d->candidates = 0;
    d->coll[0] = 0;
    d->coll[1] = 0;
  }
  for (int b = g; b < ntiles; b += gridDim.x * blockDim.x) {
    const int begin = b * kTile;
    const int end = min(begin + kTile, n);
    work[b] = make_int4(0, begin, end, 0);
  }
}

// ---- Resident path: one CTA per instance, all of its steps, words in shared memory ------
//
// Instances are independent, so a CTA takes one instance at a time (in the caller's
// order, from a queue counter) and runs all of its steps with the instance's words in
// shared memory: the sweep reads them there, decisions read the neighbours' compartments
// there, and count updates are shared-memory atomics.  Only CSR rows, row offsets and hub
// counts come from global memory, and the row offsets of a member whose words leave room
// for them are staged in shared memory too.  A step is three phases separated by
// __syncthreads:
//   sweep     warp w takes the 1024-agent chunks w, w + 16, ... of the words and appends
//             the susceptible agents with infected neighbours (and every susceptible hub,
//             whose count only its decision reads) and the infected agents to two lists
//             (their first entries in shared memory after the words, as many as fit
//             without lowering the CTAs per SM; the rest in the CTA's global scratch,
//             L2-resident).
//   decide    warps take paired rounds from a round counter, so that every warp has work
//             however small the instance: per lane one susceptible agent (rows longer
//             than 32 slots by the whole warp) and one infected agent's recovery draw;
//             the recovery chain and the susceptible agent's key derivation run while its
//             row is in flight.  Changes go to the CTA's change list.  Nothing is written
//             to the words, so every decision sees the pre-step states.
//   apply     warps take groups of 32 changes: +1 on each changed agent's compartment
//             field and +-1 on its neighbours' counts (push of the concatenated rows);
//             meanwhile thread 0 records the step's S/I/R counts and advances the keys.
// In steps with more rounds than warps, rounds are taken two ahead, so that the list
// entries and row offsets of the next rounds are in flight while one is decided.  Draws compare the 23 random mantissa bits
// with an integer threshold, which equals the float comparison of jax.random.uniform.
// An instance at step 0 may build its words in the kernel from the int8 compartments
// (hub marks, column hub tags, initial counts) instead of reading packed words.  The
// words are written back, with the 2-bit compartment copy, when the instance's steps of
// the call are done.
// The host orders the members longest first by a predicted device time; the order never
// changes results.  No CTA waits on another; the results equal the grid path's (integer
// atomics commute).
constexpr int kResThreads = 512;
constexpr int kResChunk = 1024;  // agents per warp chunk, 32 per lane

struct ResState {
  int inst;        // queue position taken by the CTA
  int next_round;  // round counter of the step's decisions
  int next_group;  // group counter of the step's count updates
  int ns, ni;      // entries in the candidate and infected lists
  int nchanges;    // entries in the change list
  int si, ir;      // transitions of the step
  int num_s, num_i, num_r;
  uint32_t rng0, rng1, coll0, coll1;
  unsigned long long scanned, pushed, cands, draws;
  uint32_t st_scanned, st_pushed, st_cands, st_draws;  // this step's, folded by thread 0
};

// First lane whose inclusive prefix sum `incl` exceeds f (f below the warp total), by a
// five-step binary search over the lanes; called by all lanes.
__device__ __forceinline__ int owner_lane(int incl, int f) {
  int lo = 0;
#pragma unroll
  for (int st = 16; st > 0; st >>= 1) {
    const int p = __shfl_sync(kFull, incl, lo + st - 1);
    if (p <= f) lo += st;
  }
  return lo;
}

__device__ __forceinline__ int warp_inclusive_sum(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// +v (already shifted into place) on the aligned 32-bit word of shared memory holding
// byte i of the words.
__device__ __forceinline__ void sw_add(uint8_t* sw, int i, uint32_t v) {
  atomicAdd(reinterpret_cast<uint32_t*>(sw + (i & ~3)), v << (8u * static_cast<uint32_t>(i & 3)));
}

// Count updates of up to 32 rows of one instance, one per lane (len 0: none; up: +1,
// else -1), by the whole warp over the concatenated rows, kResPushPasses passes in flight
// (six here, four on the grid path: each measured best on its path).
constexpr int kResPushPasses = 6;
// A column with the hub tag sends its update to hub_counts.  Columns are within the
// instance (checked when its words are built).
__device__ __forceinline__ void push_rows_shared(const int32_t* __restrict__ adj, uint8_t* sw,
                                                 int32_t* hubs, bool up, int row0, int len,
                                                 int lane) {
  const int incl = warp_inclusive_sum(len, lane);
  const int total = __shfl_sync(kFull, incl, 31);
  const int shift = row0 - (incl - len);
  const int sign = up ? 1 : 0;
  for (int base = 0; base < total; base += 32 * kResPushPasses) {
    uint32_t v[kResPushPasses];
    int d[kResPushPasses];
#pragma unroll
    for (int u = 0; u < kResPushPasses; ++u) {
      const int f = base + 32 * u + lane;
      const int lo = owner_lane(incl, f);
      const int sh = __shfl_sync(kFull, shift, lo);
      d[u] = __shfl_sync(kFull, sign, lo) ? 1 : -1;
      v[u] = f < total ? ld_col(adj, f + sh) : 0u;
    }
#pragma unroll
    for (int u = 0; u < kResPushPasses; ++u) {
      if (base + 32 * u + lane < total) {
        const uint32_t t = v[u] & kIdx;
        if (v[u] & kTag) red_add(hubs + t, d[u]);
        else sw_add(sw, static_cast<int>(t), static_cast<uint32_t>(4 * d[u]));
      }
    }
  }
}

// Entry k of a CTA list: the first scap entries are in shared memory (sl), the rest in the
// CTA's global list (gl, indexed from 0 like the shared part; streaming stores and loads,
// which leave the small L1 to row offsets and columns).
__device__ __forceinline__ void list_put(uint32_t* sl, uint32_t* gl, int scap, int k, uint32_t v) {
  if (k < scap) sl[k] = v;
  else __stcs(gl + k, v);
}
__device__ __forceinline__ uint32_t list_get(const uint32_t* sl, const uint32_t* gl, int scap,
                                             int k) {
  return k < scap ? sl[k] : __ldcs(gl + k);
}

// Appends (agent << 2 | new compartment) of the round's changes to the change list, the
// recoveries (lanes with rec, agent ei) then the infections (lanes with inf, agent e),
// with one counter atomic per warp.
__device__ __forceinline__ void res_record(bool rec, int ei, bool inf, int e, uint32_t* s_changes,
                                           uint32_t* changes, int scap, int* count, int lane) {
  const unsigned m1 = __ballot_sync(kFull, rec), m2 = __ballot_sync(kFull, inf);
  if (!(m1 | m2)) return;
  const int c1 = __popc(m1);
  int at = 0;
  if (lane == 0) at = atomicAdd(count, c1 + __popc(m2));
  at = __shfl_sync(kFull, at, 0);
  const unsigned below = (1u << lane) - 1u;
  if (rec)
    list_put(s_changes, changes, scap, at + __popc(m1 & below), (static_cast<uint32_t>(ei) << 2) | 2u);
  if (inf)
    list_put(s_changes, changes, scap, at + c1 + __popc(m2 & below),
             (static_cast<uint32_t>(e) << 2) | kI);
}

__global__ void __launch_bounds__(kResThreads, 2)
sir_resident_kernel(abm_sir_instance* __restrict__ insts, int ninst,
                    const int32_t* __restrict__ order, int nsteps, int max_bytes,
                    const int8_t* __restrict__ states8, const uint8_t* words_base,
                    int32_t* __restrict__ queue, uint32_t* __restrict__ lists, int cap,
                    int scap, int32_t* __restrict__ status) {
  extern __shared__ __align__(16) uint8_t sw[];
  __shared__ ResState S;
  const int lane = threadIdx.x & 31;
  // this CTA's lists: changes, susceptible candidates, infected agents (cap entries each);
  // the first scap entries of each are kept in shared memory after the words
  uint32_t* __restrict__ changes = lists + static_cast<size_t>(blockIdx.x) * 3 * cap;
  uint32_t* __restrict__ slist = changes + cap;
  uint32_t* __restrict__ ilist = slist + cap;
  uint32_t* s_changes = reinterpret_cast<uint32_t*>(sw + max_bytes);
  uint32_t* s_slist = s_changes + scap;
  uint32_t* s_ilist = s_slist + scap;
  for (;;) {
    if (threadIdx.x == 0) S.inst = atomicAdd(queue, 1);
    __syncthreads();
    const int q = S.inst;
    __syncthreads();  // every thread holds q before S is rewritten
    if (q >= ninst) break;
    abm_sir_instance* I = insts + (order != nullptr ? order[q] : q);
    const int n = I->n;
    const int npad = static_cast<int>(round16(n));
    const int t_begin = I->t;
    const int t_end = min(I->steps, t_begin + nsteps);
    if (t_begin >= t_end) continue;  // uniform
    if (npad > max_bytes || n > cap) {
      if (threadIdx.x == 0) atomicOr(status, ABM_SIR_STATUS_OVERSIZE);
      continue;
    }
    const int32_t* __restrict__ rp = I->row_ptr;
    int32_t* __restrict__ adj = I->adj;
    int32_t* hubs = I->hub_counts;
    const uint32_t tbeta = abm::unit_threshold(I->beta), tgamma = abm::unit_threshold(I->gamma);
    if (states8 != nullptr && t_begin == 0) {
      // words built here from the int8 compartments: compartment, hub mark (degree >=
      // 63, whose count starts at 0 in hub_counts), the columns' hub tags, then every
      // infected agent adds one to its neighbours' counts
      // (each loop keeps several independent loads per thread in flight)
      const int8_t* __restrict__ st = states8 + (I->words - words_base);
      constexpr int kWordsIn = 4, kColsIn = 8;
      for (int k0 = threadIdx.x; k0 < npad; k0 += kResThreads * kWordsIn) {
        int c[kWordsIn], a[kWordsIn], e[kWordsIn];
#pragma unroll
        for (int u = 0; u < kWordsIn; ++u) {
          const int k = k0 + kResThreads * u;
          c[u] = 2;
          a[u] = e[u] = 0;
          if (k < n) {
            c[u] = st[k];
            a[u] = __ldg(rp + k);
            e[u] = __ldg(rp + k + 1);
          }
        }
#pragma unroll
        for (int u = 0; u < kWordsIn; ++u) {
          const int k = k0 + kResThreads * u;
          if (k >= npad) continue;
          uint32_t w = 2u;  // padding: R
          if (k < n) {
            int cc = c[u];
            if (cc < 0 || cc > 2) {
              atomicOr(status, ABM_SIR_STATUS_BAD_COMPARTMENT);
              cc = 2;
            }
            w = static_cast<uint32_t>(cc);
            if (e[u] - a[u] >= kHubDeg) {
              w |= kHubMark << 2;
              hubs[k] = 0;
            }
          }
          sw[k] = static_cast<uint8_t>(w);
        }
      }
      __syncthreads();
      // hub tags on the columns (bit 31 where the neighbour is a hub), in place; a column
      // outside 0..n-1 is flagged and replaced by a self-loop, as abm_sir_pack does, so that
      // no step reads outside the instance
      const int nslots = __ldg(rp + n);
      for (int k0 = threadIdx.x; k0 < nslots; k0 += kResThreads * kColsIn) {
        uint32_t v[kColsIn];
#pragma unroll
        for (int u = 0; u < kColsIn; ++u) {
          const int k = k0 + kResThreads * u;
          v[u] = k < nslots ? static_cast<uint32_t>(adj[k]) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kColsIn; ++u) {
          const int k = k0 + kResThreads * u;
          if (k >= nslots) continue;
          uint32_t t = v[u] & kIdx;
          if (t >= static_cast<uint32_t>(n)) {
            atomicOr(status, ABM_SIR_STATUS_BAD_COLUMN);
            int lo = 0, hi = n - 1;  // the row holding slot k: last i with rp[i] <= k
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (__ldg(rp + mid) <= k) lo = mid;
              else hi = mid - 1;
            }
            t = static_cast<uint32_t>(lo);
          }
          const uint32_t want = (sw[t] >> 2) == kHubMark ? (t | kTag) : t;
          if (want != v[u]) adj[k] = static_cast<int32_t>(want);
        }
      }
      __syncthreads();
      for (int b = threadIdx.x & ~31; b < n; b += kResThreads) {
        const int k = b + lane;
        const bool inf = k < n && (sw[k] & 3u) == kI;
        if (!__any_sync(kFull, inf)) continue;  // uniform: no infected agent here
        int r0 = 0, len = 0;
        if (inf) {
          r0 = __ldg(rp + k);
          len = __ldg(rp + k + 1) - r0;
        }
        push_rows_shared(adj, sw, hubs, true, r0, len, lane);
      }
    } else {
      for (int k = threadIdx.x; k < npad / 16; k += kResThreads)
        reinterpret_cast<uint4*>(sw)[k] = reinterpret_cast<const uint4*>(I->words)[k];
    }
    // row offsets staged in shared memory after the words where they fit (the smaller
    // members of a batch): the row lookups of every step are then shared-memory loads
    const bool staged = npad + 4 * (n + 1) <= max_bytes;
    const int32_t* srp = reinterpret_cast<const int32_t*>(sw + npad);
    if (staged) {
      for (int k0 = threadIdx.x; k0 <= n; k0 += 4 * kResThreads) {
        int32_t v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = k0 + kResThreads * u;
          v[u] = k <= n ? __ldg(rp + k) : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = k0 + kResThreads * u;
          if (k <= n) reinterpret_cast<int32_t*>(sw + npad)[k] = v[u];
        }
      }
    }
    // (row offsets not staged are read through L1: neighbouring entries share lines)
    auto row_at = [&](int k) { return staged ? srp[k] : __ldca(rp + k); };
    if (threadIdx.x == 0) {
      const uint2 rng = make_uint2(I->rng[0], I->rng[1]);
      const uint2 c = step_key_of(I, t_begin, rng);
      S.rng0 = rng.x;
      S.rng1 = rng.y;
      S.coll0 = c.x;
      S.coll1 = c.y;
      S.num_s = I->num_s;
      S.num_i = I->num_i;
      S.num_r = I->num_r;
      S.si = S.ir = 0;
      S.ns = S.ni = 0;
      S.nchanges = 0;
      S.next_round = S.next_group = 0;
      S.scanned = S.pushed = S.cands = S.draws = 0;
      S.st_scanned = S.st_pushed = S.st_cands = S.st_draws = 0;
    }
    __syncthreads();
    const int nchunks = (n + kResChunk - 1) / kResChunk;
    int t = t_begin;
    for (; t < t_end; ++t) {
      if (S.num_i == 0) break;  // uniform: nothing can change any more
      // counters of the previous step's apply, free since its closing barrier
      if (threadIdx.x == 0) {
        S.nchanges = 0;
        S.next_group = 0;
        S.pushed += S.st_pushed;
        S.st_pushed = 0;
      }
      // ---- sweep: lists of susceptible agents with infected neighbours, infected agents
      int my_cands = 0;
      for (int c = static_cast<int>(threadIdx.x >> 5); c < nchunks; c += kResThreads / 32) {
        const int base = c * kResChunk + 32 * lane;
        uint32_t qw[8];
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          if (base + 16 * v + 16 <= npad) {
            const uint4 x = *reinterpret_cast<const uint4*>(sw + base + 16 * v);
            qw[4 * v] = x.x;
            qw[4 * v + 1] = x.y;
            qw[4 * v + 2] = x.z;
            qw[4 * v + 3] = x.w;
          } else {
#pragma unroll
            for (int z = 0; z < 4; ++z) qw[4 * v + z] = 0x02020202u;  // beyond the agents: R
          }
        }
        // every susceptible hub is listed (its count is read by its decision, which scans
        // nothing when the count is 0): cheaper here than reading the hub counts
        unsigned need_s, need_i, hub_s;
        sweep_flags(qw, need_s, need_i, hub_s);
        const int ms = __popc(need_s), mi = __popc(need_i);
        my_cands += ms + mi;
        // one list position per agent: warp prefix sums, one counter atomic per warp
        const int both = ms | (mi << 16);
        const int incl = warp_inclusive_sum(both, lane);
        const int total = __shfl_sync(kFull, incl, 31);
        int bs = 0, bi = 0;
        if (lane == 31) {
          if (total & 0xFFFF) bs = atomicAdd(&S.ns, total & 0xFFFF);
          if (total >> 16) bi = atomicAdd(&S.ni, total >> 16);
        }
        bs = __shfl_sync(kFull, bs, 31) + ((incl - both) & 0xFFFF);
        bi = __shfl_sync(kFull, bi, 31) + ((incl - both) >> 16);
        for (unsigned m = need_s; m; m &= m - 1) list_put(s_slist, slist, scap, bs++, base + __ffs(m) - 1);
        for (unsigned m = need_i; m; m &= m - 1) list_put(s_ilist, ilist, scap, bi++, base + __ffs(m) - 1);
      }
      my_cands = __reduce_add_sync(kFull, my_cands);
      if (lane == 0 && my_cands) atomicAdd(&S.st_cands, static_cast<uint32_t>(my_cands));
      __syncthreads();
      // ---- decide: paired rounds taken from a round counter -----------------------------
      // Round p holds susceptible entries 32p..32p+31 and infected entries 32p..32p+31, one
      // of each per lane: the infected entry's recovery chain and the susceptible entry's
      // key derivation run while its row is in flight.  Entries are loaded two rounds ahead
      // and row offsets one round ahead.
      const uint2 coll = make_uint2(S.coll0, S.coll1);
      const int ns = S.ns, ni = S.ni;
      const int rounds = max((ns + 31) >> 5, (ni + 31) >> 5);
      int my_scanned = 0;
      int my_si = 0, my_ir = 0, my_draws = 0;
      auto take = [&]() {
        int r = 0;
        if (lane == 0) r = atomicAdd(&S.next_round, 1);
        return __shfl_sync(kFull, r, 0);
      };
      auto s_entry = [&](int r) {
        const int f = 32 * r + lane;
        return r < rounds && f < ns ? static_cast<int>(list_get(s_slist, slist, scap, f)) : -1;
      };
      auto i_entry = [&](int r) {
        const int f = 32 * r + lane;
        return r < rounds && f < ni ? static_cast<int>(list_get(s_ilist, ilist, scap, f)) : -1;
      };
      // rounds are taken one ahead only when there are more rounds than warps: with fewer,
      // a warp holding two rounds would leave another warp without one.  Without taking
      // ahead each warp takes exactly one round index (0..15 over the 16 warps), which
      // covers every round only because the threshold is the warp count.
      const bool ahead = rounds > kResThreads / 32;
      int r_cur = take(), r_nxt = ahead ? take() : rounds;
      int es_cur = s_entry(r_cur), ei_cur = i_entry(r_cur);
      int es_nxt = s_entry(r_nxt), ei_nxt = i_entry(r_nxt);
      int a_cur = 0, b_cur = 0;
      if (es_cur >= 0) {
        a_cur = row_at(es_cur);
        b_cur = row_at(es_cur + 1);
      }
      while (r_cur < rounds) {
        const int e = es_cur, ei = ei_cur;
        const int ra = a_cur, rb = b_cur;
        a_cur = b_cur = 0;
        if (es_nxt >= 0) {
          a_cur = row_at(es_nxt);
          b_cur = row_at(es_nxt + 1);
        }
        r_cur = r_nxt;
        es_cur = es_nxt;
        ei_cur = ei_nxt;
        r_nxt = ahead ? take() : rounds;
        es_nxt = s_entry(r_nxt);
        ei_nxt = i_entry(r_nxt);
        // susceptible entry (a susceptible agent with infected neighbours): the first
        // columns of its row are loaded before the draw chains below
        const bool valid = e >= 0;
        const int row0 = ra, deg = valid ? rb - ra : 0;
        int cnt = 0, scanned = 0;
        bool infected = false;
        const bool heavy = deg > kHeavyDeg;
        unsigned imask = 0;
        int nb[kResScan];
#pragma unroll
        for (int z = 0; z < kResScan; ++z)
          nb[z] = !heavy && z < deg ? static_cast<int>(ld_col(adj, row0 + z) & kIdx) : -1;
        // infected entry: recovery draw
        bool rec = false;
        if (ei >= 0) {
          const uint2 krec = abm::split_at(abm::split_at(coll, (uint64_t)ei), 1);
          rec = abm::unit_below(abm::bits_at(krec, 0), tgamma);
        }
        my_ir += rec;
        uint2 kinf = make_uint2(0, 0);
        if (valid) {
          kinf = abm::split_at(abm::split_at(coll, (uint64_t)e), 0);
          // infected neighbours: the word's count, or a hub's count in global memory
          // (exact since the last apply; read through L2)
          cnt = static_cast<int>(sw[e] >> 2);
          if (cnt == static_cast<int>(kHubMark)) cnt = __ldcg(hubs + e);
          if (!heavy) {
            int seen = 0;
#pragma unroll
            for (int z = 0; z < kResScan; ++z) {
              const bool inf = nb[z] >= 0 && (sw[nb[z]] & 3u) == kI;
              imask |= static_cast<unsigned>(inf) << z;
              seen += inf;
            }
            int k1 = kResScan;
            for (; k1 < deg && seen < cnt; k1 += kResScan) {
#pragma unroll
              for (int z = 0; z < kResScan; ++z)
                nb[z] = k1 + z < deg ? static_cast<int>(ld_col(adj, row0 + k1 + z) & kIdx) : -1;
#pragma unroll
              for (int z = 0; z < kResScan; ++z) {
                const bool inf = nb[z] >= 0 && (sw[nb[z]] & 3u) == kI;
                // slots past the row (k1 + z may reach 34 for a 32-slot row) are never
                // infected; the mask keeps their shift defined
                imask |= static_cast<unsigned>(inf) << ((k1 + z) & 31);
                seen += inf;
              }
            }
            scanned = min(k1, deg);
          }
        }
        // draws at the infected slots in row order, one per pass; the first that fires
        // infects (the outcome is the OR over the slots, the count is the sequential one)
        while (__any_sync(kFull, imask != 0)) {
          if (imask) {
            const int s1 = __ffs(imask) - 1;
            imask &= imask - 1;
            const bool f1 = abm::unit_below(abm::bits_at(kinf, (uint64_t)s1), tbeta);
            ++my_draws;
            if (f1) {
              infected = true;
              imask = 0;
            }
          }
        }
        unsigned hmask = __ballot_sync(kFull, heavy);
        while (hmask) {
          const int src = __ffs(hmask) - 1;
          hmask &= hmask - 1;
          const int hrow = __shfl_sync(kFull, row0, src);
          const int hdeg = __shfl_sync(kFull, deg, src);
          int remaining = __shfl_sync(kFull, cnt, src);
          const uint2 hk = make_uint2(__shfl_sync(kFull, kinf.x, src),
                                      __shfl_sync(kFull, kinf.y, src));
          // the whole row is scanned (the warp reads 32 x kResHeavyUnroll columns per pass
          // and draws only at infected slots): on the resident kernel this beats drawing
          // at every slot first, which the grid path does for rows longer than
          // kDrawFirstDeg
          bool fired = false;
          int cpos = 0;
          for (; cpos < hdeg && !fired && remaining > 0; cpos += 32 * kResHeavyUnroll) {
            uint32_t wv[kResHeavyUnroll];
#pragma unroll
            for (int u = 0; u < kResHeavyUnroll; ++u) {
              const int slot = cpos + 32 * u + lane;
              wv[u] = slot < hdeg ? ld_col(adj, hrow + slot) : kTag;
            }
            bool hit = false;
            int seen = 0;
#pragma unroll
            for (int u = 0; u < kResHeavyUnroll; ++u) {
              const int slot = cpos + 32 * u + lane;
              if (slot < hdeg && (sw[wv[u] & kIdx] & 3u) == kI) {
                ++seen;
                if (!hit) {
                  ++my_draws;
                  hit = abm::unit_below(abm::bits_at(hk, (uint64_t)slot), tbeta);
                }
              }
            }
            fired = __any_sync(kFull, hit);
            remaining -= __reduce_add_sync(kFull, seen);
          }
          if (lane == src) {
            infected = fired;
            scanned = min(cpos, hdeg);
          }
        }
        my_scanned += scanned;
        my_si += infected;
        res_record(rec, ei, infected, e, s_changes, changes, scap, &S.nchanges, lane);
      }
      my_si = __reduce_add_sync(kFull, my_si);
      my_ir = __reduce_add_sync(kFull, my_ir);
      my_draws = __reduce_add_sync(kFull, my_draws);
      my_scanned = __reduce_add_sync(kFull, my_scanned);
      if (lane == 0) {
        if (my_si) atomicAdd(&S.si, my_si);
        if (my_ir) atomicAdd(&S.ir, my_ir);
        if (my_scanned) atomicAdd(&S.st_scanned, static_cast<uint32_t>(my_scanned));
        if (my_draws) atomicAdd(&S.st_draws, static_cast<uint32_t>(my_draws));
      }
      __syncthreads();
      // ---- apply: groups of 32 changes, taken from a group counter ------------------------
      const int nch = S.nchanges;
      const int groups = (nch + 31) >> 5;
      // the step's counts and the next step's keys, by thread 0 while the warps apply (every
      // field written here was last read before the barrier above; the step loop reads
      // num_i after the closing barrier)
      if (threadIdx.x == 0) {
        const int si = S.si, ir = S.ir;
        S.num_s -= si;
        S.num_i += si - ir;
        S.num_r += ir;
        I->counts[3 * t] = S.num_s;
        I->counts[3 * t + 1] = S.num_i;
        I->counts[3 * t + 2] = S.num_r;
        S.si = S.ir = 0;
        S.ns = S.ni = 0;
        S.next_round = 0;
        S.scanned += S.st_scanned;
        S.cands += S.st_cands;
        S.draws += S.st_draws;
        S.st_scanned = S.st_cands = S.st_draws = 0;
        const uint2 next_rng = abm::split_at(make_uint2(S.rng0, S.rng1), 0);
        uint2 next_coll = make_uint2(0, 0);
        if (t + 1 < I->steps) next_coll = step_key_of(I, t + 1, next_rng);
        S.rng0 = next_rng.x;
        S.rng1 = next_rng.y;
        S.coll0 = next_coll.x;
        S.coll1 = next_coll.y;
      }
      int my_pushed = 0;
      for (;;) {
        int g = 0;
        if (lane == 0) g = atomicAdd(&S.next_group, 1);
        g = __shfl_sync(kFull, g, 0);
        if (g >= groups) break;
        const int k = 32 * g + lane;
        int r0 = 0, len = 0;
        bool up = false;
        if (k < nch) {
          const uint32_t e = list_get(s_changes, changes, scap, k);
          const int a = static_cast<int>(e >> 2);
          sw_add(sw, a, 1u);
          up = (e & 3u) == kI;
          r0 = row_at(a);
          len = row_at(a + 1) - r0;
        }
        my_pushed += len;
        push_rows_shared(adj, sw, hubs, up, r0, len, lane);
      }
      my_pushed = __reduce_add_sync(kFull, my_pushed);
      if (lane == 0 && my_pushed) atomicAdd(&S.st_pushed, static_cast<uint32_t>(my_pushed));
      __syncthreads();
    }
    // steps without an infected agent: constant counts, the key chain still advances
    for (int u = t + static_cast<int>(threadIdx.x); u < t_end; u += kResThreads) {
      I->counts[3 * u] = S.num_s;
      I->counts[3 * u + 1] = S.num_i;
      I->counts[3 * u + 2] = S.num_r;
    }
    if (threadIdx.x == 0 && t < t_end) {
      uint2 r = make_uint2(S.rng0, S.rng1);
      for (int u = t; u < t_end; ++u) r = abm::split_at(r, 0);
      S.rng0 = r.x;
      S.rng1 = r.y;
      if (t_end < I->steps) {
        const uint2 c = step_key_of(I, t_end, r);
        S.coll0 = c.x;
        S.coll1 = c.y;
      }
    }
    // write back: words, the 2-bit compartment copy, the descriptor
    for (int k = threadIdx.x; k < npad / 16; k += kResThreads) {
      const uint4 x = reinterpret_cast<const uint4*>(sw)[k];
      reinterpret_cast<uint4*>(I->words)[k] = x;
      const uint32_t w4[4] = {x.x, x.y, x.z, x.w};
      uint32_t packed = 0;
#pragma unroll
      for (int j = 0; j < 16; ++j) packed |= ((w4[j >> 2] >> (8 * (j & 3))) & 3u) << (2 * j);
      I->comp[k] = packed;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      I->t = t_end;
      I->rng[0] = S.rng0;
      I->rng[1] = S.rng1;
      I->coll[0] = S.coll0;
      I->coll[1] = S.coll1;
      I->num_s = S.num_s;
      I->num_i = S.num_i;
      I->num_r = S.num_r;
      I->step_si = 0;
      I->step_ir = 0;
      I->edges_scanned += S.scanned;
      I->edges_pushed += S.pushed + S.st_pushed;
      I->candidates += S.cands;
      I->draws += S.draws;
      if (t_end == I->steps && I->done_flag) {
        __threadfence_system();
        *reinterpret_cast<volatile int32_t*>(I->done_flag) = 1;
      }
    }
    __syncthreads();  // the words in shared memory are rewritten by the next instance
  }
}

// Segment k of the table is copied by CTA k (grid-stride over segments): head bytes up to
// a 16-byte boundary, 16-byte vectors, tail bytes when source and destination share their
// address mod 16, else 4-byte words when they share it mod 4, else bytes.
__global__ void copy_segments_kernel(const abm_copy_segment* __restrict__ segs, int64_t count) {
  for (int64_t k = blockIdx.x; k < count; k += gridDim.x) {
    uint8_t* d = static_cast<uint8_t*>(segs[k].dst);
    const uint8_t* s = static_cast<const uint8_t*>(segs[k].src);
    const uint64_t n = segs[k].bytes;
    const uintptr_t da = reinterpret_cast<uintptr_t>(d), sa = reinterpret_cast<uintptr_t>(s);
    if ((da & 15) == (sa & 15)) {
      uint64_t head = (16 - (da & 15)) & 15;
      if (head > n) head = n;
      for (uint64_t i = threadIdx.x; i < head; i += blockDim.x) d[i] = s[i];
      const uint64_t nv = (n - head) / 16;
      const uint4* sv = reinterpret_cast<const uint4*>(s + head);
      uint4* dv = reinterpret_cast<uint4*>(d + head);
      for (uint64_t i = threadIdx.x; i < nv; i += blockDim.x) dv[i] = sv[i];
      for (uint64_t i = head + nv * 16 + threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    } else if ((da & 3) == (sa & 3)) {
      uint64_t head = (4 - (da & 3)) & 3;
      if (head > n) head = n;
      for (uint64_t i = threadIdx.x; i < head; i += blockDim.x) d[i] = s[i];
      const uint64_t nw = (n - head) / 4;
      const uint32_t* sw4 = reinterpret_cast<const uint32_t*>(s + head);
      uint32_t* dw4 = reinterpret_cast<uint32_t*>(d + head);
      for (uint64_t i = threadIdx.x; i < nw; i += blockDim.x) dw4[i] = sw4[i];
      for (uint64_t i = head + nw * 4 + threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    } else {
      for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    }
  }
}

int default_grid(int nwork) {
  const int cap = abm_host::sm_count() * 8;  // 8 resident 256-thread CTAs per SM
  return nwork < cap ? (nwork > 0 ? nwork : 1) : cap;
}

// Persistent grid of a kernel: as many CTAs as can be resident at once.
template <typename Kernel>
int resident_grid(Kernel k, int fallback_per_sm) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kSirThreads, 0) != cudaSuccess ||
      per_sm <= 0)
    per_sm = fallback_per_sm;
  return abm_host::sm_count() * per_sm;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

size_t work_list_bytes(int64_t max_tiles) { return align256((size_t)max_tiles * sizeof(int4)); }

Lists carve_lists(void* ws, size_t bytes, int64_t max_tiles) {
  Lists L;
  L.hdr = static_cast<ListHeader*>(ws);
  const size_t wl = work_list_bytes(max_tiles);
  const size_t end = (bytes / 256) * 256;  // the work list ends here
  size_t cap = (end - wl - sizeof(ListHeader)) / (2 * sizeof(int2));
  if (cap > 0x7FFFFFFE) cap = 0x7FFFFFFE;
  L.capacity = (int)cap;
  L.changes = reinterpret_cast<int2*>(L.hdr + 1);
  L.cands = L.changes + L.capacity;
  L.live_work = reinterpret_cast<int4*>(static_cast<char*>(ws) + end - wl);
  return L;
}

// Entries of each CTA list kept in shared memory after the words (at most kResListShared,
// a multiple of 32): what is left of the SM's shared memory once the CTAs per SM that the
// words allow have their words, static shared memory and per-block reservation, less a
// slack for the allocation granularity.  0 when nothing is left or a query fails.  The
// opt-in must already cover `bytes`.
constexpr int kResListShared = 2048;

int res_list_cap(int bytes) {
  int dev = 0, smem_sm = 0, reserved = 0, per_sm = 0;
  cudaFuncAttributes fa;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) !=
          cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) !=
          cudaSuccess ||
      cudaFuncGetAttributes(&fa, sir_resident_kernel) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sir_resident_kernel, kResThreads,
                                                    bytes) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (per_sm <= 0) return 0;
  const int64_t room = static_cast<int64_t>(smem_sm / per_sm) - reserved -
                       static_cast<int64_t>(fa.sharedSizeBytes) - bytes - 256;
  if (room < 12 * 32) return 0;
  return static_cast<int>(std::min<int64_t>(kResListShared, room / 12) & ~int64_t{31});
}


}  // namespace

extern "C" {

size_t abm_sir_instance_size(void) { return sizeof(abm_sir_instance); }

int32_t abm_sir_tile_agents(void) { return kTile; }

int32_t abm_sir_hub_degree(void) { return kHubDeg; }

int abm_sir_default_launch(abm_sir_launch* out) {
  if (!out) return ABM_ERR_BADARG;
  out->sweep_grid = resident_grid(sir_sweep_kernel, 4);
  out->candidates_grid = resident_grid(sir_candidates_kernel, 4);
  out->push_grid = resident_grid(sir_push_kernel, 4);
  out->reserved = 0;
  return ABM_OK;
}

int32_t abm_sir_resident_max_agents(void) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, sir_resident_kernel) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int64_t room = static_cast<int64_t>(optin) - static_cast<int64_t>(fa.sharedSizeBytes);
  return room > 0 ? static_cast<int32_t>(room & ~static_cast<int64_t>(15)) : 0;
}

int32_t abm_sir_resident_grid(int32_t max_agents) {
  if (max_agents <= 0 || max_agents > abm_sir_resident_max_agents()) return 0;
  const int bytes = static_cast<int>(round16(max_agents));
  // the opt-in only ever grows, so launches (and captured graphs) of larger batches stay
  // valid after a smaller batch asked for its grid
  auto raise_optin = [](int want) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, sir_resident_kernel) != cudaSuccess) return false;
    return fa.maxDynamicSharedSizeBytes >= want ||
           cudaFuncSetAttribute(sir_resident_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                want) == cudaSuccess;
  };
  if (!raise_optin(bytes)) {
    cudaGetLastError();
    return 0;
  }
  // then room for the shared list heads (sized not to lower the CTAs per SM)
  const int smem = bytes + 12 * res_list_cap(bytes);
  if (!raise_optin(smem)) {
    cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sir_resident_kernel, kResThreads,
                                                    smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm * abm_host::sm_count();
}

size_t abm_sir_resident_scratch_bytes(int32_t max_agents, int32_t grid) {
  if (max_agents <= 0 || grid <= 0) return 0;
  return 256 + static_cast<size_t>(grid) * static_cast<size_t>(round16(max_agents)) * 12;
}

int abm_sir_steps_resident(abm_sir_instance* insts, int32_t ninst, const int32_t* order,
                           int32_t max_agents, int32_t nsteps, int32_t grid,
                           const int8_t* states8, const uint8_t* words_base, void* scratch,
                           size_t scratch_bytes, int32_t* status, void* stream) {
  if (!insts || ninst <= 0 || max_agents <= 0 || nsteps < 0 || grid <= 0 || !scratch || !status)
    return ABM_ERR_BADARG;
  if ((states8 == nullptr) != (words_base == nullptr)) return ABM_ERR_BADARG;
  if (!abm_host::aligned(insts, 8) || !abm_host::aligned(scratch, 256) ||
      (order && !abm_host::aligned(order, 4)) || !abm_host::aligned(status, 4))
    return ABM_ERR_BADARG;
  if (scratch_bytes < abm_sir_resident_scratch_bytes(max_agents, grid)) return ABM_ERR_WORKSPACE;
  if (nsteps == 0) return ABM_OK;
  cudaStream_t s = abm_host::as_stream(stream);
  const int bytes = static_cast<int>(round16(max_agents));
  // the shared-memory opt-in is set by abm_sir_resident_grid (not a stream operation, so
  // not repeated here, where the call may be captured into a CUDA graph); the shared list
  // heads take what the opt-in leaves, up to the size that function allowed for
  int scap = res_list_cap(bytes);
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, sir_resident_kernel) != cudaSuccess) {
    cudaGetLastError();
    scap = 0;
  } else {
    scap = std::max(0, std::min(scap, (fa.maxDynamicSharedSizeBytes - bytes) / 12 & ~31));
  }
  int st = abm_host::record_cuda_error(cudaMemsetAsync(scratch, 0, sizeof(int32_t), s),
                                       "abm_sir_steps_resident/queue");
  if (st) return st;
  sir_resident_kernel<<<grid, kResThreads, bytes + 12 * scap, s>>>(
      insts, ninst, order, nsteps, bytes, states8, words_base, static_cast<int32_t*>(scratch),
      reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + 256), bytes, scap, status);
  return abm_host::check_launch("abm_sir_steps_resident");
}

size_t abm_sir_changes_bytes(int64_t max_agents, int64_t max_tiles) {
  if (max_agents <= 0 || max_tiles < 0) return 0;
  return align256(sizeof(ListHeader) + (size_t)max_agents * 2 * sizeof(int2)) +
         work_list_bytes(max_tiles);
}

int abm_sir_pack(const int8_t* state, const int32_t* row_ptr, const int32_t* col, int64_t n,
                 int32_t* adj, uint8_t* words, int32_t* hub_counts, uint32_t* comp,
                 int32_t* sizes, int32_t* status, void* stream) {
  if (!state || !row_ptr || !col || !adj || !words || !hub_counts || !comp || !sizes ||
      !status || n <= 0 || n >= (1ll << 29))
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(words, 16) || !abm_host::aligned(comp, 4)) return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  int st = abm_host::record_cuda_error(cudaMemsetAsync(sizes, 0, 3 * sizeof(int32_t), s),
                                       "abm_sir_pack/sizes");
  if (st) return st;
  st = abm_host::record_cuda_error(cudaMemsetAsync(status, 0, sizeof(int32_t), s),
                                   "abm_sir_pack/status");
  if (st) return st;
  const int64_t npad = round16(n);
  sir_pack_mark_kernel<<<(unsigned)((npad + 255) / 256), 256, 0, s>>>(
      state, row_ptr, (int)n, (int)npad, words, sizes, status);
  if ((st = abm_host::check_launch("abm_sir_pack/mark"))) return st;
  const int ngroups = (int)(npad / 16);
  sir_pack_comp_kernel<<<(ngroups + 255) / 256, 256, 0, s>>>(words, ngroups, comp);
  if ((st = abm_host::check_launch("abm_sir_pack/comp"))) return st;
  sir_pack_count_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(row_ptr, col, adj, (int)n,
                                                                   words, hub_counts, status);
  return abm_host::check_launch("abm_sir_pack/count");
}

int abm_sir_pack_batch(const abm_sir_instance* insts, const abm_work_item* work, int32_t nwork,
                       const int8_t* states8, const uint8_t* words_base, int32_t* status,
                       void* stream) {
  if (!insts || !work || nwork <= 0 || !states8 || !words_base || !status) return ABM_ERR_BADARG;
  if (!abm_host::aligned(insts, 8) || !abm_host::aligned(work, 16)) return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  int st = abm_host::record_cuda_error(cudaMemsetAsync(status, 0, sizeof(int32_t), s),
                                       "abm_sir_pack_batch/status");
  if (st) return st;
  const int4* w4 = reinterpret_cast<const int4*>(work);
  sir_pack_mark_tiles_kernel<<<default_grid(nwork), kSirThreads, 0, s>>>(insts, w4, nwork,
                                                                         states8, words_base,
                                                                         status);
  if ((st = abm_host::check_launch("abm_sir_pack_batch/mark"))) return st;
  sir_pack_comp_tiles_kernel<<<default_grid(nwork), kSirThreads, 0, s>>>(insts, w4, nwork);
  if ((st = abm_host::check_launch("abm_sir_pack_batch/comp"))) return st;
  sir_pack_count_tiles_kernel<<<default_grid(nwork), kSirThreads, 0, s>>>(insts, w4, nwork,
                                                                          status);
  return abm_host::check_launch("abm_sir_pack_batch/count");
}

int abm_sir_count_batch(abm_sir_instance* insts, const abm_work_item* work, int32_t nwork,
                        const int8_t* states8, const uint8_t* words_base, void* stream) {
  if (!insts || !work || nwork <= 0 || !states8 || !words_base) return ABM_ERR_BADARG;
  if (!abm_host::aligned(insts, 8) || !abm_host::aligned(work, 16)) return ABM_ERR_BADARG;
  sir_count_tiles_kernel<<<default_grid(nwork), kSirThreads, 0, abm_host::as_stream(stream)>>>(
      insts, reinterpret_cast<const int4*>(work), nwork, states8, words_base);
  return abm_host::check_launch("abm_sir_count_batch");
}

int abm_copy_segments(int64_t count, void* const* dst, const void* const* src,
                      const size_t* bytes, int32_t to_device, void* stream) {
  if (count < 0 || (count > 0 && (!dst || !src || !bytes))) return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  const cudaMemcpyKind kind = to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  for (int64_t k = 0; k < count; ++k) {
    if (bytes[k] == 0) continue;
    if (!dst[k] || !src[k]) return ABM_ERR_BADARG;
    const int st = abm_host::record_cuda_error(cudaMemcpyAsync(dst[k], src[k], bytes[k], kind, s),
                                               "abm_copy_segments");
    if (st) return st;
  }
  return ABM_OK;
}

// Device address of a device or page-locked host pointer, or nullptr for anything else
// (pageable or unknown host memory, which a kernel must not touch).
static const void* device_view(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  return nullptr;
}

int abm_copy_segments_kernel(const abm_copy_segment* segs, int64_t count, void* stream) {
  if (count < 0 || (count > 0 && !segs)) return ABM_ERR_BADARG;
  if (count == 0) return ABM_OK;
  const void* table = device_view(segs);
  if (!table) return ABM_ERR_BADARG;
  for (int64_t k = 0; k < count; ++k) {
    if (segs[k].bytes == 0) continue;
    const void* d = device_view(segs[k].dst);
    const void* s = device_view(segs[k].src);
    // the kernel uses the pointers as given: they must be their own device addresses
    if (d != segs[k].dst || s != segs[k].src) return ABM_ERR_BADARG;
  }
  const int64_t grid = count < (1 << 20) ? count : (1 << 20);
  copy_segments_kernel<<<(unsigned)grid, 256, 0, abm_host::as_stream(stream)>>>(
      static_cast<const abm_copy_segment*>(table), count);
  return abm_host::check_launch("abm_copy_segments_kernel");
}

int abm_sir_unpack(const uint8_t* words, int64_t n, int8_t* state, void* stream) {
  if (!words || !state || n <= 0 || n >= (1ll << 29)) return ABM_ERR_BADARG;
  sir_unpack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, abm_host::as_stream(stream)>>>(
      words, (int)n, state);
  return abm_host::check_launch("abm_sir_unpack");
}

int abm_sir_steps(abm_sir_instance* insts, int32_t ninst, const abm_work_item* work,
                  int32_t nwork, const int32_t* live_work, int32_t nsteps,
                  const abm_sir_launch* launch,
                  void* changes, size_t changes_bytes, void* stream) {
  if (!insts || ninst <= 0 || ninst > (1 << kInstBits) || nwork < 0 || nsteps < 0 ||
      (nwork > 0 && !work) || !changes)
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(insts, 8) || (work && !abm_host::aligned(work, 16)) ||
      !abm_host::aligned(changes, 16) || (live_work && !abm_host::aligned(live_work, 4)))
    return ABM_ERR_BADARG;
  if (changes_bytes < abm_sir_changes_bytes(1, nwork)) return ABM_ERR_WORKSPACE;
  if (nsteps == 0) return ABM_OK;
  const Lists L = carve_lists(changes, changes_bytes, nwork);
  cudaStream_t s = abm_host::as_stream(stream);
  abm_sir_launch cfg;
  abm_sir_default_launch(&cfg);
  if (launch) {
    if (launch->sweep_grid > 0) cfg.sweep_grid = launch->sweep_grid;
    if (launch->candidates_grid > 0) cfg.candidates_grid = launch->candidates_grid;
    if (launch->push_grid > 0) cfg.push_grid = launch->push_grid;
  }
  int g = cfg.sweep_grid;
  if (nwork > 0 && g > nwork) g = nwork;
  const int cand_grid = cfg.candidates_grid;
  const int push_grid = cfg.push_grid;
  const int fin_blocks = (ninst + 255) / 256;
  // few instances: the push kernel's last CTA finalizes the step (one launch less per step)
  const bool fuse = ninst <= kFusedFinalizeMax;
  const int compact_blocks = nwork > 0 ? min((nwork + 255) / 256, abm_host::sm_count() * 4) : 1;
  sir_prepare_kernel<<<fin_blocks, 256, 0, s>>>(insts, ninst);
  int st = abm_host::check_launch("abm_sir_steps/prepare");
  if (st) return st;
  for (int32_t k = 0; k < nsteps; ++k) {
    if (nwork > 0) {
      if (k % kCompactEvery == 0) {
        st = abm_host::record_cuda_error(
            cudaMemsetAsync(&L.hdr->live_tiles, 0, sizeof(int32_t), s), "abm_sir_steps/compact");
        if (st) return st;
        sir_compact_kernel<<<compact_blocks, 256, 0, s>>>(
            insts, reinterpret_cast<const int4*>(work), nwork, live_work, L);
        if ((st = abm_host::check_launch("abm_sir_steps/compact"))) return st;
      }
      sir_sweep_kernel<<<g, kSirThreads, 0, s>>>(insts, L.live_work, nwork, &L.hdr->live_tiles, L);
      if ((st = abm_host::check_launch("abm_sir_steps/sweep"))) return st;
      sir_candidates_kernel<<<cand_grid, kSirThreads, 0, s>>>(insts, L);
      if ((st = abm_host::check_launch("abm_sir_steps/candidates"))) return st;
      sir_push_kernel<<<push_grid, kSirThreads, 0, s>>>(insts, L, fuse ? ninst : 0);
      if ((st = abm_host::check_launch("abm_sir_steps/push"))) return st;
    }
    if (!fuse || nwork == 0) {
      sir_finalize_kernel<<<fin_blocks, 256, 0, s>>>(insts, ninst, L.hdr);
      if ((st = abm_host::check_launch("abm_sir_steps/finalize"))) return st;
    }
  }
  return ABM_OK;
}

size_t abm_sir_run_workspace_bytes(int64_t n, int64_t num_edges) {
  if (n <= 0 || num_edges < 0) return 0;
  const int64_t tiles = (n + kTile - 1) / kTile;
  return align256(sizeof(abm_sir_instance)) + align256((size_t)tiles * sizeof(int4)) +
         align256((size_t)round16(n)) + align256((size_t)n * sizeof(int32_t)) +
         align256((size_t)round16(n) / 4) + 256 +
         align256((size_t)num_edges * sizeof(int32_t)) + align256(abm_sir_changes_bytes(n, tiles));
}

int abm_sir_run(const int32_t* row_ptr, const int32_t* col, int64_t n, int64_t num_edges,
                int8_t* state, const uint32_t* coll_keys, int32_t steps, float beta, float gamma,
                int32_t* counts, void* workspace, size_t workspace_bytes, void* stream) {
  if (!row_ptr || !col || !state || !coll_keys || !counts || n <= 0 || n >= (1ll << 29) ||
      num_edges < 0 || num_edges >= (1ll << 31) || steps < 0)
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(coll_keys, 8)) return ABM_ERR_BADARG;
  const size_t need = abm_sir_run_workspace_bytes(n, num_edges);
  if (!workspace || workspace_bytes < need || !abm_host::aligned(workspace, 256))
    return ABM_ERR_WORKSPACE;
  if (steps == 0) return ABM_OK;
  cudaStream_t s = abm_host::as_stream(stream);
  char* p = static_cast<char*>(workspace);
  abm_sir_instance* d = reinterpret_cast<abm_sir_instance*>(p);
  p += align256(sizeof(abm_sir_instance));
  const int ntiles = (int)((n + kTile - 1) / kTile);
  int4* work = reinterpret_cast<int4*>(p);
  p += align256((size_t)ntiles * sizeof(int4));
  uint8_t* words = reinterpret_cast<uint8_t*>(p);
  p += align256((size_t)round16(n));
  int32_t* hubs = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)n * sizeof(int32_t));
  uint32_t* comp = reinterpret_cast<uint32_t*>(p);
  p += align256((size_t)round16(n) / 4);
  int32_t* misc = reinterpret_cast<int32_t*>(p);  // sizes[3], status
  p += 256;
  int32_t* adj = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)num_edges * sizeof(int32_t));
  void* lists = p;
  int st = abm_sir_pack(state, row_ptr, col, n, adj, words, hubs, comp, misc, misc + 3, stream);
  if (st) return st;
  st = abm_host::record_cuda_error(cudaMemsetAsync(lists, 0, sizeof(ListHeader), s),
                                   "abm_sir_run/lists");
  if (st) return st;
  sir_setup_single_kernel<<<(ntiles + 255) / 256, 256, 0, s>>>(
      d, work, ntiles, row_ptr, adj, words, hubs, comp, counts, coll_keys, (int32_t)n, steps,
      beta, gamma, misc);
  st = abm_host::check_launch("abm_sir_run/setup");
  if (st) return st;
  const size_t lists_bytes = align256(abm_sir_changes_bytes(n, ntiles));
  // a model whose words fit shared memory runs every step in one launch of one resident CTA
  // (no per-step launches; the descriptor's per-step keys drive it); larger ones step
  // through the per-step kernels over the whole GPU
  if (abm_sir_resident_grid(static_cast<int32_t>(n)) > 0 &&
      abm_sir_resident_scratch_bytes(static_cast<int32_t>(n), 1) <= lists_bytes) {
    st = abm_sir_steps_resident(d, 1, nullptr, static_cast<int32_t>(n), steps, 1, nullptr,
                                nullptr, lists, lists_bytes, misc + 3, stream);
  } else {
    st = abm_sir_steps(d, 1, reinterpret_cast<const abm_work_item*>(work), ntiles, nullptr,
                       steps, nullptr, lists, lists_bytes, stream);
  }
  if (st) return st;
  return abm_sir_unpack(words, n, state, stream);
}

}  // extern "C"

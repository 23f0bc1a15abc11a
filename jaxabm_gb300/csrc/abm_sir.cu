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
// Work-efficient ("frontier") formulation.  Each agent has one int32 word
//     word = (number of infected neighbours << 2) | compartment
// and a step is four launches:
//   sweep      over (instance, 4096-agent tile) work items, 16 agents per thread read with
//              128-bit loads: agents that need a decision are appended to a candidate list
//              -- susceptible ones with infected neighbours from its front, infected ones
//              from its back -- with one counter atomic per CTA and tile (block scan for
//              the offsets).  Everyone else (most agents) costs one 4-byte read.
//   candidates one lane per candidate: a susceptible candidate scans its CSR row, eight
//              column/neighbour loads in flight per pass, stopping at the first firing draw
//              or once all its infected neighbours were seen (rows longer than 32 slots are
//              scanned by the whole warp, 32 slots per pass, with warp votes); an infected
//              candidate draws its recovery.  Changes go to a change list.  Nothing is
//              written to the words, so every decision sees the pre-step states.
//   push       one thread per change (one warp for rows longer than 32 slots): adds +-4 to
//              the word of every neighbour (infected-neighbour count) and +1 to the agent's
//              own compartment; counts the instance's S->I and I->R transitions.
//   finalize   one thread per instance: S/I/R counts of the step from the transitions,
//              rng = split(rng)[0], t += 1, the next step's collection key, done flag after
//              the last step; clears the lists.
// Integer atomics commute, so every result is exact and independent of scheduling.  No
// kernel waits on anything.

#include "abm_common.cuh"

namespace {

constexpr int kSirThreads = 256;
constexpr int kWarpsPerCta = kSirThreads / 32;
constexpr int kVec = 4;                            // words per 128-bit load
constexpr int kVecsPerThread = 4;
constexpr int kPerThread = kVec * kVecsPerThread;  // 16 agents per thread
constexpr int kTile = kSirThreads * kPerThread;    // 4096 agents per work item
constexpr int kHeavyDeg = 32;
constexpr int kChunk = 8;                          // row slots per scan pass
constexpr unsigned kFull = 0xffffffffu;
constexpr int kS = 0, kI = 1;

static_assert(sizeof(abm_sir_instance) == 120, "abm_sir_instance layout");
static_assert(sizeof(abm_work_item) == 16, "abm_work_item layout");

// Lists workspace: this header, then `capacity` change entries (int2 {inst, agent << 2 |
// new compartment}), then `capacity` candidate entries (int4 {inst, agent, word, 0});
// susceptible candidates fill the candidate array from the front, infected ones from the
// back (an agent is at most one candidate, so the two never meet).
struct ListHeader {
  int32_t changes;
  int32_t overflow;
  int32_t cand_s;
  int32_t cand_i;
};

struct Lists {
  ListHeader* hdr;
  int2* changes;
  int4* cands;
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

__global__ void __launch_bounds__(kSirThreads)
sir_sweep_kernel(const abm_sir_instance* __restrict__ insts, const int4* __restrict__ work,
                 int nwork_max, const int32_t* __restrict__ live, Lists L) {
  __shared__ int swarp[kWarpsPerCta];
  __shared__ int sbase_s, sbase_i;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwork = live_count(live, nwork_max);
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int4 item = work[w];
    const abm_sir_instance* I = insts + item.x;
    // finished instances, and instances without an infected agent (nothing can change in
    // them any more: no infection source, no recovery), need no decisions
    if (I->t >= I->steps || I->num_i == 0) continue;  // uniform over the CTA
    const int32_t* __restrict__ word = I->state;
    // thread t owns agents begin + v*1024 + 4t + c (v, c < 4): four 128-bit loads when the
    // words are 16-byte aligned, scalar loads for a partial last vector
    const bool vec_ok = ((reinterpret_cast<uintptr_t>(word) & 15) == 0) && ((item.y & 3) == 0);
    int32_t wv[kPerThread];
#pragma unroll
    for (int v = 0; v < kVecsPerThread; ++v) {
      const int base = item.y + v * (kSirThreads * kVec) + kVec * threadIdx.x;
      if (vec_ok && base + kVec <= item.z) {
        const int4 q = *reinterpret_cast<const int4*>(word + base);
        wv[kVec * v] = q.x;
        wv[kVec * v + 1] = q.y;
        wv[kVec * v + 2] = q.z;
        wv[kVec * v + 3] = q.w;
      } else {
#pragma unroll
        for (int c = 0; c < kVec; ++c) wv[kVec * v + c] = base + c < item.z ? word[base + c] : 2;
      }
    }
    unsigned need_s = 0, need_i = 0;
#pragma unroll
    for (int j = 0; j < kPerThread; ++j) {
      const int s = wv[j] & 3;
      if (s == kS && (wv[j] >> 2) > 0) need_s |= 1u << j;
      if (s == kI) need_i |= 1u << j;
    }
    // one counter atomic per list, CTA and tile: both counts scanned at once (16 bits each)
    const int mine = __popc(need_s) | (__popc(need_i) << 16);
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) swarp[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      int total = 0;
      for (int q = 0; q < kWarpsPerCta; ++q) total += swarp[q];
      const int ts = total & 0xFFFF, ti = total >> 16;
      sbase_s = ts ? atomicAdd(&L.hdr->cand_s, ts) : 0;
      sbase_i = ti ? atomicAdd(&L.hdr->cand_i, ti) : 0;
    }
    __syncthreads();
    int before = incl - mine;
    for (int q = 0; q < warp; ++q) before += swarp[q];
    int pos_s = sbase_s + (before & 0xFFFF);
    int pos_i = sbase_i + (before >> 16);
    __syncthreads();  // swarp/sbase_* are rewritten by the next tile
    if (need_s | need_i) {
#pragma unroll
      for (int j = 0; j < kPerThread; ++j) {
        const int i = item.y + (j / kVec) * (kSirThreads * kVec) + kVec * threadIdx.x + (j % kVec);
        if ((need_s >> j) & 1u) {
          if (pos_s < L.capacity) L.cands[pos_s] = make_int4(item.x, i, wv[j], 0);
          else L.hdr->overflow = 1;
          ++pos_s;
        } else if ((need_i >> j) & 1u) {
          if (pos_i < L.capacity) L.cands[L.capacity - 1 - pos_i] = make_int4(item.x, i, wv[j], 0);
          else L.hdr->overflow = 1;
          ++pos_i;
        }
      }
    }
  }
}

// Per-instance sum of `v` over the lanes of a warp (lanes grouped by instance), added to
// the group's instance by the group's lowest lane.
__device__ __forceinline__ void add_scanned(int inst, int v, abm_sir_instance* insts, int lane) {
  if (!__any_sync(kFull, v != 0)) return;
  const unsigned group = __match_any_sync(kFull, inst);
  const int sum = __reduce_add_sync(group, v);
  if (lane == __ffs(group) - 1 && sum) atomicAdd(&insts[inst].edges_scanned, (unsigned long long)sum);
}

__device__ __forceinline__ void record_change(bool changed, int inst, int i, int ns, Lists& L,
                                              int lane) {
  const int pos = warp_append(changed, &L.hdr->changes, lane);
  if (changed) {
    if (pos < L.capacity) L.changes[pos] = make_int2(inst, (i << 2) | ns);
    else L.hdr->overflow = 1;
  }
}

__global__ void __launch_bounds__(kSirThreads)
sir_candidates_kernel(abm_sir_instance* __restrict__ insts, Lists L) {
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * kWarpsPerCta;
  const int wid = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);

  // infected candidates: recovery draws
  const int ni = min(L.hdr->cand_i, L.capacity);
  for (int b = wid * 32; b < ni; b += warps * 32) {
    const int k = b + lane;
    const bool valid = k < ni;
    const int4 e = valid ? L.cands[L.capacity - 1 - k] : make_int4(0, 0, 2, 0);
    bool changed = false;
    if (valid) {
      const abm_sir_instance* I = insts + e.x;
      const uint2 coll = make_uint2(I->coll[0], I->coll[1]);
      const uint2 krec = abm::split_at(abm::split_at(coll, (uint64_t)e.y), 1);
      changed = abm::unit_float(abm::bits_at(krec, 0)) < I->gamma;
    }
    record_change(changed, e.x, e.y, 2, L, lane);
  }

  // susceptible candidates with infected neighbours: row scans
  const int ns_count = min(L.hdr->cand_s, L.capacity);
  for (int b = wid * 32; b < ns_count; b += warps * 32) {
    const int k = b + lane;
    const bool valid = k < ns_count;
    const int4 e = valid ? L.cands[k] : make_int4(0, 0, 2, 0);
    const int inst = e.x, i = e.y;
    const abm_sir_instance* I = insts + inst;
    int cnt = e.z >> 2;
    bool infected = false, heavy = false;
    int row0 = 0, deg = 0, scanned = 0;
    uint2 coll = make_uint2(0, 0);
    if (valid) {
      coll = make_uint2(I->coll[0], I->coll[1]);
      const int32_t* __restrict__ rp = I->row_ptr;
      row0 = rp[i];
      deg = rp[i + 1] - row0;
      if (deg > kHeavyDeg) {
        heavy = true;
      } else {
        const int32_t* __restrict__ col = I->col;
        const int32_t* __restrict__ word = I->state;
        const float beta = I->beta;
        const uint2 kinf = abm::split_at(abm::split_at(coll, (uint64_t)i), 0);
        // eight slots per pass: the eight column loads, then the eight neighbour-word
        // loads, are issued together before any is used
        scanned = deg;
        bool done = false;
        for (int k0 = 0; k0 < deg && !done; k0 += kChunk) {
          int nb[kChunk];
          int32_t wn[kChunk];
#pragma unroll
          for (int q = 0; q < kChunk; ++q) nb[q] = k0 + q < deg ? col[row0 + k0 + q] : -1;
#pragma unroll
          for (int q = 0; q < kChunk; ++q) wn[q] = nb[q] >= 0 ? word[nb[q]] : 0;
#pragma unroll
          for (int q = 0; q < kChunk; ++q) {
            if (!done && nb[q] >= 0 && (wn[q] & 3) == kI) {
              const int slot = k0 + q;
              if (abm::unit_float(abm::bits_at(kinf, (uint64_t)slot)) < beta) {
                infected = true;
                done = true;
                scanned = slot + 1;
              } else if (--cnt == 0) {
                done = true;
                scanned = slot + 1;
              }
            }
          }
        }
      }
    }

    // rows longer than kHeavyDeg: the whole warp scans them, one at a time
    unsigned hmask = __ballot_sync(kFull, heavy);
    while (hmask) {
      const int src = __ffs(hmask) - 1;
      hmask &= hmask - 1;
      const int hinst = __shfl_sync(kFull, inst, src);
      const int hi = __shfl_sync(kFull, i, src);
      const int hrow = __shfl_sync(kFull, row0, src);
      const int hdeg = __shfl_sync(kFull, deg, src);
      int remaining = __shfl_sync(kFull, cnt, src);
      const abm_sir_instance* H = insts + hinst;
      const uint2 hcoll = make_uint2(H->coll[0], H->coll[1]);
      const int32_t* __restrict__ col = H->col;
      const int32_t* __restrict__ word = H->state;
      const float beta = H->beta;
      const uint2 kinf = abm::split_at(abm::split_at(hcoll, (uint64_t)hi), 0);
      bool fired = false;
      int c = 0;
      for (; c < hdeg && !fired && remaining > 0; c += 32) {
        const int slot = c + lane;
        bool isI = false, f = false;
        if (slot < hdeg) {
          isI = (word[col[hrow + slot]] & 3) == kI;
          if (isI) f = abm::unit_float(abm::bits_at(kinf, (uint64_t)slot)) < beta;
        }
        fired = __any_sync(kFull, f);
        remaining -= __popc(__ballot_sync(kFull, isI));
      }
      if (lane == src) {
        infected = fired;
        scanned = min(c, hdeg);
      }
    }

    record_change(infected, inst, i, kI, L, lane);
    add_scanned(inst, scanned, insts, lane);
  }
}

// Neighbours' infected counts +-1 and own compartment +1 for every change: one thread per
// change for rows up to kHeavyDeg slots (atomics issued without waiting for results), one
// warp for longer rows.
__global__ void __launch_bounds__(kSirThreads)
sir_push_kernel(abm_sir_instance* __restrict__ insts, Lists L) {
  const int lane = threadIdx.x & 31;
  const int count = min(L.hdr->changes, L.capacity);
  const int threads = gridDim.x * kSirThreads;
  for (int b = (blockIdx.x * kSirThreads + threadIdx.x) & ~31; b < count; b += threads) {
    const int k = b + lane;
    const bool valid = k < count;
    int inst = 0, agent = 0, r0 = 0, r1 = 0, delta = 0;
    abm_sir_instance* I = insts;
    if (valid) {
      const int2 ent = L.changes[k];
      inst = ent.x;
      agent = ent.y >> 2;
      I = insts + inst;
      delta = (ent.y & 3) == kI ? 4 : -4;
      r0 = I->row_ptr[agent];
      r1 = I->row_ptr[agent + 1];
      atomicAdd(&I->state[agent], 1);  // S(0) -> I(1) and I(1) -> R(2) both add one
      atomicAdd(delta > 0 ? &I->step_si : &I->step_ir, 1);
      atomicAdd(&I->edges_pushed, (unsigned long long)(r1 - r0));
    }
    const bool heavy = valid && r1 - r0 > kHeavyDeg;
    if (valid && !heavy) {
      int32_t* __restrict__ word = I->state;
      const int32_t* __restrict__ col = I->col;
      for (int e0 = r0; e0 < r1; e0 += kChunk) {
        int nb[kChunk];
#pragma unroll
        for (int q = 0; q < kChunk; ++q) nb[q] = e0 + q < r1 ? col[e0 + q] : -1;
#pragma unroll
        for (int q = 0; q < kChunk; ++q)
          if (nb[q] >= 0) atomicAdd(&word[nb[q]], delta);
      }
    }
    unsigned hmask = __ballot_sync(kFull, heavy);
    while (hmask) {
      const int src = __ffs(hmask) - 1;
      hmask &= hmask - 1;
      const int hinst = __shfl_sync(kFull, inst, src);
      const int hr0 = __shfl_sync(kFull, r0, src);
      const int hr1 = __shfl_sync(kFull, r1, src);
      const int hdelta = __shfl_sync(kFull, delta, src);
      int32_t* __restrict__ word = insts[hinst].state;
      const int32_t* __restrict__ col = insts[hinst].col;
      for (int e = hr0 + lane; e < hr1; e += 32) atomicAdd(&word[col[e]], hdelta);
    }
  }
}

// Counts after the step, key chain, step counter, next step's key, done flag; clears the
// lists.
__global__ void sir_finalize_kernel(abm_sir_instance* __restrict__ insts, int ninst,
                                    ListHeader* __restrict__ hdr) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0) {
    hdr->changes = 0;
    hdr->cand_s = 0;
    hdr->cand_i = 0;
  }
  if (k >= ninst) return;
  abm_sir_instance* I = insts + k;
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

__device__ __forceinline__ int32_t pack_word(const int8_t* __restrict__ st,
                                             const int32_t* __restrict__ rp,
                                             const int32_t* __restrict__ col, int i, int s) {
  int c = 0;
  for (int k = rp[i]; k < rp[i + 1]; ++k) c += st[col[k]] == kI;
  return (c << 2) | s;
}

// word[i] = (infected neighbours << 2) | state[i]; compartment sizes into *sizes.
__global__ void sir_pack_kernel(const int8_t* __restrict__ state, const int32_t* __restrict__ rp,
                                const int32_t* __restrict__ col, int n, int32_t* __restrict__ word,
                                int32_t* __restrict__ sizes, int32_t* __restrict__ bad) {
  __shared__ int sc[3];
  if (threadIdx.x < 3) sc[threadIdx.x] = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int s = state[i];
    if (s < 0 || s > 2) {
      atomicExch(bad, 1);
    } else {
      word[i] = pack_word(state, rp, col, i, s);
      atomicAdd(&sc[s], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x < 3 && sc[threadIdx.x]) atomicAdd(&sizes[threadIdx.x], sc[threadIdx.x]);
}

// The same over the tiles of many instances: the int8 compartments of an instance sit in
// states8 at the same element offset as its words from words_base.
__global__ void sir_pack_tiles_kernel(const abm_sir_instance* __restrict__ insts,
                                      const int4* __restrict__ work, int nwork,
                                      const int8_t* __restrict__ states8,
                                      const int32_t* __restrict__ words_base,
                                      int32_t* __restrict__ bad) {
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int4 item = work[w];
    const abm_sir_instance* I = insts + item.x;
    int32_t* word = I->state;
    const int8_t* st = states8 + (word - words_base);
    for (int i = item.y + threadIdx.x; i < item.z; i += blockDim.x) {
      const int s = st[i];
      if (s < 0 || s > 2) {
        atomicExch(bad, 1);
        continue;
      }
      word[i] = pack_word(st, I->row_ptr, I->col, i, s);
    }
  }
}

__global__ void sir_unpack_kernel(const int32_t* __restrict__ word, int n, int8_t* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (int8_t)(word[i] & 3);
}

// Single-instance descriptor and tile list written on the device, so abm_sir_run makes
// no host-to-device copy and can be captured in a CUDA graph.
__global__ void sir_setup_single_kernel(abm_sir_instance* d, int4* work, int ntiles,
                                       const int32_t* row_ptr, const int32_t* col, int32_t* words,
                                       int32_t* counts, const uint32_t* coll_keys, int32_t n,
                                       int32_t steps, float beta, float gamma,
                                       const int32_t* sizes) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g == 0) {
    d->row_ptr = row_ptr;
    d->col = col;
    d->state = words;
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
    d->coll[0] = 0;
    d->coll[1] = 0;
  }
  for (int b = g; b < ntiles; b += gridDim.x * blockDim.x) {
    const int begin = b * kTile;
    const int end = min(begin + kTile, n);
    work[b] = make_int4(0, begin, end, 0);
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

Lists carve_lists(void* ws, size_t bytes) {
  Lists L;
  L.hdr = static_cast<ListHeader*>(ws);
  size_t cap = (bytes - sizeof(ListHeader)) / (sizeof(int2) + sizeof(int4));
  if (cap > 0x7FFFFFFE) cap = 0x7FFFFFFE;
  cap &= ~(size_t)1;  // even: keeps the int4 candidate entries 16-byte aligned
  L.capacity = (int)cap;
  L.changes = reinterpret_cast<int2*>(L.hdr + 1);
  L.cands = reinterpret_cast<int4*>(L.changes + L.capacity);
  return L;
}

}  // namespace

extern "C" {

size_t abm_sir_instance_size(void) { return sizeof(abm_sir_instance); }

int32_t abm_sir_tile_agents(void) { return kTile; }

int abm_sir_default_launch(abm_sir_launch* out) {
  if (!out) return ABM_ERR_BADARG;
  out->sweep_grid = resident_grid(sir_sweep_kernel, 4);
  out->candidates_grid = resident_grid(sir_candidates_kernel, 4);
  out->push_grid = resident_grid(sir_push_kernel, 4);
  out->reserved = 0;
  return ABM_OK;
}

size_t abm_sir_changes_bytes(int64_t max_agents) {
  if (max_agents <= 0) return 0;
  const size_t cap = ((size_t)max_agents + 1) & ~(size_t)1;
  return sizeof(ListHeader) + cap * (sizeof(int2) + sizeof(int4));
}

int abm_sir_pack(const int8_t* state, const int32_t* row_ptr, const int32_t* col, int64_t n,
                 int32_t* words, int32_t* sizes, int32_t* status, void* stream) {
  if (!state || !row_ptr || !col || !words || !sizes || !status || n <= 0 || n >= (1ll << 29))
    return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  int st = abm_host::record_cuda_error(cudaMemsetAsync(sizes, 0, 3 * sizeof(int32_t), s),
                                       "abm_sir_pack/sizes");
  if (st) return st;
  st = abm_host::record_cuda_error(cudaMemsetAsync(status, 0, sizeof(int32_t), s),
                                   "abm_sir_pack/status");
  if (st) return st;
  sir_pack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(state, row_ptr, col, (int)n, words,
                                                             sizes, status);
  return abm_host::check_launch("abm_sir_pack");
}

int abm_sir_pack_batch(const abm_sir_instance* insts, const abm_work_item* work, int32_t nwork,
                       const int8_t* states8, const int32_t* words_base, int32_t* status,
                       void* stream) {
  if (!insts || !work || nwork <= 0 || !states8 || !words_base || !status) return ABM_ERR_BADARG;
  if (!abm_host::aligned(insts, 8) || !abm_host::aligned(work, 16)) return ABM_ERR_BADARG;
  cudaStream_t s = abm_host::as_stream(stream);
  int st = abm_host::record_cuda_error(cudaMemsetAsync(status, 0, sizeof(int32_t), s),
                                       "abm_sir_pack_batch/status");
  if (st) return st;
  sir_pack_tiles_kernel<<<default_grid(nwork), kSirThreads, 0, s>>>(
      insts, reinterpret_cast<const int4*>(work), nwork, states8, words_base, status);
  return abm_host::check_launch("abm_sir_pack_batch");
}

int abm_sir_unpack(const int32_t* words, int64_t n, int8_t* state, void* stream) {
  if (!words || !state || n <= 0 || n >= (1ll << 29)) return ABM_ERR_BADARG;
  sir_unpack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, abm_host::as_stream(stream)>>>(
      words, (int)n, state);
  return abm_host::check_launch("abm_sir_unpack");
}

int abm_sir_steps(abm_sir_instance* insts, int32_t ninst, const abm_work_item* work,
                  int32_t nwork, const int32_t* live_work, int32_t nsteps,
                  const abm_sir_launch* launch,
                  void* changes, size_t changes_bytes, void* stream) {
  if (!insts || ninst <= 0 || nwork < 0 || nsteps < 0 || (nwork > 0 && !work) || !changes)
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(insts, 8) || (work && !abm_host::aligned(work, 16)) ||
      !abm_host::aligned(changes, 16) || (live_work && !abm_host::aligned(live_work, 4)))
    return ABM_ERR_BADARG;
  if (changes_bytes < abm_sir_changes_bytes(1)) return ABM_ERR_WORKSPACE;
  if (nsteps == 0) return ABM_OK;
  const Lists L = carve_lists(changes, changes_bytes);
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
  sir_prepare_kernel<<<fin_blocks, 256, 0, s>>>(insts, ninst);
  int st = abm_host::check_launch("abm_sir_steps/prepare");
  if (st) return st;
  for (int32_t k = 0; k < nsteps; ++k) {
    if (nwork > 0) {
      sir_sweep_kernel<<<g, kSirThreads, 0, s>>>(insts, reinterpret_cast<const int4*>(work), nwork,
                                                 live_work, L);
      if ((st = abm_host::check_launch("abm_sir_steps/sweep"))) return st;
      sir_candidates_kernel<<<cand_grid, kSirThreads, 0, s>>>(insts, L);
      if ((st = abm_host::check_launch("abm_sir_steps/candidates"))) return st;
      sir_push_kernel<<<push_grid, kSirThreads, 0, s>>>(insts, L);
      if ((st = abm_host::check_launch("abm_sir_steps/push"))) return st;
    }
    sir_finalize_kernel<<<fin_blocks, 256, 0, s>>>(insts, ninst, L.hdr);
    if ((st = abm_host::check_launch("abm_sir_steps/finalize"))) return st;
  }
  return ABM_OK;
}

size_t abm_sir_run_workspace_bytes(int64_t n) {
  if (n <= 0) return 0;
  const int64_t tiles = (n + kTile - 1) / kTile;
  return align256(sizeof(abm_sir_instance)) + align256((size_t)tiles * sizeof(int4)) +
         align256((size_t)n * sizeof(int32_t)) + 256 + align256(abm_sir_changes_bytes(n));
}

int abm_sir_run(const int32_t* row_ptr, const int32_t* col, int64_t n, int8_t* state,
                const uint32_t* coll_keys, int32_t steps, float beta, float gamma,
                int32_t* counts, void* workspace, size_t workspace_bytes, void* stream) {
  if (!row_ptr || !col || !state || !coll_keys || !counts || n <= 0 || n >= (1ll << 29) ||
      steps < 0)
    return ABM_ERR_BADARG;
  if (!abm_host::aligned(coll_keys, 8)) return ABM_ERR_BADARG;
  const size_t need = abm_sir_run_workspace_bytes(n);
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
  int32_t* words = reinterpret_cast<int32_t*>(p);
  p += align256((size_t)n * sizeof(int32_t));
  int32_t* misc = reinterpret_cast<int32_t*>(p);  // sizes[3], status
  p += 256;
  void* lists = p;
  int st = abm_sir_pack(state, row_ptr, col, n, words, misc, misc + 3, stream);
  if (st) return st;
  st = abm_host::record_cuda_error(cudaMemsetAsync(lists, 0, sizeof(ListHeader), s),
                                   "abm_sir_run/lists");
  if (st) return st;
  sir_setup_single_kernel<<<(ntiles + 255) / 256, 256, 0, s>>>(
      d, work, ntiles, row_ptr, col, words, counts, coll_keys, (int32_t)n, steps, beta, gamma,
      misc);
  st = abm_host::check_launch("abm_sir_run/setup");
  if (st) return st;
  st = abm_sir_steps(d, 1, reinterpret_cast<const abm_work_item*>(work), ntiles, nullptr, steps,
                     nullptr, lists, align256(abm_sir_changes_bytes(n)), stream);
  if (st) return st;
  return abm_sir_unpack(words, n, state, stream);
}

}  // extern "C"

/*
 * jaxabm_gb300 — C ABI of the GB300 agent-step engine.
 *
 * Every entry point:
 *   - returns an int status (ABM_OK = 0, else one of the ABM_ERR_* codes below);
 *   - takes a `void* stream` that is a cudaStream_t (NULL = legacy default stream);
 *   - borrows the device pointers it is given for the duration of the call (work is
 *     enqueued on `stream`; the caller keeps the buffers alive until the stream has
 *     finished it) and keeps no pointer after return;
 *   - allocates no device memory: scratch comes from a caller-provided workspace whose
 *     size the matching *_workspace_bytes() query returns.
 *
 * PRNG keys are uint32 pairs in device memory, laid out exactly like a JAX raw key
 * (`jax.random.PRNGKey(seed)` = [seed >> 32, seed & 0xffffffff]).
 * `mode` selects the `jax_threefry_partitionable` behaviour: ABM_RNG_PARTITIONABLE (the
 * JAX >= 0.5 default) or ABM_RNG_LEGACY (the original mode).  Model kernels use the
 * partitionable mode.
 *
 * Reference interfaces are cited as path:line inside the JaxABM 0.1.5 source tree.
 */
#ifndef JAXABM_GB300_H
#define JAXABM_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ABM_API __attribute__((visibility("default")))
#else
#define ABM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------ */
#define ABM_OK 0
#define ABM_ERR_BADARG 1       /* null pointer, non-positive size, bad mode, misalignment */
#define ABM_ERR_OOM 2          /* request does not fit the free device memory            */
#define ABM_ERR_TIMEOUT 3      /* a bounded device-side wait ran out                      */
#define ABM_ERR_BOUNDS 4       /* a checked gather/scatter index was out of range         */
#define ABM_ERR_UNREGISTERED 5 /* no step kernel registered for the agent class           */
#define ABM_ERR_CUDA 6         /* a CUDA runtime call or kernel launch failed             */
#define ABM_ERR_WORKSPACE 7    /* caller workspace is null or smaller than required       */

#define ABM_RNG_LEGACY 0
#define ABM_RNG_PARTITIONABLE 1

/* Library version (major*10000 + minor*100 + patch). */
ABM_API int abm_version(void);

/* Static string naming a status code. */
ABM_API const char* abm_status_string(int status);

/* Text of the last CUDA error seen by the library on this host thread ("" if none). */
ABM_API const char* abm_last_cuda_error(void);

/* Range-checked build.  The library compiled with -DABM_CHECKED
 * (libjaxabm_gb300_checked.so) checks every gather whose index comes from caller data --
 * CSR row offsets and columns of the opinion kernels, row indices of abm_gather_rows --
 * and an entry point that met an index outside its array waits for its stream and returns
 * ABM_ERR_BOUNDS (the access itself is redirected to element 0); abm_bounds_detail() then
 * names the entry point, the first bad index, its bound and the checking source line.  A
 * stream being captured into a CUDA graph is not waited for and not checked.  This is the
 * stand-in for a device memory checker; it has no counterpart in the reference, whose
 * gathers run inside JAX.  abm_checked_build() is 1 in that build and 0 in the normal one,
 * where abm_bounds_detail() stays empty. */
ABM_API const char* abm_bounds_detail(void);
ABM_API int abm_checked_build(void);

/* SM count and compute capability of the current device. */
ABM_API int abm_device_info(int* sm_count, int* cc_major, int* cc_minor);

/* ---- K1: threefry2x32-20 and jax.random -------------------------------------------- */

/* vmap(lambda k: jax.random.split(k, num))(keys): keys uint32[nkeys][2] ->
 * out uint32[nkeys][num][2].  Replaces jax.random.split at jaxabm/model.py:129,156,164,183
 * and jaxabm/agent.py:115,156. */
ABM_API int abm_rng_split(const uint32_t* keys, int64_t nkeys, int64_t num, uint32_t* out, int mode,
                  void* stream);

/* vmap(lambda k: jax.random.bits(k, (count,), uint32))(keys) -> out uint32[nkeys][count]. */
ABM_API int abm_rng_bits(const uint32_t* keys, int64_t nkeys, int64_t count, uint32_t* out, int mode,
                 void* stream);

/* vmap(lambda k: jax.random.uniform(k, (count,), float32, minval, maxval))(keys). */
ABM_API int abm_rng_uniform(const uint32_t* keys, int64_t nkeys, int64_t count, float minval,
                    float maxval, float* out, int mode, void* stream);

/* vmap(lambda k: jax.random.normal(k, (count,), float32))(keys).  The inverse error
 * function is Giles' single-precision approximation (GPU Computing Gems, 2011). */
ABM_API int abm_rng_normal(const uint32_t* keys, int64_t nkeys, int64_t count, float* out, int mode,
                   void* stream);

/* vmap(lambda k: jax.random.bernoulli(k, p, (count,)))(keys) -> out uint8 0/1. */
ABM_API int abm_rng_bernoulli(const uint32_t* keys, int64_t nkeys, int64_t count, float p,
                      uint8_t* out, int mode, void* stream);

/* vmap(lambda k: jax.random.randint(k, (count,), minval, maxval, int32))(keys): two bit
 * draws from split(key) combined modulo the span, as jax.random.randint does.  Used by
 * Grid.position_agents (jaxabm/agentpy.py:509-512). */
ABM_API int abm_rng_randint(const uint32_t* keys, int64_t nkeys, int64_t count, int32_t minval,
                            int32_t maxval, int32_t* out, int mode, void* stream);

/* Key chain of Model.step (jaxabm/model.py:155-190) for `steps` steps of `ninst`
 * independent models with `ncoll` agent collections each:
 *   rng, step_key = split(rng); for c: step_key, coll_key[c] = split(step_key)
 * rng uint32[ninst][2] is read and overwritten with the advanced key;
 * coll_keys uint32[ninst][steps][ncoll][2] receives the per-step collection keys and
 * update_keys (nullable) uint32[ninst][steps][2] the key handed to update_state_fn
 * (split(step_key)[1] after the collections, jaxabm/model.py:183).
 * Partitionable mode. */
ABM_API int abm_keychain(uint32_t* rng, int64_t ninst, int32_t ncoll, int32_t steps,
                         uint32_t* coll_keys, uint32_t* update_keys, void* stream);

/* ---- random walk (quick-start model) ----------------------------------------------- */
/* Agent init: agent_key_i = split(init_key, n)[i]; kx, ky = split(agent_key_i);
 * x_i = uniform(kx), y_i = uniform(ky).  Replaces AgentCollection.init
 * (jaxabm/agent.py:92-130) for the random-walk agent. */
ABM_API int abm_randomwalk_init(float* x, float* y, int64_t n, const uint32_t* init_key, void* stream);

ABM_API size_t abm_randomwalk_workspace_bytes(int64_t n, int32_t steps);

/* `steps` synchronous steps of the random walk: for step t with collection key
 * coll_keys[t] (uint32[steps][2], as written by abm_keychain with ncoll = 1):
 *   agent_key_i = split(coll_key, n)[i]; kx, ky = split(agent_key_i);
 *   x_i = (x_i + sigma * normal(kx)) mod 1.0; y_i likewise with ky;
 *   means[t] = (mean x, mean y) after the update (float32[steps][2]).
 * Replaces the Python loop of JaxModel.run (jaxabm/model.py:240-241) over
 * AgentCollection.update (jaxabm/agent.py:132-179) and the metrics reduction
 * (jaxabm/model.py:193-200). */
ABM_API int abm_randomwalk_run(float* x, float* y, int64_t n, const uint32_t* coll_keys, int32_t steps,
                       float sigma, float* means, void* workspace, size_t workspace_bytes,
                       void* stream);

/* Batches of `members` independent random-walk models of n agents each, in one launch
 * (the ensembles of Model.batch_run / SensitivityAnalysis.run, jaxabm/agentpy.py:1116-1152,
 * jaxabm/analysis.py:97-165, which the reference runs one model after another): member m
 * holds x, y at [m * n, (m + 1) * n), its init key init_keys[m] (uint32[members][2]), its
 * collection keys coll_keys[m] (uint32[members][steps][2]), sigma sigmas[m] (device
 * float32[members]) and means[m] (float32[members][steps][2]).  Every member's result
 * equals abm_randomwalk_init / abm_randomwalk_run of that member alone, bit for bit.
 * 1 <= members <= 65535. */
ABM_API int abm_randomwalk_init_batch(float* x, float* y, int64_t n, int32_t members,
                                      const uint32_t* init_keys, void* stream);
ABM_API size_t abm_randomwalk_batch_workspace_bytes(int64_t n, int32_t steps, int32_t members);
ABM_API int abm_randomwalk_run_batch(float* x, float* y, int64_t n, int32_t members,
                                     const uint32_t* coll_keys, int32_t steps,
                                     const float* sigmas, float* means, void* workspace,
                                     size_t workspace_bytes, void* stream);

/* ---- Network construction (HOST memory; native setup code) ------------------------- */
/* Directed-entry count 2*m*(n-m) of a Barabasi-Albert graph, or -1 for bad sizes. */
ABM_API int64_t abm_graph_ba_num_edges(int64_t n, int32_t m);

/* Barabasi-Albert preferential attachment (star on nodes 0..m, then each new node links
 * to m distinct nodes drawn from the degree-weighted node list), written as symmetric CSR
 * with rows sorted ascending into HOST buffers row_ptr int32[n+1] and col int32[capacity].
 * Replaces building the graph with Network.add_edge (jaxabm/agentpy.py:559-582). */
ABM_API int abm_graph_barabasi_albert(int64_t n, int32_t m, uint64_t seed, int32_t* row_ptr,
                                      int32_t* col, int64_t col_capacity);

/* Simple d-regular graph (d even) as the union of d/2 edge-disjoint random Hamiltonian
 * cycles; symmetric CSR into HOST buffers (col holds n*d entries). */
ABM_API int abm_graph_random_regular(int64_t n, int32_t d, uint64_t seed, int32_t* row_ptr,
                                     int32_t* col, int64_t col_capacity);

/* ---- Network CSR construction on the device ------------------------------------------ */
/* Workspace of abm_csr_from_edges for num_edges edges over n nodes (four edge-sized
 * buffers and the per-tile digit histograms). */
ABM_API size_t abm_csr_workspace_bytes(int64_t num_edges, int64_t n);

/* CSR of a directed edge list on the device: row i of (row_ptr int32[n+1], col int32[E])
 * holds dst[e] of the edges with src[e] == i in ascending e (a stable radix sort by
 * source).  Edges whose source is outside 0..n-1 are left out of every row (they follow
 * row_ptr[n] in col) and set *status to 1, as does a destination outside 0..n-1.  col must
 * not alias src or dst.  Replaces building a Network edge by edge (Network.add_edge,
 * jaxabm/agentpy.py:559-582) and the host-side sort of its edge list. */
ABM_API int abm_csr_from_edges(const int32_t* src, const int32_t* dst, int64_t num_edges,
                               int64_t n, int32_t* row_ptr, int32_t* col, int32_t* status,
                               void* workspace, size_t workspace_bytes, void* stream);

/* ---- K5: SIR contagion on a Network ------------------------------------------------- */
/* Device-side descriptor of one SIR model instance (152 bytes, 8-byte aligned).
 * words holds one byte per agent, (infected neighbours << 2) | compartment (0 S, 1 I,
 * 2 R); an agent of degree >= abm_sir_hub_degree() (a hub) has 63 in the count field and
 * its count in hub_counts[i] (int32[n]).  words is 16-byte aligned and round_up(n, 16)
 * bytes long (padding bytes read as R).  comp holds the compartments again, 2 bits per
 * agent (agent i in bits 2(i%16)..2(i%16)+1 of comp[i/16]; round_up(n,16)/16 words).
 * adj is the instance's CSR column array with bit 31 set on entries whose neighbour is a
 * hub.  All four are written by abm_sir_pack / abm_sir_pack_batch; abm_sir_unpack reads
 * the compartments back.
 * The collection key of step t is coll_keys[t] (uint32[steps][2]) when coll_keys is not
 * NULL, else it is derived from rng, the instance's Model.step key-chain state
 * (jaxabm/model.py:156,164), which is advanced once per step either way.  num_s/num_i/num_r
 * are the current compartment sizes (set by the caller before step 0); counts receives
 * S, I, R after each step (int32[steps][3]); step_si/step_ir are the transitions of the
 * step in flight (zero before step 0); done_flag (nullable, may be host-mapped) is set to
 * 1 after the last step; edges_scanned / edges_pushed accumulate the CSR slots read by
 * the decide and push phases, candidates the agents that needed a decision (susceptible
 * agents with an infected neighbour and infected agents, summed over steps) and draws the
 * infection draws made (one threefry2x32 block each; all zero before step 0). */
typedef struct abm_sir_instance {
  const int32_t* row_ptr;
  int32_t* adj;
  uint8_t* words;
  int32_t* hub_counts;
  uint32_t* comp;
  int32_t* counts;
  int32_t* done_flag;
  const uint32_t* coll_keys;
  uint32_t rng[2];
  int32_t n;
  int32_t t;
  int32_t steps;
  float beta;
  float gamma;
  int32_t num_s;
  int32_t num_i;
  int32_t num_r;
  int32_t step_si;
  int32_t step_ir;
  unsigned long long edges_scanned;
  unsigned long long edges_pushed;
  unsigned long long candidates;
  uint32_t coll[2]; /* collection key of the current step (written by abm_sir_steps) */
  unsigned long long draws;
} abm_sir_instance;

/* Bits of the status word of abm_sir_pack, abm_sir_pack_batch and abm_sir_steps_resident
 * (device int32, zeroed by the caller; bits are OR-ed in, so one word reports every kind
 * of bad input a call met). */
#define ABM_SIR_STATUS_OVERSIZE 1        /* instance larger than the resident call's max_agents */
#define ABM_SIR_STATUS_BAD_COMPARTMENT 2 /* compartment outside 0..2 (stored as R)              */
#define ABM_SIR_STATUS_BAD_COLUMN 4      /* CSR column outside 0..n-1 (replaced by a self-loop) */

/* A tile of agents [begin, end) of instance `inst` (end - begin <= abm_sir_tile_agents()). */
typedef struct abm_work_item {
  int32_t inst;
  int32_t begin;
  int32_t end;
  int32_t reserved;
} abm_work_item;

ABM_API size_t abm_sir_instance_size(void);

/* Largest tile (agents per work item) of the SIR kernels: 8192.  Words are read with
 * 128-bit loads (16 agents) where a tile's bytes are 16-byte aligned, byte loads
 * otherwise. */
ABM_API int32_t abm_sir_tile_agents(void);

/* Degree from which an agent's infected-neighbour count lives in hub_counts: 63. */
ABM_API int32_t abm_sir_hub_degree(void);

/* Words of one instance from int8 compartments state[n] (n < 2^29): compartments, hub
 * marks, infected-neighbour counts over the CSR (row_ptr[n+1], col[row_ptr[n]]); adj
 * (row_ptr[n] entries, may be col itself) receives the columns with hub tags; words
 * (16-byte aligned, round_up(n,16) bytes), hub_counts (int32[n]) and comp
 * (round_up(n,16)/16 words) as described at abm_sir_instance; sizes (device int32[3])
 * receives the S, I, R totals; *status (device int32) gets ABM_SIR_STATUS_BAD_COMPARTMENT
 * for a compartment outside 0..2 (stored as R) and ABM_SIR_STATUS_BAD_COLUMN for a column
 * outside 0..n-1 (replaced by a self-loop). */
ABM_API int abm_sir_pack(const int8_t* state, const int32_t* row_ptr, const int32_t* col,
                         int64_t n, int32_t* adj, uint8_t* words, int32_t* hub_counts,
                         uint32_t* comp, int32_t* sizes, int32_t* status, void* stream);

/* abm_sir_pack for every tile of `work` at once, in place on each descriptor's adj: the
 * int8 compartments of an instance are read from states8 at the same byte offset as its
 * words from words_base.  Descriptors must already point at their CSR, words, hub counts
 * and comp; tiles start at multiples of 16 agents. */
ABM_API int abm_sir_pack_batch(const abm_sir_instance* insts, const abm_work_item* work,
                               int32_t nwork, const int8_t* states8, const uint8_t* words_base,
                               int32_t* status, void* stream);

/* Adds the S, I and R totals of every instance's int8 compartments (laid out as for
 * abm_sir_pack_batch) to its descriptor's num_s / num_i / num_r, which the caller zeroes
 * first; compartments outside 0..2 are not counted.  Lets a server admit requests without
 * counting their compartments on the host. */
ABM_API int abm_sir_count_batch(abm_sir_instance* insts, const abm_work_item* work,
                                int32_t nwork, const int8_t* states8, const uint8_t* words_base,
                                void* stream);

/* count independent copies on one stream, one cudaMemcpyAsync each (host to device when
 * to_device is non-zero, else device to host): dst[k] <- src[k], bytes[k] bytes (0 skips the
 * entry).  Host buffers should be page-locked for the copies to be asynchronous.  One call
 * replaces a host loop of copy calls when a server admits or retires many requests. */
ABM_API int abm_copy_segments(int64_t count, void* const* dst, const void* const* src,
                              const size_t* bytes, int32_t to_device, void* stream);

/* One segment of abm_copy_segments_kernel: bytes bytes from src to dst. */
typedef struct abm_copy_segment {
  void* dst;
  const void* src;
  uint64_t bytes;
} abm_copy_segment;

/* The same copies as abm_copy_segments, done by one kernel launch instead of one
 * cudaMemcpyAsync per segment: segs[0..count) is read by the kernel, and every segs[k].dst
 * and segs[k].src is device memory or page-locked host memory (both are in the device's
 * address space); this is checked on the host for the table and every pointer
 * (cudaPointerGetAttributes), and pageable or unknown memory gives ABM_ERR_BADARG before
 * anything is launched -- copy those through abm_copy_segments.  Segments are copied with
 * 16-byte accesses where source and destination share their alignment.  When a server
 * admits or retires thousands of requests at once this replaces thousands of copy calls
 * (the host link's bandwidth is the same either way). */
ABM_API int abm_copy_segments_kernel(const abm_copy_segment* segs, int64_t count, void* stream);

/* int8 compartments of n packed words. */
ABM_API int abm_sir_unpack(const uint8_t* words, int64_t n, int8_t* state, void* stream);

/* Bytes of the list workspace of abm_sir_steps for up to max_agents live agents in up to
 * max_tiles work items: a 32-byte header {changes, overflow, candidates, live tiles, push
 * ticket, 0, 0, 0}, zeroed once by the caller, then 16 bytes per agent (a change list and
 * a candidate list),
 * then a compacted copy of the work list (16 bytes per tile, rebuilt every 8 steps from
 * the tiles of instances that can still change). */
ABM_API size_t abm_sir_changes_bytes(int64_t max_agents, int64_t max_tiles);

/* Persistent-grid sizes (CTAs of 256 threads) of the three per-step SIR kernels; 0 picks
 * the default (as many CTAs as are resident at once).  Any choice gives identical results;
 * jaxabm_gb300.autotune picks them per GPU and workload. */
typedef struct abm_sir_launch {
  int32_t sweep_grid;
  int32_t candidates_grid;
  int32_t push_grid;
  int32_t reserved;
} abm_sir_launch;

/* The default launch configuration on the current device. */
ABM_API int abm_sir_default_launch(abm_sir_launch* out);

/* nsteps synchronous SIR steps of every instance with t < steps, over the tiles `work`
 * (launch: grid sizes in host memory, NULL for the defaults).  When live_work (device int32) is not
 * NULL, only the first min(*live_work, nwork) tiles are read, so a CUDA graph of this call
 * stays valid while the number of live tiles changes.  Per step and agent i of an instance:
 * agent_key = split(coll_key, n)[i], k_inf, k_rec = split(agent_key);
 *   S -> I if some neighbour slot k with an I neighbour has uniform(k_inf,(deg,))[k] < beta;
 *   I -> R if uniform(k_rec) < gamma.
 * A susceptible agent whose word says it has no infected neighbour reads nothing else;
 * changes are pushed to the neighbours' words after all decisions (four launches per
 * step: sweep, candidates, push, finalize; with at most 256 instances the push kernel's last
 * CTA finalizes, three launches).  At most 2^26 instances.  `changes` (16-byte
 * aligned) must hold abm_sir_changes_bytes(total agents of all live instances, nwork); its
 * overflow flag is set (and changes dropped) if it is smaller.
 * Replaces Model.step's AgentCollection.update (jaxabm/model.py:163-171,
 * jaxabm/agent.py:132-179) for the SIR agent, batched over instances (the serial loops of
 * Model.batch_run, jaxabm/agentpy.py:1116-1152).  Descriptors and tiles are device memory
 * and may be rewritten between calls (e.g. to admit instances) without re-capturing a
 * CUDA graph of this call. */
ABM_API int abm_sir_steps(abm_sir_instance* insts, int32_t ninst, const abm_work_item* work,
                          int32_t nwork, const int32_t* live_work, int32_t nsteps,
                          const abm_sir_launch* launch, void* changes, size_t changes_bytes,
                          void* stream);

/* Resident path: one CTA (512 threads) per instance at a time, running all of the
 * instance's steps with its words in shared memory (decisions read neighbours'
 * compartments there, count updates are shared-memory atomics); no per-step launches.
 * abm_sir_resident_max_agents: largest instance (agents) it can hold on the current device
 * (0 without a device).  abm_sir_resident_grid: resident CTAs for instances of up to
 * max_agents agents (also sets the kernel's shared-memory opt-in, which covers the words
 * and the lists' first entries kept in shared memory; call it before capturing
 * abm_sir_steps_resident into a CUDA graph); 0 if they do not fit.
 * abm_sir_resident_scratch_bytes: scratch of abm_sir_steps_resident (a queue counter and, per
 * CTA, three lists of max_agents entries: changes, susceptible candidates, infected agents). */
ABM_API int32_t abm_sir_resident_max_agents(void);
ABM_API int32_t abm_sir_resident_grid(int32_t max_agents);
ABM_API size_t abm_sir_resident_scratch_bytes(int32_t max_agents, int32_t grid);

/* Same contract as abm_sir_steps (nsteps steps of every instance with t < steps, identical
 * results) on the resident path: CTAs take instances in the order order[0..ninst) (device
 * int32, NULL for index order; longest running first balances best -- SIRBatch predicts
 * each instance's time from its size, excess degree and beta/gamma -- and the order never
 * changes results) and run each for min(nsteps, steps - t) steps.  Every instance must have n <= max_agents; one that does
 * not is left untouched and ORs ABM_SIR_STATUS_OVERSIZE into *status (device int32,
 * zeroed by the caller).  grid
 * from abm_sir_resident_grid(max_agents); scratch 256-byte aligned.
 * With states8 and words_base (both NULL or both set: int8 compartments of an instance at
 * the same byte offset from states8 as its words from words_base, as for
 * abm_sir_pack_batch), an instance at t == 0 builds its words in the kernel from its
 * compartments (hub marks by degree, hub tags on its columns in place, infected-neighbour
 * counts, hub counts zeroed) instead of reading words, so no abm_sir_pack_batch is needed
 * before the call; without them the words and column tags must come from
 * abm_sir_pack_batch (or an earlier call).  A compartment outside 0..2 (stored as R) ORs
 * ABM_SIR_STATUS_BAD_COMPARTMENT and a column outside 0..n-1 (replaced by a self-loop)
 * ABM_SIR_STATUS_BAD_COLUMN into *status. */
ABM_API int abm_sir_steps_resident(abm_sir_instance* insts, int32_t ninst, const int32_t* order,
                                   int32_t max_agents, int32_t nsteps, int32_t grid,
                                   const int8_t* states8, const uint8_t* words_base,
                                   void* scratch, size_t scratch_bytes, int32_t* status,
                                   void* stream);

/* Workspace of abm_sir_run for n agents and num_edges = row_ptr[n] CSR entries. */
ABM_API size_t abm_sir_run_workspace_bytes(int64_t n, int64_t num_edges);

/* One SIR model for `steps` steps (the plain engine: one simulation per call) with the
 * per-step collection keys coll_keys uint32[steps][2] (abm_keychain, ncoll = 1).  A model
 * whose one-byte words fit shared memory (abm_sir_resident_max_agents) runs all steps in one
 * resident launch of one CTA; a larger one steps through the per-step kernels over the whole
 * GPU.  Both give the same results.  The CSR (row_ptr[n+1], col[num_edges]) is only read.
 * state int8[n] holds the compartments before the run and receives them after it; counts
 * int32[steps][3].  Replaces JaxModel.run stepping one SIR collection
 * (jaxabm/model.py:218-262, jaxabm/agent.py:132-179). */
ABM_API int abm_sir_run(const int32_t* row_ptr, const int32_t* col, int64_t n, int64_t num_edges,
                        int8_t* state, const uint32_t* coll_keys, int32_t steps, float beta,
                        float gamma, int32_t* counts, void* workspace, size_t workspace_bytes,
                        void* stream);

/* ---- K3/K4: Schelling segregation on a torus Grid ----------------------------------- */
/* Cell (x, y) of a W x H grid has index x*H + y; grid int8[W*H] holds -1 (empty) or the
 * occupant's type, cell_agent int32[W*H] the occupant id or -1. */
ABM_API size_t abm_schelling_workspace_bytes(int64_t n, int32_t W, int32_t H);

/* Build grid and cell_agent from agent positions pos int32[n] (cell indices) and types
 * int8[n] (>= 0).  *status (device int32) becomes 1 if a position is out of range or two
 * agents share a cell.  Replaces Grid.position_agents + the grid fill of the Schelling
 * example (jaxabm/agentpy.py:496-527, examples/models/schelling_model.py:118-133). */
ABM_API int abm_schelling_place(const int32_t* pos, const int8_t* type, int64_t n, int32_t W,
                                int32_t H, int8_t* grid, int32_t* cell_agent, int32_t* status,
                                void* stream);

/* `steps` synchronous Schelling steps with per-step collection keys coll_keys
 * uint32[steps][2]: an agent is unhappy iff thr_den*same < thr_num*occupied over its
 * Moore-8 torus neighbours (same/occupied below the threshold thr_num/thr_den; the
 * example's similarity_threshold, examples/models/schelling_model.py:36-40, as an exact
 * fraction, 0 <= thr_num, 0 < thr_den, both <= 2^27); each unhappy agent draws
 * idx = min(floor(uniform(agent_key) * e), e - 1) into the ascending list of the e
 * pre-step empty cells and claims that cell; the lowest claiming id moves.  pos, grid and
 * cell_agent are updated in place; stats int32[steps][2] receives (unhappy, moved) per
 * step.  Replaces the vmapped Agent.step of the Schelling model
 * (examples/models/schelling_model.py:33-68, jaxabm/agent.py:168-177) with the
 * neighbourhood rule and relocation it leaves as placeholders. */
ABM_API int abm_schelling_run(int32_t* pos, const int8_t* type, int64_t n, int32_t W, int32_t H,
                              int8_t* grid, int32_t* cell_agent, const uint32_t* coll_keys,
                              int32_t steps, int32_t thr_num, int32_t thr_den, int32_t* stats,
                              void* workspace, size_t workspace_bytes, void* stream);

/* One model of a Schelling batch (device descriptor, 8-byte aligned): its arrays as for
 * abm_schelling_run (grid and cell_agent placed by abm_schelling_place), its key chain
 * coll_keys uint32[steps][2], stats int32[steps][2], a workspace of
 * abm_schelling_workspace_bytes(n, W, H) bytes (256-byte aligned, no set-up needed), n
 * agents and its threshold. */
typedef struct abm_schelling_member {
  int32_t* pos;
  const int8_t* type;
  int8_t* grid;
  int32_t* cell_agent;
  const uint32_t* coll_keys;
  int32_t* stats;
  void* workspace;
  int64_t n;
  int32_t thr_num;
  int32_t thr_den;
} abm_schelling_member;

/* `count` Schelling models of one W x H grid (W*H <= 2^18) in one launch, one
 * thread-block cluster per model (the ensembles of Model.batch_run / SensitivityAnalysis,
 * jaxabm/agentpy.py:1116-1152, jaxabm/analysis.py:97-165, which the reference runs one
 * model after another).  Each model's result equals abm_schelling_run of it alone.
 * members: device array of count descriptors (count <= 8191). */
ABM_API int abm_schelling_run_batch(const abm_schelling_member* members, int32_t count,
                                    int32_t W, int32_t H, int32_t steps, void* stream);

/* ---- K8: differentiable bounded-confidence opinion model ---------------------------- */
/* B instances (B a power of two, 4 <= B <= 128) share one symmetric CSR graph; opinions
 * are interleaved o float32[n][B] (16-byte aligned); mu, eps, tau are float32[B].
 * Per step: o_i += mu * (sum_j sigmoid((eps - |o_j - o_i|) / tau) (o_j - o_i)) / deg_i.
 * The forward is a fixed sequence of float32 operations, each rounded to nearest (fused
 * multiply-adds only where written): d = o_j - o_i; z = (eps - |d|) * (1 / tau);
 * s = 1 / (1 + exp(-z)); acc = fma(s, d, acc) over the row in CSR order;
 * o_i' = fma(mu, acc / deg_i, o_i); exp is the table-driven method of Tang (ACM TOMS 15(2),
 * 1989) with x clamped to [-87, 88] (see abm_opinion_sigmoid).  Results are therefore
 * reproducible bit for bit by any IEEE-754 float32 implementation of the same sequence.
 * The reference trains such models with jit(grad(loss)) through its whole run loop
 * (jaxabm/analysis.py:494-522); these entry points give the forward pass, checkpoints and
 * the hand-written reverse pass. */

/* `steps` forward steps in place (o_tmp: scratch of the same shape).  When checkpoints is
 * not NULL, the state before step t is stored at checkpoints[t / ckpt_every] for every t
 * that is a multiple of ckpt_every. */
ABM_API int abm_opinion_run(float* o, float* o_tmp, const int32_t* row_ptr, const int32_t* col,
                            int64_t n, int32_t B, const float* mu, const float* eps,
                            const float* tau, int32_t steps, int32_t ckpt_every,
                            float* checkpoints, void* stream);

/* One forward step from o_in to o_out (distinct buffers); the reverse pass recomputes a
 * segment's states from its checkpoint with it. */
ABM_API int abm_opinion_step(const float* o_in, float* o_out, const int32_t* row_ptr,
                             const int32_t* col, int64_t n, int32_t B, const float* mu,
                             const float* eps, const float* tau, void* stream);

/* s[k] = sigmoid(z[k]) exactly as the forward step evaluates it (n values, device float32),
 * so the forward's sigmoid can be compared bit for bit with another implementation of the
 * same sequence. */
ABM_API int abm_opinion_sigmoid(const float* z, float* s, int64_t n, void* stream);

/* inv_deg float32[n] = 1 / deg_i (0 for isolated nodes), read by abm_opinion_adjoint_step. */
ABM_API int abm_opinion_inv_degree(const int32_t* row_ptr, int64_t n, float* inv_deg,
                                   void* stream);

ABM_API size_t abm_opinion_moments_workspace_bytes(int64_t n, int32_t B);

/* Raw moments m_k = mean_i o_i^k, k = 1..4, per instance -> moments float64[B][4]. */
ABM_API int abm_opinion_moments(const float* o, int64_t n, int32_t B, double* moments,
                                void* workspace, size_t workspace_bytes, void* stream);

/* Terminal adjoint lambda_i = sum_k dloss_dmoments[b][k-1] * k * o_i^(k-1) / n. */
ABM_API int abm_opinion_adjoint_init(const float* o, int64_t n, int32_t B,
                                     const double* dloss_dmoments, float* lam, void* stream);

/* Bytes of the per-CTA parameter-gradient partials (float64) of abm_opinion_adjoint_step;
 * the caller zeroes them once before the reverse sweep. */
ABM_API size_t abm_opinion_grad_workspace_bytes(int64_t n, int32_t B);

/* One reverse step at forward state o (= o^t): lam_out = lambda^t from lam_in =
 * lambda^{t+1}, and grad_partials += lambda^{t+1} . dF/d(mu, eps, tau). */
ABM_API int abm_opinion_adjoint_step(const float* o, const float* lam_in, float* lam_out,
                                     const int32_t* row_ptr, const int32_t* col,
                                     const float* inv_deg, int64_t n, int32_t B, const float* mu,
                                     const float* eps, const float* tau, double* grad_partials,
                                     size_t grad_partials_bytes, void* stream);

/* grads float64[B][3] (d/dmu, d/deps, d/dtau) from the accumulated partials. */
ABM_API int abm_opinion_grad_reduce(const double* grad_partials, int64_t n, int32_t B,
                                    double* grads, void* stream);

/* ---- K6: stable compaction (AgentList.select / AgentCollection.filter) -------------- */
ABM_API size_t abm_select_workspace_bytes(int64_t n);

/* Indices i (ascending) with mask[i] != 0 -> out_idx int32[n]; *count (device int64)
 * receives how many.  Replaces `int(jnp.sum(mask))` and the boolean-mask gather of
 * AgentCollection.filter (jaxabm/agent.py:227-242) / AgentList.select
 * (jaxabm/agentpy.py:316-345).  n <= 2^31 - 1. */
ABM_API int abm_select_indices(const uint8_t* mask, int64_t n, int32_t* out_idx, int64_t* count,
                               void* workspace, size_t workspace_bytes, void* stream);

/* Compaction by a simple condition, without a mask array: the condition is a postfix
 * program of at most 16 operations over at most 4 attribute arrays of n entries.
 * ABM_SELECT_LT..NE push (attrs[op.attr][i] <op> op.value) -- float32 attributes compare
 * in float32 with value rounded to float32 (as a float32 array compared with a Python
 * number does), integer attributes compare exactly; ABM_SELECT_AND / OR pop two flags and
 * push one; ABM_SELECT_NOT flips the top.  The program must leave exactly one flag.
 * Output as abm_select_indices (ascending indices, *count), workspace of
 * abm_select_workspace_bytes(n).  Replaces the eager boolean mask of AgentList.select /
 * AgentCollection.filter (jaxabm/agentpy.py:316-345, jaxabm/agent.py:213-243) for
 * conditions such as (s["x"] > 0.5) & ~(s["state"] == 2). */
#define ABM_SELECT_LT 1
#define ABM_SELECT_LE 2
#define ABM_SELECT_GT 3
#define ABM_SELECT_GE 4
#define ABM_SELECT_EQ 5
#define ABM_SELECT_NE 6
#define ABM_SELECT_AND 7
#define ABM_SELECT_OR 8
#define ABM_SELECT_NOT 9
#define ABM_SELECT_F32 0
#define ABM_SELECT_I32 1
#define ABM_SELECT_I8 2
#define ABM_SELECT_U8 3
typedef struct abm_select_attr {
  const void* data; /* device array of n entries */
  int32_t dtype;    /* ABM_SELECT_F32 / I32 / I8 / U8 (bool) */
  int32_t reserved;
} abm_select_attr;
typedef struct abm_select_op {
  int32_t code;
  int32_t attr;  /* attribute index of a comparison */
  double value;  /* constant of a comparison */
} abm_select_op;
ABM_API int abm_select_where(const abm_select_attr* attrs, int32_t nattrs,
                             const abm_select_op* program, int32_t nops, int64_t n,
                             int32_t* out_idx, int64_t* count, void* workspace,
                             size_t workspace_bytes, void* stream);

/* Same result as abm_select_indices, without any workspace and without allocating.
 * No counterpart in the reference (it allocates through JAX for every selection).
 * For callers that cannot allocate device memory when they select: a host application
 * that gives the engine a fixed device-memory budget, or a latency-critical loop that must
 * not risk the device-wide synchronisation cudaMalloc/cudaFree can cause.  Its scratch is a
 * fixed 192 KiB array inside the library's device image, held by every GPU that loads the
 * library until the process exits.  Limit: n <= 67,108,864 (2^26); larger n returns
 * ABM_ERR_BADARG (use abm_select_indices).  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress, with that device current); make that first
 * call before any stream capture.  The address is kept with the id of the CUDA context it
 * belongs to; the first call in a new context of the device (after cudaDeviceReset, or
 * once the primary context was destroyed and created again) looks it up again, so make
 * that call outside any stream capture too.  All calls share the one array, so calls that
 * overlap on the GPU (other streams, other host threads) race: serialise them on one
 * stream. */
ABM_API int abm_select_indices_noalloc(const uint8_t* mask, int64_t n, int32_t* out_idx,
                                       int64_t* count, void* stream);

/* dst[r] = src[idx[r]] for `count` rows of `row_bytes` bytes (the per-attribute
 * `v[mask]` of jaxabm/agent.py:242). */
ABM_API int abm_gather_rows(const void* src, int64_t nrows_src, int64_t row_bytes,
                            const int32_t* idx, int64_t count, void* dst, void* stream);

/* ---- K7: reductions (AgentCollection.aggregate, jaxabm/agent.py:198-211) ------------ */
#define ABM_REDUCE_SUM 0
#define ABM_REDUCE_MEAN 1
#define ABM_REDUCE_MIN 2
#define ABM_REDUCE_MAX 3
ABM_API size_t abm_reduce_workspace_bytes(int64_t n);
/* *out (device float) = op over x[0..n); sums accumulate in float64; min and max return
 * NaN when any input is NaN (as jnp.min / jnp.max do). */
ABM_API int abm_reduce_f32(const float* x, int64_t n, int op, float* out, void* workspace,
                           size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* JAXABM_GB300_H */

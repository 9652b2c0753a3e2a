// Host side of libsopgpu.so: the context, device memory layout, the step
// loop captured as CUDA graphs, overflow recovery and the C ABI
// (include/sop_gpu.h).
//
// Replaces the reference's device-side host code: alloc_GPU_arrays /
// alloc_cudpp / setup_rng (GPUvars.cu:99-293, 417-453), force_eval /
// random_force (energy.cu:81-167), underdamped_iteration (sop.cu:466-484),
// update_neighbor_list / update_pair_list (sop.cu:928-1262, 1456-1706) and the
// per-step loop body of underdamped_ctrl (sop.cu:197-243).
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "sop_dev.cuh"
#include "../../include/sop_gpu.h"

namespace sop {
// kernels_lists.cu
struct NLScratch {
  int* ncell;
  int* block_sums;
  int* cells_total;
};
void launch_nl_rebuild(const DevSys& s, const NLScratch& w, int koff, cudaStream_t st);
void launch_pl_rebuild(const DevSys& s, int koff, cudaStream_t st);
void launch_rebin(const DevSys& s, const NLScratch& w, cudaStream_t st);
void launch_scan(const int* in, long long n, int* out, int* block_sums, cudaStream_t st);
long long scan_block_sums_needed(long long n);
// kernels_step.cu
void launch_step(const DevSys& s, int G, bool split, int koff, bool step, int wcap,
                 cudaStream_t st);
cudaError_t allow_step_window(int wcap);
cudaError_t launch_step_block(const DevSys& s, int G, int koff0, int count, bool step,
                              cudaStream_t st);
cudaError_t launch_step_persist(const DevSys& s, int G, int koff0, int count, bool step,
                                unsigned* bar, unsigned long long limit_ns, cudaStream_t st);
cudaError_t launch_barrier_check(const DevSys& s, int G, unsigned* bar, int missing, int rounds,
                                 unsigned long long limit_ns, cudaStream_t st);
void launch_step_tiles(const DevSys& s, int koff, bool step, const int4* tiles, int ntiles,
                       bool any_split, cudaStream_t st);
void launch_advance(const DevSys& s, int steps, cudaStream_t st);
void launch_gather_current(const DevSys& s, float* out, int* flag_out, cudaStream_t st);
void launch_energy(const DevSys& s, int mol_start, int mol_n, int m, double* part, double* out,
                   double k_bnd_R0sq_half, cudaStream_t st);
void launch_observables(const DevSys& s, int mol_start, int mol_n, int m, int nnat,
                        double* part, double* out, cudaStream_t st);
}  // namespace sop

using namespace sop;

namespace {

std::string g_lib_error;

struct HostMol {
  int n = 0;
  std::vector<int> bi, bj, ai, ak, ni, nj, types;
  std::vector<float> br0, nr0, neps, nepse, unc, pos, vel;
  double T = 0.6;
  unsigned traj = 0;
  long long nsteps = -1;
  int start = -1;                 // first bead slot; -1: not on the device
  int slot = -1;                  // molecule slot
  long long off_b = 0, off_a = 0, off_n = 0;  // topology pool offsets
};

// Capacities of the device pools.
struct Caps {
  long long beads = 0, mols = 0, bonds = 0, angles = 0, natives = 0, cells = 0;
  long long max_mol_beads = 0, stride = 64;
};

// First-fit allocator of ranges in [0, cap), coalescing on release.
struct RangeAlloc {
  long long cap = 0;
  std::map<long long, long long> free_;  // start -> length
  void reset(long long c) {
    cap = c;
    free_.clear();
    if (c > 0) free_[0] = c;
  }
  long long alloc(long long n) {
    if (n <= 0) return 0;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      long long st = it->first, len = it->second;
      free_.erase(it);
      if (len > n) free_[st + n] = len - n;
      return st;
    }
    return -1;
  }
  void release(long long st, long long n) {
    if (n <= 0) return;
    auto it = free_.emplace(st, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  // one past the last allocated position (0 when nothing is allocated)
  long long high_water() const {
    if (free_.empty()) return cap;
    auto last = std::prev(free_.end());
    return last->first + last->second == cap ? last->first : cap;
  }
  long long largest() const {
    long long m = 0;
    for (auto& kv : free_) m = std::max(m, kv.second);
    return m;
  }
};

// sigma_rep[itype][jtype] (energy.cu:9-13)
const float kSigmaRep[3][3] = {{0.f, 0.f, 0.f}, {0.f, 3.8f, 5.4f}, {0.f, 5.4f, 7.0f}};

// The reference's cut-off: rcut = fac * r in double, rounded to FP32
// (sop.cu:746-747), or an absolute value; squared in FP32.
float rcut_of(double fac, double absval, float r) {
  return (fac > 0.0) ? (float)(fac * (double)r) : (float)absval;
}
float rcut2_of(double fac, double absval, float r) {
  float rc = rcut_of(fac, absval, r);
  return rc * rc;
}

float bits_f(int v) {
  float f;
  std::memcpy(&f, &v, sizeof f);
  return f;
}
int bits_i(float v) {
  int i;
  std::memcpy(&i, &v, sizeof i);
  return i;
}

struct Graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
};

// A served job: queued (its molecule on the host), active (in a molecule
// slot) or finished (its results on the host).
struct Job {
  enum { QUEUED = 0, ACTIVE = 1, FINISHED = 2 };
  HostMol mol;
  int state = QUEUED;
  int slot = -1;
  int n = 0;
  long long nsteps = 0;
  double t_submit = 0.0, t_done = 0.0;
  std::vector<float> unc, vel;
  double energy[5] = {0, 0, 0, 0, 0};
  int status = 0;
  long long steps = 0;
  std::vector<char> resume;   // checkpoint to continue from (empty: start at step 0)
  long long resume_step = 0;
};

double now_seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct SopCtx {
  sop_params P{};
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<HostMol> mols;
  bool committed = false;

  DevSys s{};
  std::vector<void*> allocs;
  std::map<void*, size_t> alloc_bytes;
  long long bytes = 0;
  NLScratch w{};
  int G = 8;
  bool split = false;         // step as force kernel + finish kernel
  int wcap = 0;               // > 0: step blocks stage their molecules (up to wcap beads)
  bool persist = false;       // steps between list rebuilds in one cooperative launch
  bool one_block = false;     // steps between list rebuilds in one block
  // tiled form: per-molecule tiles, lanes and form chosen per size bucket
  bool tiled = false;
  int4* d_tiles = nullptr;    // {first bead, end bead, lanes, two-kernel form}
  int ntiles = 0;
  bool tiles_split = false;   // some bucket uses the two-kernel form (k_finish follows)
  int bucket_lanes[3] = {0, 0, 0}, bucket_form[3] = {0, 0, 0};
  long long bucket_beads[3] = {0, 0, 0};
  float ms_tiled = 0.f, ms_whole = 0.f;  // tuning times of the two step layouts
  double* e_part = nullptr;   // energy / observable partials
  double* e_out = nullptr;    // 8 doubles
  double* h_out = nullptr;    // pinned copy of e_out
  float4* stage = nullptr;    // gather buffer of sop_download_all
  // sop_download_all_async: two gather buffers (packed xyz, then the
  // overflow flag the gather saw), a copy stream, and per buffer the events
  // of its gather and of its copy to the host
  cudaStream_t copy_stream = nullptr;
  float4* astage[2] = {nullptr, nullptr};
  cudaEvent_t gathered[2] = {nullptr, nullptr};
  cudaEvent_t copied[2] = {nullptr, nullptr};
  int* h_flag = nullptr;      // pinned: the flag of each buffer's last copy
  long long next_ticket = 0;
  std::map<int, float> tuning;  // step time (ms) per lanes-per-bead candidate (its faster form)
  Caps caps;
  MolConst* dmol = nullptr;
  RangeAlloc bead_alloc, bond_alloc, ang_alloc, nat_alloc;
  std::vector<int> free_slots;  // molecule slots not in use (back = next)
  // serving
  bool served = false;
  long long budget = 0;
  std::vector<Job> jobs;
  std::deque<int> queue;          // queued job ids in arrival order
  std::vector<int> slot_job;      // job in each molecule slot, -1: free
  std::vector<int> finished_new;  // finished since the last sop_serve_finished
  bool stepped = false;       // a step was queued since the context was committed
  long long host_step = 0;    // common step of plain / batched contexts
  long long target_step = 0;  // step every molecule should reach after the queued work
  std::map<std::string, Graph> graphs;
  std::vector<MolConst> mc;

  ~SopCtx() { release(); }

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return SOP_ERR_CUDA;
  }
  template <class T>
  T* dalloc(size_t count) {
    void* p = nullptr;
    size_t b = sizeof(T) * (count ? count : 1);
    if (cudaMalloc(&p, b) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    allocs.push_back(p);
    alloc_bytes[p] = b;
    bytes += (long long)b;
    return (T*)p;
  }
  void dfree(void* p) {
    if (!p) return;
    auto it = std::find(allocs.begin(), allocs.end(), p);
    if (it != allocs.end()) allocs.erase(it);
    auto sz = alloc_bytes.find(p);
    if (sz != alloc_bytes.end()) {
      bytes -= (long long)sz->second;
      alloc_bytes.erase(sz);
    }
    cudaFree(p);
  }
  void drop_graphs() {
    for (auto& kv : graphs) {
      if (kv.second.e) cudaGraphExecDestroy(kv.second.e);
      if (kv.second.g) cudaGraphDestroy(kv.second.g);
    }
    graphs.clear();
  }
  void release() {
    if (copy_stream) cudaStreamSynchronize(copy_stream);  // copies into caller memory
    for (int k = 0; k < 2; ++k) {
      if (gathered[k]) cudaEventDestroy(gathered[k]);
      if (copied[k]) cudaEventDestroy(copied[k]);
      gathered[k] = copied[k] = nullptr;
    }
    if (copy_stream) cudaStreamDestroy(copy_stream);
    copy_stream = nullptr;
    if (h_flag) cudaFreeHost(h_flag);
    h_flag = nullptr;
    drop_graphs();
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    if (h_out) cudaFreeHost(h_out);
    h_out = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

static SopCtx* C(void* p) { return static_cast<SopCtx*>(p); }

int grow_nl_keep(SopCtx* ctx, long long stride);

#define CK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return ctx->cuda_fail(e_, #call); \
  } while (0)

namespace {

int graph_steps(const SopCtx* ctx);

// The rows of the molecule whose beads are o .. o + n - 1 in the repulsive
// neighbour list (r = 0) or pair list (r = 1), every entry as an index
// relative to bead o (as stored), full row stride.
int read_rows(SopCtx* ctx, int r, int o, int n, std::vector<int>& rows) {
  const long long stride = ctx->s.nl_stride, len = stride * n;
  rows.assign((size_t)len, 0);
  if (!len) return SOP_OK;
  std::vector<unsigned short> h((size_t)len);
  CK(cudaMemcpy(h.data(), (r == 0 ? ctx->s.nl_j : ctx->s.pl_j) + (long long)o * stride,
                sizeof(unsigned short) * len, cudaMemcpyDeviceToHost));
  for (size_t k = 0; k < h.size(); ++k) rows[k] = h[k];
  return SOP_OK;
}

int lanes_for(const SopCtx* ctx) {
  int g = ctx->P.lanes_per_bead;
  if (g == 2 || g == 4 || g == 8 || g == 16) return g;
  return 0;  // autotune
}

// The step's form: 1 one kernel, 2 force kernel + finish kernel, 3 every
// step between two list rebuilds in one cooperative launch, 4 the same in
// one block, 0 autotuned.
int split_for(const SopCtx* ctx) {
  const int f = ctx->P.step_split;
  return (f >= 1 && f <= 4) ? f : 0;
}

// Contexts of up to this many bead slots let the tuner try the one-block
// form (one SM does every bead: larger ones are faster spread over the GPU).
constexpr int kOneBlockMaxBeads = 2048;

// Wait limit of the persistent form's device-wide barrier: a step of the
// largest context takes well under a millisecond.
constexpr unsigned long long kBarrierLimitNs = 2000000000ull;

unsigned* barrier_words(SopCtx* ctx) { return reinterpret_cast<unsigned*>(ctx->s.flags + 2); }

// The step's window: sop_params.step_window > 0 fixes it, < 0 turns it off,
// 0 lets the autotuner choose.
int window_param(const SopCtx* ctx) { return ctx->P.step_window; }
constexpr int kMaxStepWindow = 12288;  // 192 KB of shared memory per block
constexpr int kMaxMolBeads = 65535;    // 16-bit molecule-relative pair-list partners

// Picks the lanes per bead G and the form (one kernel or two) of the step
// for this context by timing the force-only step (idempotent: it recomputes
// the same forces and look-ahead from the same state) for each candidate not
// fixed by the parameters; results are bit-identical for every G, form and
// window, so only the speed differs.  A fixed window or the persistent form
// (step_window > 0, step_split = 3) is timed as given.
// Timed launches per tuning candidate (after one warm-up): step times repeat
// to about 1%, and the candidates the tuner separates differ by more.
constexpr int kTuneReps = 2;

int autotune_lanes(SopCtx* ctx) {
  const int fixed_g = lanes_for(ctx), fixed_f = split_for(ctx), fixed_w = window_param(ctx);
  const int cand[4] = {2, 4, 8, 16};
  // the shared-memory window and the persistent form are measured slower
  // than global gathers and per-step launches on every workload, so they are
  // used where the parameters ask for them and not tried here
  std::vector<int> wins = {(!ctx->served && fixed_w > 0) ? fixed_w : 0};
  // the opt-in is a per-kernel ceiling shared by every context of the
  // process: always the same (largest) value, so contexts never lower it
  // under one another; each launch asks for its own window only
  if (wins.size() > 1 || wins[0] > 0) CK(allow_step_window(kMaxStepWindow));
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  // steps between two list rebuilds (the pair list's cadence, at most a graph)
  const int run_len = std::max(1, std::min(graph_steps(ctx), ctx->P.nplup > 1 ? ctx->P.nplup : 1));
  float best = 1e30f;
  int bestg = fixed_g ? fixed_g : 8;
  int bestf = fixed_f ? fixed_f : 1;
  int bestw = wins[0];
  for (int g : cand) {
    if (fixed_g && g != fixed_g) continue;
    float gbest = 1e30f;
    for (int f = 1; f <= 4; ++f) {
      if (fixed_f ? f != fixed_f : (f == 3 || (f == 4 && ctx->s.nlive > kOneBlockMaxBeads)))
        continue;
      if (f >= 3 && ctx->served) continue;
      const bool sp = f == 2;
      for (int wc : wins) {
        if (f >= 3 && wc != 0) continue;
        // kTuneReps force-only evaluations (idempotent): as many launches,
        // or one persistent launch (with barriers between them)
        auto run = [&](int reps) -> cudaError_t {
          if (f == 3)
            return launch_step_persist(ctx->s, g, 0, reps, false, barrier_words(ctx),
                                       kBarrierLimitNs, ctx->stream);
          if (f == 4) return launch_step_block(ctx->s, g, 0, reps, false, ctx->stream);
          for (int r = 0; r < reps; ++r) launch_step(ctx->s, g, sp, 0, false, wc, ctx->stream);
          return cudaGetLastError();
        };
        // a form that runs every step between two rebuilds in one launch is
        // timed over such a run (its launch is paid once per run); the
        // others pay their launches per step, so two steps show their cost
        const int reps = f == 4 ? run_len : kTuneReps;
        CK(run(1));  // warm-up
        CK(cudaEventRecord(a, ctx->stream));
        CK(run(reps));
        CK(cudaEventRecord(b, ctx->stream));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, a, b));
        ms /= (float)reps;  // per step
        gbest = std::min(gbest, ms);
        if (ms < best) { best = ms; bestg = g; bestf = f; bestw = wc; }
      }
    }
    ctx->tuning[g] = gbest;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  int flags = 0;
  CK(cudaMemcpy(&flags, ctx->s.flags, sizeof(int), cudaMemcpyDeviceToHost));
  if (flags & FLAG_BARRIER_TIMEOUT)
    return ctx->fail(SOP_ERR_CUDA, "the persistent step's barrier timed out while tuning");
  ctx->G = bestg;
  ctx->split = bestf == 2;
  ctx->persist = bestf == 3;
  ctx->one_block = bestf == 4;
  ctx->wcap = bestw;
  return SOP_OK;
}

// (Re)allocates the fixed-stride neighbour / pair-list rows.
int alloc_nl(SopCtx* ctx, long long stride) {
  stride = (stride + 31) / 32 * 32;  // rows stay 64-byte aligned
  const long long entries = stride * (long long)ctx->s.nbead;
  // rows are addressed with 64-bit offsets; the bound only keeps the byte
  // count (two arrays of 16-bit entries) far from overflow
  if (entries > (1LL << 40)) return ctx->fail(SOP_ERR_CAPACITY, "neighbour list exceeds 2^40 entries");
  ctx->dfree(ctx->s.nl_j);
  ctx->dfree(ctx->s.pl_j);
  ctx->s.nl_j = ctx->dalloc<unsigned short>(entries);
  ctx->s.pl_j = ctx->dalloc<unsigned short>(entries);
  if (!ctx->s.nl_j || !ctx->s.pl_j) return ctx->fail(SOP_ERR_ALLOC, "neighbour-list allocation failed");
  ctx->s.nl_stride = stride;
  ctx->drop_graphs();  // kernel arguments changed
  return SOP_OK;
}

// After a neighbour-list overflow: regrow the row stride to 1.25x the longest
// row the rebuild needed and clear the flag.  The rows are kept: the rebuild
// that runs again rewrites those of the molecules it covers, and a molecule
// it does not cover (finished or stopped) keeps the lists of its last step,
// which its energy is evaluated on.  The stream must be idle.
int grow_nl(SopCtx* ctx) {
  int maxrow = 0;
  CK(cudaMemcpy(&maxrow, ctx->s.nl_maxrow, sizeof(int), cudaMemcpyDeviceToHost));
  long long stride = std::max<long long>(ctx->s.nl_stride + 32, (long long)maxrow * 5 / 4 + 32);
  int rc = grow_nl_keep(ctx, stride);
  if (rc) return rc;
  CK(cudaMemsetAsync(ctx->s.nl_maxrow, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->s.flags, 0, sizeof(int), ctx->stream));
  return SOP_OK;
}

// Neighbour-list rebuild that regrows the rows on overflow and rebuilds
// again; only_mol >= 0 rebuilds that molecule's lists alone.  Synchronous.
int nl_rebuild_checked(SopCtx* ctx, int koff, int only_mol = -1) {
  for (int attempt = 0; attempt < 4; ++attempt) {
    DevSys s = ctx->s;  // re-read: a regrow changes the rows
    s.only_mol = only_mol;
    launch_nl_rebuild(s, ctx->w, koff, ctx->stream);
    CK(cudaGetLastError());
    int flags = 0;
    CK(cudaMemcpyAsync(&flags, ctx->s.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!(flags & FLAG_NL_OVERFLOW)) return SOP_OK;
    int rc = grow_nl(ctx);
    if (rc) return rc;
  }
  return ctx->fail(SOP_ERR_CAPACITY, "neighbour list kept overflowing");
}

void force_eval_async(SopCtx* ctx) {
  launch_step(ctx->s, ctx->G, ctx->split, 0, false, ctx->wcap, ctx->stream);
}

// Step kernels for steps koff0 .. koff0 + count - 1 of a block (no rebuild
// among them): one persistent launch, or one launch per step.
void launch_steps(SopCtx* ctx, int koff0, int count) {
  if (count <= 0) return;
  if (ctx->tiled) {
    for (int k = koff0; k < koff0 + count; ++k)
      launch_step_tiles(ctx->s, k, true, ctx->d_tiles, ctx->ntiles, ctx->tiles_split, ctx->stream);
    return;
  }
  if (ctx->persist) {
    launch_step_persist(ctx->s, ctx->G, koff0, count, true, barrier_words(ctx), kBarrierLimitNs,
                        ctx->stream);
    return;
  }
  if (ctx->one_block) {
    launch_step_block(ctx->s, ctx->G, koff0, count, true, ctx->stream);
    return;
  }
  for (int k = koff0; k < koff0 + count; ++k)
    launch_step(ctx->s, ctx->G, ctx->split, k, true, ctx->wcap, ctx->stream);
}

// Which rebuilds precede step n (1-based): bit 0 neighbour list, bit 1 pair list.
int rebuilds_before(const sop_params& P, long long n) {
  int r = 0;
  if (P.nnlup > 0 && n % P.nnlup == 0) r |= 1;
  if ((r & 1) || P.nplup <= 1 || n % P.nplup == 0) r |= 2;
  return r;
}

// Launch sequence of steps s0+1 .. s0+count and the step-count advance.
// The clocks advance ahead of every neighbour-list rebuild by the steps run
// since the last advance, and koff counts from there: a rebuild that
// overflows the rows then stops every later kernel of the block with the
// clocks at the rebuild, and the steps before it, already done, are not run
// again when the host regrows the rows and replays from the clock.
void enqueue_block(SopCtx* ctx, long long s0, int count) {
  int run0 = 0;  // first step of the current run without rebuilds
  int base = 0;  // steps of the block the clocks already count
  for (int k = 0; k < count; ++k) {
    int r = rebuilds_before(ctx->P, s0 + 1 + k);
    if (r) {
      launch_steps(ctx, run0 - base, k - run0);
      run0 = k;
    }
    if ((r & 1) && k > base) {
      launch_advance(ctx->s, k - base, ctx->stream);
      base = k;
    }
    if (r & 1) launch_nl_rebuild(ctx->s, ctx->w, k - base, ctx->stream);
    if (r & 2) launch_pl_rebuild(ctx->s, k - base, ctx->stream);
  }
  launch_steps(ctx, run0 - base, count - run0);
  launch_advance(ctx->s, count - base, ctx->stream);
}

int graph_for(SopCtx* ctx, long long s0, int count, cudaGraphExec_t* out) {
  std::string key(count, '0');
  for (int k = 0; k < count; ++k) key[k] = (char)('0' + rebuilds_before(ctx->P, s0 + 1 + k));
  auto it = ctx->graphs.find(key);
  if (it != ctx->graphs.end()) {
    *out = it->second.e;
    return SOP_OK;
  }
  Graph g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_block(ctx, s0, count);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g.g);
  if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&g.e, g.g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g.g);
    return ctx->cuda_fail(e, "cudaGraphInstantiate");
  }
  ctx->graphs[key] = g;
  *out = g.e;
  return SOP_OK;
}

int graph_steps(const SopCtx* ctx) {
  int P = ctx->P.graph_steps > 0 ? ctx->P.graph_steps : 10;
  return P;
}

// Queues nsteps steps of every molecule (no synchronisation).
int step_async(SopCtx* ctx, long long nsteps) {
  const int P = graph_steps(ctx);
  if (nsteps > 0) ctx->stepped = true;
  long long s0 = ctx->host_step;
  long long left = nsteps;
  while (left > 0) {
    long long phase = s0 % P;
    if (phase == 0 && left >= P) {
      cudaGraphExec_t ge;
      int rc = graph_for(ctx, s0, P, &ge);
      if (rc) return rc;
      CK(cudaGraphLaunch(ge, ctx->stream));
      s0 += P;
      left -= P;
    } else {
      int cnt = (int)std::min<long long>(left, P - phase);
      enqueue_block(ctx, s0, cnt);
      CK(cudaGetLastError());
      s0 += cnt;
      left -= cnt;
    }
  }
  ctx->host_step = s0;
  ctx->target_step = s0;
  return SOP_OK;
}

// Waits for queued work; on a neighbour-list overflow regrows the list and
// re-runs the steps that were skipped.
// A timed-out wait of the persistent step's barrier leaves the steps it was
// running half done: the flag and the barrier words are cleared (so the
// context can be restored from a checkpoint) and the failure reported.
int barrier_failure(SopCtx* ctx) {
  CK(cudaMemsetAsync(ctx->s.flags, 0, 4 * sizeof(int), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return ctx->fail(SOP_ERR_CUDA,
                   "the persistent step's device-wide barrier timed out; the state of the "
                   "steps it was running is undefined");
}

int sync_checked(SopCtx* ctx) {
  for (int round = 0; round < 8; ++round) {
    int flags = 0;
    CK(cudaMemcpyAsync(&flags, ctx->s.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (flags & FLAG_BARRIER_TIMEOUT) return barrier_failure(ctx);
    if (!(flags & FLAG_NL_OVERFLOW)) return SOP_OK;
    // Every molecule froze at the neighbour-list rebuild that overflowed,
    // and the context's clock with them (enqueue_block advances the clocks
    // ahead of each such rebuild).
    long long done = 0;
    CK(cudaMemcpy(&done, ctx->s.sys_step, sizeof(long long), cudaMemcpyDeviceToHost));
    int rc = grow_nl(ctx);
    if (rc) return rc;
    long long target = ctx->target_step;
    ctx->host_step = done;
    rc = step_async(ctx, target - done);
    if (rc) return rc;
  }
  return ctx->fail(SOP_ERR_CAPACITY, "neighbour list kept overflowing");
}

MolConst make_const(const sop_params& P, const HostMol& hm) {
  MolConst c{};
  c.start = hm.start;
  c.n = hm.n;
  double h = P.h, z = P.zeta, T = hm.T, halfh = h / 2.0;
  c.a1 = (float)(h * (1.0 - z * halfh));
  c.a2 = (float)(h * halfh);
  c.a3 = (float)((1.0 - h * z / 2.0 + (h * z) * (h * z) / 4.0) / h);
  c.a4 = (float)(halfh * (1.0 - h * z / 2.0));
  if (P.integrator == 1) {
    // overdamped: incr = a5 f (sop.cu:495-497), a5 = h / zeta (param.cpp:110).
    // The step kernel's incr = fma(a1, v, a2 f) with a1 = 0 and a zero
    // velocity is exactly that product, and v = a3 incr + a4 f stays 0.
    c.a1 = 0.0f;
    c.a2 = (float)(h / z);
    c.a3 = 0.0f;
    c.a4 = 0.0f;
  }
  c.sigma_f = (float)std::sqrt(2.0 * T * z / h);
  c.t_zero = T < 1.0e-5 ? 1 : 0;
  c.traj = hm.traj;
  c.active = 1;
  c.nsteps = hm.nsteps;
  return c;
}

// Scalar constants of the force field and the lists (DevSys fields).
void set_constants(SopCtx* ctx) {
  const sop_params& P = ctx->P;
  DevSys& s = ctx->s;
  s.boxl = (float)P.boxl;
  s.eps_rep = (float)P.eps_rep;
  s.rep6 = P.rep6;
  s.k_bnd = (float)P.k_bnd;
  s.R0 = (float)P.R0;
  s.R0sq = (float)(P.R0 * P.R0);
  s.inv_R0sq = (float)(1.0 / (P.R0 * P.R0));
  double sig6 = std::pow(P.sigma_ss, 6.0);
  s.f_ss = (float)(6.0 * P.eps_ss * sig6);
  s.e_ss = (float)(P.eps_ss * sig6);
  float rcmax = 0.f;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      float sg = kSigmaRep[a][b];
      s.sig2[a][b] = sg * sg;
      s.rep_tol[a][b] = sg * 1.0e-7f;
      s.rc2_nl_rep[a][b] = rcut2_of(P.nl_rep_fac, P.nl_rep_abs, sg);
      s.rc2_pl_rep[a][b] = rcut2_of(P.pl_rep_fac, P.pl_rep_abs, sg);
      if (a > 0 && b > 0) rcmax = std::max(rcmax, rcut_of(P.nl_rep_fac, P.nl_rep_abs, sg));
    }
  s.rc_nl_rep_max = rcmax;
  s.seed_lo = (unsigned)(P.seed & 0xffffffffULL);
  s.seed_hi = (unsigned)(P.seed >> 32);
}

// Device arrays sized by capacities: beads, molecule slots, topology entries
// (each pair counted for both beads).  Free bead slots have mol_of = -1.
int alloc_pools(SopCtx* ctx, const Caps& c) {
  DevSys& s = ctx->s;
  ctx->caps = c;
  const size_t nb = (size_t)c.beads, nm = (size_t)c.mols;
  s.nbead = (int)c.beads;
  s.nlive = s.nbead;
  s.only_mol = -1;
  s.nmol = (int)c.mols;
  for (int b = 0; b < 2; ++b) {
    s.x[b] = ctx->dalloc<float4>(nb);
    s.p[b] = ctx->dalloc<float4>(nb);
  }
  s.v = ctx->dalloc<float4>(nb);
  s.incr = ctx->dalloc<float4>(nb);
  s.f = ctx->dalloc<float4>(nb);
  s.fsum = ctx->dalloc<float4>(nb);
  s.mol_of = ctx->dalloc<int>(nb);
  ctx->dmol = ctx->dalloc<MolConst>(nm);
  s.mol = ctx->dmol;
  s.mol_step = ctx->dalloc<long long>(nm);
  s.mol_status = ctx->dalloc<int>(nm);
  s.sys_step = ctx->dalloc<long long>(1);
  s.bond_row = ctx->dalloc<int2>(nb);
  s.ang_row = ctx->dalloc<int2>(nb);
  s.nat_row = ctx->dalloc<int2>(nb);
  s.bond_j = ctx->dalloc<int>(c.bonds);
  s.bond_r0 = ctx->dalloc<float>(c.bonds);
  s.ang_j = ctx->dalloc<int>(c.angles);
  s.nat_j = ctx->dalloc<int>(c.natives);
  s.nat_par = ctx->dalloc<float4>(c.natives);
  s.nat_rc2 = ctx->dalloc<float2>(c.natives);
  s.nl_att_cnt = ctx->dalloc<int>(nb);
  s.pl_att_cnt = ctx->dalloc<int>(nb);
  s.nl_att_e = ctx->dalloc<int>(c.natives);
  s.pl_att = ctx->dalloc<float4>(c.natives);
  s.nl_cnt = ctx->dalloc<int>(nb);
  s.pl_cnt = ctx->dalloc<int>(nb);
  s.nl_maxrow = ctx->dalloc<int>(1);
  s.nl_j = nullptr;
  s.pl_j = nullptr;
  int rc = alloc_nl(ctx, c.stride);
  if (rc) return rc;
  s.bbox = ctx->dalloc<unsigned>(6 * nm);
  s.grid = ctx->dalloc<MolGrid>(nm);
  s.cell_cap = c.cells;
  s.cell_cnt = ctx->dalloc<int>(c.cells);
  s.cell_start = ctx->dalloc<int>(c.cells + 1);
  s.bead_cell = ctx->dalloc<int>(nb);
  s.bead_slot = ctx->dalloc<int>(nb);
  s.sorted = ctx->dalloc<int>(nb);
  s.xs = ctx->dalloc<float4>(nb);
  s.flags = ctx->dalloc<int>(4);  // [0] flags, [2..3] the persistent step's barrier
  s.noise = nullptr;
  s.use_noise = 0;
  ctx->w.ncell = ctx->dalloc<int>(nm);
  ctx->w.block_sums = ctx->dalloc<int>(scan_block_sums_needed(std::max<long long>(c.cells, nb)));
  ctx->w.cells_total = ctx->dalloc<int>(1);
  ctx->e_part = ctx->dalloc<double>(6 * ((size_t)c.max_mol_beads / 256 + 2));
  ctx->e_out = ctx->dalloc<double>(8);
  if (!s.x[0] || !s.x[1] || !s.p[0] || !s.p[1] || !s.v || !s.incr || !s.f || !s.fsum || !s.mol_of ||
      !s.mol || !s.mol_step || !s.mol_status || !s.sys_step || !s.bond_row || !s.ang_row ||
      !s.nat_row || !s.bond_j || !s.bond_r0 || !s.ang_j || !s.nat_j || !s.nat_par ||
      !s.nat_rc2 || !s.nl_att_cnt || !s.pl_att_cnt || !s.nl_att_e || !s.pl_att || !s.nl_cnt ||
      !s.pl_cnt || !s.nl_maxrow || !s.bbox || !s.grid || !s.cell_cnt || !s.cell_start ||
      !s.bead_cell || !s.bead_slot || !s.sorted || !s.xs || !s.flags || !ctx->w.ncell ||
      !ctx->w.block_sums || !ctx->w.cells_total || !ctx->e_part || !ctx->e_out)
    return ctx->fail(SOP_ERR_ALLOC, "device allocation failed");
  if (!ctx->h_out) CK(cudaMallocHost(&ctx->h_out, 8 * sizeof(double)));
  cudaStream_t st = ctx->stream;
  CK(cudaMemsetAsync(s.mol_of, 0xff, sizeof(int) * nb, st));   // -1: free
  CK(cudaMemsetAsync(s.fsum, 0, sizeof(float4) * nb, st));      // no step in flight
  CK(cudaMemsetAsync(ctx->dmol, 0, sizeof(MolConst) * nm, st));  // inactive
  CK(cudaMemsetAsync(s.mol_step, 0, sizeof(long long) * nm, st));
  CK(cudaMemsetAsync(s.mol_status, 0, sizeof(int) * nm, st));
  CK(cudaMemsetAsync(s.sys_step, 0, sizeof(long long), st));
  CK(cudaMemsetAsync(s.flags, 0, 4 * sizeof(int), st));
  CK(cudaMemsetAsync(s.nl_maxrow, 0, sizeof(int), st));
  CK(cudaMemsetAsync(s.nl_att_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.pl_att_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.nl_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.pl_cnt, 0, sizeof(int) * nb, st));
  CK(cudaMemsetAsync(s.cell_cnt, 0, sizeof(int) * (size_t)c.cells, st));
  CK(cudaMemsetAsync(s.cell_start, 0, sizeof(int) * (size_t)(c.cells + 1), st));  // nothing binned yet
  CK(cudaMemsetAsync(s.bond_row, 0, sizeof(int2) * nb, st));
  CK(cudaMemsetAsync(s.ang_row, 0, sizeof(int2) * nb, st));
  CK(cudaMemsetAsync(s.nat_row, 0, sizeof(int2) * nb, st));
  ctx->bead_alloc.reset(c.beads);
  ctx->bond_alloc.reset(c.bonds);
  ctx->ang_alloc.reset(c.angles);
  ctx->nat_alloc.reset(c.natives);
  ctx->free_slots.clear();
  for (long long m = c.mols - 1; m >= 0; --m) ctx->free_slots.push_back((int)m);
  ctx->mc.assign(c.mols, MolConst{});
  return SOP_OK;
}

// Writes molecule hm into molecule slot `slot`: bead and topology ranges from
// the pools, rows with absolute offsets, x_0 in both coordinate buffers, its
// lists empty, and mol_step = step0 (0: starts now; < 0: starts -step0 steps
// into the next block sequence).  Returns SOP_ERR_CAPACITY if a pool is full.
// Host copies of the device rows of one or more molecules installed in
// consecutive pool ranges (beads [o, o + n), bond / angle / native entries
// from ob / oa / on, molecule slots from slot0), uploaded with one copy per
// array.
// A host array that is sized without being cleared: every entry of a staged
// array is written by fill_rows (the ranges of the staged molecules tile it),
// so clearing tens of MB first would only cost time.
template <class T>
struct RawArray {
  std::unique_ptr<T[]> p;
  size_t n = 0;
  void reset(size_t k) {
    p.reset(k ? new T[k] : nullptr);  // default-initialised: not cleared
    n = k;
  }
  T* data() { return p.get(); }
  const T* data() const { return p.get(); }
  size_t size() const { return n; }
  bool empty() const { return n == 0; }
  T& operator[](size_t i) { return p[i]; }
  const T& operator[](size_t i) const { return p[i]; }
};

struct Staged {
  long long o = 0, ob = 0, oa = 0, on = 0;
  int slot0 = 0;
  RawArray<int2> brow, arow, nrow;
  RawArray<int> bj, aj, nj, molof;
  RawArray<float> br;
  RawArray<float4> np, x0, p0, v0;
  RawArray<float2> nr;
  std::vector<long long> step0;
  std::vector<MolConst> mc;
  long long beads() const { return (long long)x0.size(); }
};

// Takes pool ranges for molecule `hm` in slot `slot`.  SOP_ERR_CAPACITY when
// the pools cannot hold it.
int take_ranges(SopCtx* ctx, int slot, HostMol& hm) {
  const long long nb2 = 2LL * (long long)hm.bi.size(), na2 = 2LL * (long long)hm.ai.size(),
                  nn2 = 2LL * (long long)hm.ni.size();
  long long b0 = ctx->bead_alloc.alloc(hm.n);
  if (b0 < 0) return SOP_ERR_CAPACITY;
  long long ob = ctx->bond_alloc.alloc(nb2);
  long long oa = ctx->ang_alloc.alloc(na2);
  long long on = ctx->nat_alloc.alloc(nn2);
  if (ob < 0 || oa < 0 || on < 0) {
    ctx->bead_alloc.release(b0, hm.n);
    if (ob >= 0) ctx->bond_alloc.release(ob, nb2);
    if (oa >= 0) ctx->ang_alloc.release(oa, na2);
    if (on >= 0) ctx->nat_alloc.release(on, nn2);
    return SOP_ERR_CAPACITY;
  }
  hm.start = (int)b0;
  hm.slot = slot;
  hm.off_b = ob; hm.off_a = oa; hm.off_n = on;
  return SOP_OK;
}

// Builds molecule `hm`'s device rows (its ranges already taken) into S,
// whose arrays start at pool positions S.o / S.ob / S.oa / S.on and are
// sized to hold it; k is its index among S's molecules.  Touches only the
// molecule's own part of S, so molecules may be built concurrently.
void fill_rows(const SopCtx* ctx, const HostMol& hm, int k, long long step0, Staged& S) {
  const sop_params& P = ctx->P;
  const int n = hm.n, o = hm.start;
  const long long ob = hm.off_b, oa = hm.off_a, on = hm.off_n;
  int2* brow = S.brow.data() + (o - S.o);
  int2* arow = S.arow.data() + (o - S.o);
  int2* nrow = S.nrow.data() + (o - S.o);
  std::vector<int> cnt_b(n, 0), cnt_a(n, 0), cnt_n(n, 0);
  for (size_t q = 0; q < hm.bi.size(); ++q) { cnt_b[hm.bi[q]]++; cnt_b[hm.bj[q]]++; }
  for (size_t q = 0; q < hm.ai.size(); ++q) { cnt_a[hm.ai[q]]++; cnt_a[hm.ak[q]]++; }
  for (size_t q = 0; q < hm.ni.size(); ++q) { cnt_n[hm.ni[q]]++; cnt_n[hm.nj[q]]++; }
  {
    int eb = (int)ob, ea = (int)oa, en = (int)on;
    for (int i = 0; i < n; ++i) {
      brow[i] = make_int2(eb, 0); eb += cnt_b[i];
      arow[i] = make_int2(ea, 0); ea += cnt_a[i];
      nrow[i] = make_int2(en, 0); en += cnt_n[i];
    }
  }
  auto put_b = [&](int i, int j, float r0) {
    const long long e = brow[i].x + brow[i].y++ - S.ob;
    S.bj[e] = o + j; S.br[e] = r0;
  };
  auto put_a = [&](int i, int j) { S.aj[arow[i].x + arow[i].y++ - S.oa] = o + j; };
  auto put_n = [&](int i, int j, float r0, float ef, float ee) {
    const long long e = nrow[i].x + nrow[i].y++ - S.on;
    S.nj[e] = o + j;
    S.np[e] = make_float4(r0, ef, ee, 0.f);
    S.nr[e] = make_float2(rcut2_of(P.nl_att_fac, P.nl_att_abs, r0),
                          rcut2_of(P.pl_att_fac, P.pl_att_abs, r0));
  };
  for (size_t q = 0; q < hm.bi.size(); ++q) {
    put_b(hm.bi[q], hm.bj[q], hm.br0[q]);
    put_b(hm.bj[q], hm.bi[q], hm.br0[q]);
  }
  for (size_t q = 0; q < hm.ai.size(); ++q) {
    put_a(hm.ai[q], hm.ak[q]);
    put_a(hm.ak[q], hm.ai[q]);
  }
  for (size_t q = 0; q < hm.ni.size(); ++q) {
    put_n(hm.ni[q], hm.nj[q], hm.nr0[q], hm.neps[q], hm.nepse[q]);
    put_n(hm.nj[q], hm.ni[q], hm.nr0[q], hm.neps[q], hm.nepse[q]);
  }
  const std::vector<float>& pp = hm.pos.empty() ? hm.unc : hm.pos;
  for (int i = 0; i < n; ++i) {
    const size_t d = (size_t)(o - S.o) + i;
    const int t = hm.types.empty() ? 1 : hm.types[i];
    S.molof[d] = hm.slot;
    S.x0[d] = make_float4(hm.unc[3 * i], hm.unc[3 * i + 1], hm.unc[3 * i + 2], bits_f(t));
    S.p0[d] = make_float4(pp[3 * i], pp[3 * i + 1], pp[3 * i + 2], 0.f);
    S.v0[d] = hm.vel.empty() ? make_float4(0.f, 0.f, 0.f, 0.f)
                             : make_float4(hm.vel[3 * i], hm.vel[3 * i + 1], hm.vel[3 * i + 2], 0.f);
  }
  S.mc[k] = make_const(P, hm);
  S.step0[k] = step0;
}

// Sizes S for `beads` beads, `b2` / `a2` / `n2` bond / angle / native entries
// and `nm` molecules starting at the given pool positions and slot.
void size_staged(Staged& S, long long o, long long ob, long long oa, long long on, int slot0,
                 long long beads, long long b2, long long a2, long long n2, int nm) {
  S.o = o; S.ob = ob; S.oa = oa; S.on = on; S.slot0 = slot0;
  S.brow.reset(beads); S.arow.reset(beads); S.nrow.reset(beads);
  S.molof.reset(beads);
  S.x0.reset(beads); S.p0.reset(beads); S.v0.reset(beads);
  S.bj.reset(b2); S.br.reset(b2);
  S.aj.reset(a2);
  S.nj.reset(n2); S.np.reset(n2); S.nr.reset(n2);
  S.mc.assign(nm, MolConst{});
  S.step0.assign(nm, 0);
}

// One molecule: its ranges and rows, staged on the host.
int stage_install(SopCtx* ctx, int slot, HostMol& hm, long long step0, Staged& S) {
  int rc = take_ranges(ctx, slot, hm);
  if (rc) return rc;
  size_staged(S, hm.start, hm.off_b, hm.off_a, hm.off_n, slot, hm.n, 2LL * (long long)hm.bi.size(),
              2LL * (long long)hm.ai.size(), 2LL * (long long)hm.ni.size(), 1);
  fill_rows(ctx, hm, 0, step0, S);
  ctx->mc[slot] = S.mc[0];
  return SOP_OK;
}

// Uploads staged rows (one copy per array) and waits for the copies.
int upload_staged(SopCtx* ctx, const Staged& S) {
  if (S.mc.empty()) return SOP_OK;
  DevSys& s = ctx->s;
  cudaStream_t st = ctx->stream;
  const long long n = S.beads(), o = S.o;
  const size_t f4 = sizeof(float4) * (size_t)n;
  auto up = [&](auto* dst, const auto& v) -> cudaError_t {
    if (v.empty()) return cudaSuccess;
    return cudaMemcpyAsync(dst, v.data(), sizeof(v[0]) * v.size(), cudaMemcpyHostToDevice, st);
  };
  for (int b = 0; b < 2; ++b) {
    CK(up(s.x[b] + o, S.x0));
    CK(up(s.p[b] + o, S.p0));
  }
  CK(up(s.v + o, S.v0));
  CK(cudaMemsetAsync(s.incr + o, 0, f4, st));
  CK(cudaMemsetAsync(s.f + o, 0, f4, st));
  CK(up(s.bond_row + o, S.brow));
  CK(up(s.ang_row + o, S.arow));
  CK(up(s.nat_row + o, S.nrow));
  CK(up(s.bond_j + S.ob, S.bj));
  CK(up(s.bond_r0 + S.ob, S.br));
  CK(up(s.ang_j + S.oa, S.aj));
  CK(up(s.nat_j + S.on, S.nj));
  CK(up(s.nat_par + S.on, S.np));
  CK(up(s.nat_rc2 + S.on, S.nr));
  CK(cudaMemsetAsync(s.nl_cnt + o, 0, sizeof(int) * (size_t)n, st));
  CK(cudaMemsetAsync(s.pl_cnt + o, 0, sizeof(int) * (size_t)n, st));
  CK(cudaMemsetAsync(s.nl_att_cnt + o, 0, sizeof(int) * (size_t)n, st));
  CK(cudaMemsetAsync(s.pl_att_cnt + o, 0, sizeof(int) * (size_t)n, st));
  CK(up(s.mol_step + S.slot0, S.step0));
  CK(cudaMemsetAsync(s.mol_status + S.slot0, 0, sizeof(int) * S.mc.size(), st));
  CK(up(s.mol_of + o, S.molof));
  CK(up(ctx->dmol + S.slot0, S.mc));
  CK(cudaStreamSynchronize(st));  // the host arrays may go out of scope
  return SOP_OK;
}

// One molecule into slot `slot`, its step counter at step0.
int install(SopCtx* ctx, int slot, HostMol& hm, long long step0) {
  Staged S;
  int rc = stage_install(ctx, slot, hm, step0, S);
  if (rc) return rc;
  return upload_staged(ctx, S);
}

// Frees molecule slot `slot`: inactive on the device, its beads unowned,
// its pool ranges returned.  The stream must be idle.
int uninstall(SopCtx* ctx, int slot) {
  HostMol& hm = ctx->mols[slot];
  if (hm.start < 0) return SOP_OK;
  MolConst off{};
  CK(cudaMemcpy(ctx->dmol + slot, &off, sizeof(MolConst), cudaMemcpyHostToDevice));
  CK(cudaMemset(ctx->s.mol_of + hm.start, 0xff, sizeof(int) * (size_t)hm.n));
  ctx->bead_alloc.release(hm.start, hm.n);
  ctx->bond_alloc.release(hm.off_b, 2LL * (long long)hm.bi.size());
  ctx->ang_alloc.release(hm.off_a, 2LL * (long long)hm.ai.size());
  ctx->nat_alloc.release(hm.off_n, 2LL * (long long)hm.ni.size());
  ctx->mc[slot] = MolConst{};
  hm.start = -1;
  ctx->free_slots.push_back(slot);
  return SOP_OK;
}

// Size buckets of the tiled form: molecules of fewer than 200 beads, of 200
// to 599, and of 600 or more.
constexpr int kBuckets = 3;
int bucket_of(int n) { return n < 200 ? 0 : n < 600 ? 1 : 2; }

// The tiles of every molecule (or of bucket `only` alone): runs of
// 128 / lanes beads from the molecule's first bead, never across molecules.
void build_tiles(const SopCtx* ctx, const int* lanes, const int* forms, int only,
                 std::vector<int4>& out) {
  out.clear();
  for (const HostMol& hm : ctx->mols) {
    if (hm.start < 0 || hm.n <= 0) continue;
    const int b = bucket_of(hm.n);
    if (only >= 0 && b != only) continue;
    const int g = lanes[b], bpb = 128 / g;
    for (int st = hm.start; st < hm.start + hm.n; st += bpb)
      out.push_back(make_int4(st, std::min(st + bpb, hm.start + hm.n), g, forms[b] == 2));
  }
}

// Times `reps` force-only evaluations of the current step layout (the tiles
// in d_tiles when `tiles`, else the whole-context form); idempotent.
int time_step(SopCtx* ctx, bool tiles, int ntiles, bool any_split, float* ms) {
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  auto run = [&] {
    if (tiles) launch_step_tiles(ctx->s, 0, false, ctx->d_tiles, ntiles, any_split, ctx->stream);
    else launch_step(ctx->s, ctx->G, ctx->split, 0, false, ctx->wcap, ctx->stream);
  };
  run();  // warm-up
  CK(cudaEventRecord(a, ctx->stream));
  for (int r = 0; r < kTuneReps; ++r) run();
  CK(cudaEventRecord(b, ctx->stream));
  CK(cudaEventSynchronize(b));
  CK(cudaEventElapsedTime(ms, a, b));
  *ms /= (float)kTuneReps;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CK(cudaGetLastError());
  return SOP_OK;
}

// The per-size-bucket tuner of a batched context: for each bucket, the lanes
// per bead (4 or 8) and the form (one kernel or two) of its molecules' tiles,
// timed on that bucket's tiles alone; then the tiled step with every
// bucket's choice against the best whole-context form, and the faster one is
// kept (sop_params.step_buckets 1 keeps the tiled step, -1 never tries it).
// Both give the same bits.
int autotune_buckets(SopCtx* ctx) {
  const int want = ctx->P.step_buckets;
  ctx->tiled = false;
  if (want < 0 || ctx->served || ctx->persist || ctx->one_block || ctx->wcap > 0) return SOP_OK;
  int present = 0;
  for (int b = 0; b < kBuckets; ++b) ctx->bucket_beads[b] = 0;
  long long cap = 0;
  for (const HostMol& hm : ctx->mols)
    if (hm.start >= 0 && hm.n > 0) {
      ctx->bucket_beads[bucket_of(hm.n)] += hm.n;
      cap += (hm.n + 15) / 16;
    }
  for (int b = 0; b < kBuckets; ++b) present += ctx->bucket_beads[b] > 0;
  if (want == 0 && (present < 2 || ctx->mols.size() < 2)) return SOP_OK;
  if (!ctx->d_tiles) {
    ctx->d_tiles = ctx->dalloc<int4>((size_t)cap);
    if (!ctx->d_tiles) return ctx->fail(SOP_ERR_ALLOC, "tile allocation failed");
  }
  std::vector<int4> t;
  int lanes[kBuckets] = {4, 4, 4}, forms[kBuckets] = {1, 1, 1};
  for (int b = 0; b < kBuckets; ++b) {
    if (!ctx->bucket_beads[b]) continue;
    float best = 1e30f;
    for (int g : {4, 8})
      for (int f : {1, 2}) {
        int gl[kBuckets] = {g, g, g}, fl[kBuckets] = {f, f, f};
        build_tiles(ctx, gl, fl, b, t);
        CK(cudaMemcpy(ctx->d_tiles, t.data(), sizeof(int4) * t.size(), cudaMemcpyHostToDevice));
        float ms = 0.f;
        int rc = time_step(ctx, true, (int)t.size(), f == 2, &ms);
        if (rc) return rc;
        if (ms < best) { best = ms; lanes[b] = g; forms[b] = f; }
      }
  }
  build_tiles(ctx, lanes, forms, -1, t);
  CK(cudaMemcpy(ctx->d_tiles, t.data(), sizeof(int4) * t.size(), cudaMemcpyHostToDevice));
  bool any_split = false;
  for (int b = 0; b < kBuckets; ++b) any_split |= ctx->bucket_beads[b] && forms[b] == 2;
  int rc = time_step(ctx, true, (int)t.size(), any_split, &ctx->ms_tiled);
  if (rc) return rc;
  rc = time_step(ctx, false, 0, false, &ctx->ms_whole);
  if (rc) return rc;
  for (int b = 0; b < kBuckets; ++b) {
    ctx->bucket_lanes[b] = ctx->bucket_beads[b] ? lanes[b] : 0;
    ctx->bucket_form[b] = ctx->bucket_beads[b] ? forms[b] : 0;
  }
  ctx->ntiles = (int)t.size();
  ctx->tiles_split = any_split;
  ctx->tiled = want > 0 || ctx->ms_tiled < ctx->ms_whole;
  return SOP_OK;
}

// Set-up after installing molecules at step 0: lists from x_0, f_0 and the
// look-ahead (sop.cu:142-186), and the lanes-per-bead choice.
int setup_step0(SopCtx* ctx) {
  const int fixed_g = lanes_for(ctx), fixed_f = split_for(ctx), fixed_w = window_param(ctx);
  ctx->G = fixed_g ? fixed_g : 8;
  ctx->split = fixed_f == 2;
  ctx->persist = fixed_f == 3 && !ctx->served;
  ctx->one_block = fixed_f == 4 && !ctx->served;
  ctx->wcap = 0;
  if (fixed_w > 0 && !ctx->served) {
    CK(allow_step_window(kMaxStepWindow));
    ctx->wcap = fixed_w;
  }
  // block offset -1: these rebuilds precede the force evaluation of the
  // current step itself (x_0 sits in both coordinate buffers)
  int rc = nl_rebuild_checked(ctx, -1);
  if (rc) return rc;
  launch_pl_rebuild(ctx->s, -1, ctx->stream);
  force_eval_async(ctx);
  CK(cudaGetLastError());
  if (!fixed_g || !fixed_f) {
    rc = autotune_lanes(ctx);
    if (rc) return rc;
  }
  if (!fixed_g && !fixed_f && !ctx->served) {
    rc = autotune_buckets(ctx);
    if (rc) return rc;
  } else if (ctx->P.step_buckets > 0 && !ctx->served) {
    return ctx->fail(SOP_ERR_ARG, "step_buckets = 1 needs the lanes and the form left to the tuner");
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

// Neighbour-list row length for molecules of up to max_beads beads: the
// parameter nl_rows where it is set, else 1.3 x
// the neighbours of a bead in the densest part of a globule (6e-3 / A^3: the
// cores of the synthetic structures reach about twice their mean density of
// 2.5e-3), and no more than a molecule holds.
long long dense_stride(const SopCtx* ctx, long long max_beads) {
  if (ctx->P.nl_rows > 0) return std::max<long long>(64, ((long long)ctx->P.nl_rows + 31) / 32 * 32);
  const double rc_nl = ctx->s.rc_nl_rep_max;
  long long stride = (long long)(1.3 * 6.0e-3 * 4.18879 * rc_nl * rc_nl * rc_nl) + 32;
  stride = std::min<long long>(stride, max_beads + 32);
  return std::max<long long>(64, (stride + 31) / 32 * 32);
}

// Molecules of this many beads or more have neighbour-list rows long
// enough (about 400 entries at 32 A) that the pair-list rebuild runs faster
// with 16 lanes per bead than with 8 (the ensemble's molecules of up to
// 1,500 beads, about 190 entries, run faster with 8).
constexpr long long kLongRowBeads = 10000;

// Packs every staged molecule into exactly sized pools (plain and batched
// contexts): molecule id = slot, all at step 0.
int commit(SopCtx* ctx) {
  set_constants(ctx);
  Caps c;
  for (auto& m : ctx->mols) {
    c.beads += m.n;
    c.bonds += 2LL * (long long)m.bi.size();
    c.angles += 2LL * (long long)m.ai.size();
    c.natives += 2LL * (long long)m.ni.size();
    c.cells += std::max<long long>(64, 2LL * m.n);
    c.max_mol_beads = std::max<long long>(c.max_mol_beads, m.n);
  }
  c.mols = (long long)ctx->mols.size();
  if (c.beads <= 0) return ctx->fail(SOP_ERR_ARG, "no beads");
  // rows sized so that most contexts never regrow them (a regrowth costs a
  // second list build at commit); a longer row regrows from the first
  // rebuild's longest one
  c.stride = dense_stride(ctx, c.max_mol_beads);
  int rc = alloc_pools(ctx, c);
  if (rc) return rc;
  ctx->s.uniform_type = 1;
  ctx->s.long_rows = c.max_mol_beads >= kLongRowBeads ? 1 : 0;
  for (auto& m : ctx->mols)
    for (int t : m.types)
      if (t != 1) ctx->s.uniform_type = 0;
  // every molecule's ranges taken in id order (the pools are fresh, so they
  // follow one another from 0), its rows built on the host by a pool of
  // threads, then one copy per array
  const int nm = (int)ctx->mols.size();
  for (int k = 0; k < nm; ++k) {
    ctx->free_slots.pop_back();  // slots handed out in id order
    rc = take_ranges(ctx, k, ctx->mols[k]);
    if (rc) return ctx->fail(rc, "pool sizing error");
  }
  Staged all;
  size_staged(all, 0, 0, 0, 0, 0, c.beads, c.bonds, c.angles, c.natives, nm);
  {
    const int nthr = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
    std::atomic<int> next{0};
    auto work = [&] {
      for (int k = next++; k < nm; k = next++) fill_rows(ctx, ctx->mols[k], k, 0, all);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthr && t < nm; ++t) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
  }
  for (int k = 0; k < nm; ++k) ctx->mc[k] = all.mc[k];
  rc = upload_staged(ctx, all);
  if (rc) return rc;
  rc = setup_step0(ctx);
  if (rc) return rc;
  ctx->host_step = 0;
  ctx->target_step = 0;
  ctx->committed = true;
  return SOP_OK;
}

int check_mol(SopCtx* ctx, int mol) {
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  if (mol < 0 || mol >= (int)ctx->mols.size()) return ctx->fail(SOP_ERR_NOT_FOUND, "unknown molecule");
  return SOP_OK;
}

int read_step(SopCtx* ctx, int mol, long long* step) {
  CK(cudaMemcpyAsync(ctx->h_out, ctx->s.mol_step + mol, sizeof(long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::memcpy(step, ctx->h_out, sizeof(long long));
  return SOP_OK;
}

// float4 device rows -> 3 floats per bead on the host
int copy3(SopCtx* ctx, float* dst, const float4* src, int n) {
  CK(cudaMemcpy2DAsync(dst, 3 * sizeof(float), src, sizeof(float4), 3 * sizeof(float), n,
                       cudaMemcpyDeviceToHost, ctx->stream));
  return SOP_OK;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

void sop_params_default(sop_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->k_bnd = 20.0;      // param.cpp:14
  p->R0 = 2.0;          // param.cpp:15
  p->eps_ss = 1.0;      // param.cpp:37
  p->sigma_ss = 3.5;    // param.cpp:35
  p->eps_rep = 1.0;     // energy.cu:15-19
  p->boxl = 500.0;      // param.cpp:97
  p->h = 2.5e-3;        // param.cpp:104
  p->zeta = 5.0e-2;     // param.cpp:100
  p->nl_att_fac = 3.2;  // sop.cu:746
  p->nl_rep_fac = 3.2;  // sop.cu:815
  p->pl_att_fac = 2.5;  // sop.cu:861
  p->pl_rep_fac = 2.5;  // sop.cu:910
  p->nnlup = 50;        // param.cpp:103
  p->nplup = 1;         // sop.cu:227-232: every step
  p->rep6 = 0;
  p->device = 0;
  p->graph_steps = 0;
  p->lanes_per_bead = 0;
  p->seed = 1234;       // setup_rng(1234, 0), sop.cu:138
  p->integrator = 0;    // underdamped (param.cpp:249-253 selects)
  p->step_split = 0;    // autotuned
  p->step_window = 0;   // autotuned
  p->step_buckets = 0;  // autotuned
  p->nl_rows = 0;       // sized for dense globules
}

int sop_ctx_create(const sop_params* p, void** out) {
  if (!p || !out) return SOP_ERR_ARG;
  *out = nullptr;
  if (p->boxl <= 0 || p->h <= 0 || p->R0 <= 0 || p->graph_steps < 0 || p->integrator < 0 ||
      p->step_split < 0 || p->step_split > 4 || p->step_window > kMaxStepWindow ||
      !(p->lanes_per_bead == 0 || p->lanes_per_bead == 2 || p->lanes_per_bead == 4 ||
        p->lanes_per_bead == 8 || p->lanes_per_bead == 16) || p->nl_rows < 0 ||
      p->integrator > 1 || (p->integrator == 1 && p->zeta <= 0)) {
    g_lib_error = "invalid parameters";
    return SOP_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(p->device);
  if (e != cudaSuccess) {
    g_lib_error = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return SOP_ERR_CUDA;
  }
  SopCtx* ctx = new SopCtx();
  ctx->P = *p;
  e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    g_lib_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
    delete ctx;
    return SOP_ERR_CUDA;
  }
  *out = ctx;
  return SOP_OK;
}

int sop_ctx_destroy(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  cudaSetDevice(ctx->P.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  delete ctx;
  return SOP_OK;
}

}  // extern "C"

// Validates a molecule description and copies it to host storage.
static int make_hostmol(SopCtx* ctx, const sop_molecule* m, HostMol& h) {
  if (m->nbead <= 0 || !m->unc_pos) return ctx->fail(SOP_ERR_ARG, "molecule needs beads and coordinates");
  if (m->nbead > kMaxMolBeads)
    return ctx->fail(SOP_ERR_ARG, "a molecule holds at most 65,535 beads (pair-list rows store "
                                  "16-bit molecule-relative partners)");
  if (m->nbnd < 0 || m->nang < 0 || m->nnat < 0) return ctx->fail(SOP_ERR_ARG, "negative counts");
  if ((m->nbnd && (!m->bond_i || !m->bond_j || !m->bond_r0)) || (m->nang && (!m->ang_i || !m->ang_k)) ||
      (m->nnat && (!m->nat_i || !m->nat_j || !m->nat_r0)))
    return ctx->fail(SOP_ERR_ARG, "missing topology arrays");
  h = HostMol();
  h.n = m->nbead;
  auto in = [&](int v) { return v >= 0 && v < m->nbead; };
  for (int k = 0; k < m->nbnd; ++k)
    if (!in(m->bond_i[k]) || !in(m->bond_j[k]) || m->bond_i[k] == m->bond_j[k])
      return ctx->fail(SOP_ERR_ARG, "bond index out of range");
  for (int k = 0; k < m->nang; ++k)
    if (!in(m->ang_i[k]) || !in(m->ang_k[k]) || m->ang_i[k] == m->ang_k[k])
      return ctx->fail(SOP_ERR_ARG, "angle index out of range");
  for (int k = 0; k < m->nnat; ++k)
    if (!in(m->nat_i[k]) || !in(m->nat_j[k]) || std::abs(m->nat_i[k] - m->nat_j[k]) <= 2)
      return ctx->fail(SOP_ERR_ARG, "native contact needs |i - j| > 2 and in-range indices");
  if (m->types)
    for (int i = 0; i < m->nbead; ++i)
      if (m->types[i] != 1 && m->types[i] != 2) return ctx->fail(SOP_ERR_ARG, "bead types must be 1 or 2");
  h.bi.assign(m->bond_i, m->bond_i + m->nbnd);
  h.bj.assign(m->bond_j, m->bond_j + m->nbnd);
  h.br0.assign(m->bond_r0, m->bond_r0 + m->nbnd);
  h.ai.assign(m->ang_i, m->ang_i + m->nang);
  h.ak.assign(m->ang_k, m->ang_k + m->nang);
  h.ni.assign(m->nat_i, m->nat_i + m->nnat);
  h.nj.assign(m->nat_j, m->nat_j + m->nnat);
  h.nr0.assign(m->nat_r0, m->nat_r0 + m->nnat);
  if (m->nat_eps) h.neps.assign(m->nat_eps, m->nat_eps + m->nnat);
  else h.neps.assign(m->nnat, 1.0f);
  if (m->nat_eps_energy) h.nepse.assign(m->nat_eps_energy, m->nat_eps_energy + m->nnat);
  else h.nepse = h.neps;
  if (m->types) h.types.assign(m->types, m->types + m->nbead);
  h.unc.assign(m->unc_pos, m->unc_pos + 3 * (size_t)m->nbead);
  if (m->pos) h.pos.assign(m->pos, m->pos + 3 * (size_t)m->nbead);
  if (m->vel) h.vel.assign(m->vel, m->vel + 3 * (size_t)m->nbead);
  h.T = m->T;
  h.traj = m->traj;
  h.nsteps = m->nsteps;
  return SOP_OK;
}

// ------------------------------------------------------------- serving
static int retire(SopCtx* ctx, int slot, const std::vector<long long>& steps,
                  const std::vector<int>& status) {
  Job& jb = ctx->jobs[ctx->slot_job[slot]];
  HostMol& hm = ctx->mols[slot];
  const long long st = std::max<long long>(steps[slot], 0);
  const int cur = (int)(st & 1);
  jb.unc.resize(3 * (size_t)hm.n);
  jb.vel.resize(3 * (size_t)hm.n);
  int rc = copy3(ctx, jb.unc.data(), ctx->s.x[cur] + hm.start, hm.n);
  if (rc) return rc;
  rc = copy3(ctx, jb.vel.data(), ctx->s.v + hm.start, hm.n);
  if (rc) return rc;
  launch_energy(ctx->s, hm.start, hm.n, slot, ctx->e_part, ctx->e_out,
                0.5 * ctx->P.k_bnd * ctx->P.R0 * ctx->P.R0, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->h_out, ctx->e_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int t = 0; t < 4; ++t) jb.energy[t] = ctx->h_out[t];
  jb.energy[4] = jb.energy[0] + jb.energy[1] + jb.energy[2] + jb.energy[3];
  jb.status = status[slot] | (st >= jb.nsteps ? SOP_MOL_DONE : 0);
  jb.steps = st;
  jb.t_done = now_seconds();
  jb.state = Job::FINISHED;
  ctx->finished_new.push_back(ctx->slot_job[slot]);
  rc = uninstall(ctx, slot);
  if (rc) return rc;
  ctx->slot_job[slot] = -1;
  hm = HostMol();
  return SOP_OK;
}

// One round: wait, retire, admit, queue nnlup steps.

// ------------------------------------------------------------ checkpoints
// An exact checkpoint of one molecule: its step counter and status, both
// coordinate buffers (the last completed step and the look-ahead the next
// step reads), both wrapped-coordinate buffers, velocities, increments and
// forces, and its neighbour- and pair-list rows with bead and native indices
// relative to the molecule.  Restoring writes all of it back, so the steps
// that follow read exactly what they read in the run the checkpoint came
// from (the noise is keyed by the step, and the lists are rebuilt on the
// same cadence from the same coordinates): the continuation is the same
// bits.  The reference saves coordinates and velocities (save_coords /
// save_vels, io.cpp:261-381, from sop.cu:268-272) and restarts from them,
// not exactly.
struct CkptHeader {
  char magic[4];
  int version;
  int n;             // beads
  int nnat2;         // native row entries (both directions)
  long long step;    // last completed step
  int status;        // SOP_MOL_* bits
  int pad;
  long long cnt[4];  // row entries: attractive NL, attractive PL, repulsive NL, repulsive PL
};
const char kCkptMagic[4] = {'S', 'O', 'P', 'K'};
constexpr int kCkptVersion = 1;

long long ckpt_bytes(int n, const long long* cnt) {
  return (long long)sizeof(CkptHeader) + 7LL * 16 * n + 16LL * n + 4 * cnt[0] + 16 * cnt[1] +
         4 * cnt[2] + 4 * cnt[3];
}

// Regrows the repulsive list rows to at least `stride` entries, keeping
// every row (the other molecules' lists stay valid).  Stream idle.
int grow_nl_keep(SopCtx* ctx, long long stride) {
  stride = (stride + 31) / 32 * 32;
  DevSys& s = ctx->s;
  if (stride <= s.nl_stride) return SOP_OK;
  const long long nb = s.nbead, old = s.nl_stride, entries = stride * nb;
  if (entries > (1LL << 40)) return ctx->fail(SOP_ERR_CAPACITY, "neighbour list exceeds 2^40 entries");
  unsigned short* nj = ctx->dalloc<unsigned short>(entries);
  unsigned short* pj = ctx->dalloc<unsigned short>(entries);
  if (!nj || !pj) {
    ctx->dfree(nj);
    ctx->dfree(pj);
    return ctx->fail(SOP_ERR_ALLOC, "neighbour-list allocation failed");
  }
  CK(cudaMemcpy2D(nj, 2 * stride, s.nl_j, 2 * old, 2 * old, nb, cudaMemcpyDeviceToDevice));
  CK(cudaMemcpy2D(pj, 2 * stride, s.pl_j, 2 * old, 2 * old, nb, cudaMemcpyDeviceToDevice));
  ctx->dfree(s.nl_j);
  ctx->dfree(s.pl_j);
  s.nl_j = nj;
  s.pl_j = pj;
  s.nl_stride = stride;
  ctx->drop_graphs();  // kernel arguments changed
  return SOP_OK;
}

// Serialises molecule slot `slot` (stream idle).
int checkpoint_of(SopCtx* ctx, int slot, std::vector<char>& out) {
  DevSys& s = ctx->s;
  const HostMol& hm = ctx->mols[slot];
  const int n = hm.n, o = hm.start;
  const long long nn2 = 2LL * (long long)hm.ni.size();
  CkptHeader h{};
  std::memcpy(h.magic, kCkptMagic, 4);
  h.version = kCkptVersion;
  h.n = n;
  h.nnat2 = (int)nn2;
  CK(cudaMemcpy(&h.step, s.mol_step + slot, sizeof(long long), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&h.status, s.mol_status + slot, sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> cnt(4 * (size_t)n);
  const int* src[4] = {s.nl_att_cnt, s.pl_att_cnt, s.nl_cnt, s.pl_cnt};
  for (int t = 0; t < 4; ++t) {
    CK(cudaMemcpy(cnt.data() + (size_t)t * n, src[t] + o, sizeof(int) * n, cudaMemcpyDeviceToHost));
    h.cnt[t] = 0;
    for (int i = 0; i < n; ++i) h.cnt[t] += cnt[(size_t)t * n + i];
  }
  out.assign((size_t)ckpt_bytes(n, h.cnt), 0);
  char* w = out.data();
  auto put = [&](const void* p, size_t b) {
    std::memcpy(w, p, b);
    w += b;
  };
  put(&h, sizeof h);
  const int cur = (int)(h.step & 1);
  const float4* arr[7] = {s.x[cur] + o, s.x[cur ^ 1] + o, s.p[cur] + o, s.p[cur ^ 1] + o,
                          s.v + o, s.incr + o, s.f + o};
  std::vector<float4> tmp(n);
  for (int a = 0; a < 7; ++a) {
    CK(cudaMemcpy(tmp.data(), arr[a], sizeof(float4) * n, cudaMemcpyDeviceToHost));
    put(tmp.data(), sizeof(float4) * n);
  }
  put(cnt.data(), sizeof(int) * 4 * (size_t)n);
  std::vector<int2> nrow(n);
  CK(cudaMemcpy(nrow.data(), s.nat_row + o, sizeof(int2) * n, cudaMemcpyDeviceToHost));
  std::vector<int> ae(nn2 > 0 ? nn2 : 1);
  std::vector<float4> ap(nn2 > 0 ? nn2 : 1);
  if (nn2) {
    CK(cudaMemcpy(ae.data(), s.nl_att_e + hm.off_n, sizeof(int) * nn2, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ap.data(), s.pl_att + hm.off_n, sizeof(float4) * nn2, cudaMemcpyDeviceToHost));
  }
  for (int i = 0; i < n; ++i)
    for (int t = 0; t < cnt[i]; ++t) {
      int v = ae[nrow[i].x - hm.off_n + t] - (int)hm.off_n;
      put(&v, sizeof v);
    }
  for (int i = 0; i < n; ++i)
    for (int t = 0; t < cnt[(size_t)n + i]; ++t) {
      float4 q = ap[nrow[i].x - hm.off_n + t];
      q.x = bits_f(bits_i(q.x) - o);
      put(&q, sizeof q);
    }
  const long long stride = s.nl_stride;
  std::vector<int> rows;
  for (int r = 0; r < 2; ++r) {
    int rc = read_rows(ctx, r, o, n, rows);
    if (rc) return rc;
    for (int i = 0; i < n; ++i)
      for (int t = 0; t < cnt[(size_t)(2 + r) * n + i]; ++t) {
        int v = rows[(size_t)i * stride + t];
        put(&v, sizeof v);
      }
  }
  return SOP_OK;
}

// Writes a checkpoint into molecule slot `slot` (installed, stream idle).
int restore_into(SopCtx* ctx, int slot, const char* buf, long long len) {
  DevSys& s = ctx->s;
  const HostMol& hm = ctx->mols[slot];
  const int n = hm.n, o = hm.start;
  const long long nn2 = 2LL * (long long)hm.ni.size();
  CkptHeader h;
  if (!buf || len < (long long)sizeof h) return ctx->fail(SOP_ERR_ARG, "checkpoint too short");
  std::memcpy(&h, buf, sizeof h);
  if (std::memcmp(h.magic, kCkptMagic, 4) || h.version != kCkptVersion)
    return ctx->fail(SOP_ERR_ARG, "not a checkpoint of this format");
  if (h.n != n || h.nnat2 != nn2)
    return ctx->fail(SOP_ERR_ARG, "checkpoint of a different molecule");
  for (int t = 0; t < 4; ++t)
    if (h.cnt[t] < 0) return ctx->fail(SOP_ERR_ARG, "corrupt checkpoint");
  if (len != ckpt_bytes(n, h.cnt)) return ctx->fail(SOP_ERR_ARG, "checkpoint size mismatch");
  const char* r = buf + sizeof h;
  auto get = [&](void* p, size_t b) {
    std::memcpy(p, r, b);
    r += b;
  };
  std::vector<std::vector<float4>> arr(7, std::vector<float4>(n));
  for (int a = 0; a < 7; ++a) get(arr[a].data(), sizeof(float4) * n);
  std::vector<int> cnt(4 * (size_t)n);
  get(cnt.data(), sizeof(int) * cnt.size());
  std::vector<int2> nrow(n);
  CK(cudaMemcpy(nrow.data(), s.nat_row + o, sizeof(int2) * n, cudaMemcpyDeviceToHost));
  long long sum[4] = {0, 0, 0, 0};
  int maxrow = 0;
  for (int i = 0; i < n; ++i) {
    for (int t = 0; t < 4; ++t) {
      const int c = cnt[(size_t)t * n + i];
      if (c < 0 || (t < 2 && c > nrow[i].y)) return ctx->fail(SOP_ERR_ARG, "corrupt checkpoint");
      sum[t] += c;
      if (t >= 2) maxrow = std::max(maxrow, c);
    }
  }
  for (int t = 0; t < 4; ++t)
    if (sum[t] != h.cnt[t]) return ctx->fail(SOP_ERR_ARG, "corrupt checkpoint");
  std::vector<int> ae(nn2 > 0 ? nn2 : 1, 0);
  std::vector<float4> ap(nn2 > 0 ? nn2 : 1, make_float4(0.f, 0.f, 0.f, 0.f));
  for (int i = 0; i < n; ++i)
    for (int t = 0; t < cnt[i]; ++t) {
      int v;
      get(&v, sizeof v);
      if (v < 0 || v >= nn2) return ctx->fail(SOP_ERR_ARG, "corrupt checkpoint");
      ae[nrow[i].x - hm.off_n + t] = v + (int)hm.off_n;
    }
  for (int i = 0; i < n; ++i)
    for (int t = 0; t < cnt[(size_t)n + i]; ++t) {
      float4 q;
      get(&q, sizeof q);
      const int j = bits_i(q.x);
      if (j < 0 || j >= n) return ctx->fail(SOP_ERR_ARG, "corrupt checkpoint");
      q.x = bits_f(j + o);
      ap[nrow[i].x - hm.off_n + t] = q;
    }
  if (maxrow > s.nl_stride) {
    int rc = grow_nl_keep(ctx, (long long)maxrow * 5 / 4 + 32);
    if (rc) return rc;
  }
  const long long stride = s.nl_stride;
  std::vector<unsigned short> rows[2];   // both molecule-relative, as stored
  for (int k = 0; k < 2; ++k) {
    rows[k].assign((size_t)(stride * n), 0);
    for (int i = 0; i < n; ++i)
      for (int t = 0; t < cnt[(size_t)(2 + k) * n + i]; ++t) {
        int v;
        get(&v, sizeof v);
        if (v < 0 || v >= n) return ctx->fail(SOP_ERR_ARG, "corrupt checkpoint");
        rows[k][(size_t)i * stride + t] = (unsigned short)v;
      }
  }
  const int cur = (int)(h.step & 1);
  float4* dst[7] = {s.x[cur] + o, s.x[cur ^ 1] + o, s.p[cur] + o, s.p[cur ^ 1] + o,
                    s.v + o, s.incr + o, s.f + o};
  for (int a = 0; a < 7; ++a)
    CK(cudaMemcpy(dst[a], arr[a].data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
  int* cdst[4] = {s.nl_att_cnt, s.pl_att_cnt, s.nl_cnt, s.pl_cnt};
  for (int t = 0; t < 4; ++t)
    CK(cudaMemcpy(cdst[t] + o, cnt.data() + (size_t)t * n, sizeof(int) * n, cudaMemcpyHostToDevice));
  if (nn2) {
    CK(cudaMemcpy(s.nl_att_e + hm.off_n, ae.data(), sizeof(int) * nn2, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s.pl_att + hm.off_n, ap.data(), sizeof(float4) * nn2, cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(s.nl_j + (long long)o * stride, rows[0].data(),
                sizeof(unsigned short) * rows[0].size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.pl_j + (long long)o * stride, rows[1].data(),
                sizeof(unsigned short) * rows[1].size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.mol_step + slot, &h.step, sizeof(long long), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(s.mol_status + slot, &h.status, sizeof(int), cudaMemcpyHostToDevice));
  return SOP_OK;
}

// The header of a checkpoint, or false when buf does not hold one.
bool ckpt_head(const void* buf, long long len, CkptHeader* h) {
  if (!buf || len < (long long)sizeof(CkptHeader)) return false;
  std::memcpy(h, buf, sizeof(CkptHeader));
  return !std::memcmp(h->magic, kCkptMagic, 4) && h->version == kCkptVersion && h->step >= 0 &&
         len == ckpt_bytes(h->n, h->cnt);
}

// The per-step kernels of a served context cover the bead slots up to the
// highest one in use, rounded up to a sixteenth of the pool: the step graphs
// hold that bound, so they are re-captured only when it crosses a sixteenth.
static void update_live(SopCtx* ctx) {
  const long long cap = ctx->caps.beads;
  const long long g = std::max<long long>(1, (cap + 15) / 16);
  const long long hw = ctx->bead_alloc.high_water();
  const long long live = std::min(cap, std::max(g, (hw + g - 1) / g * g));
  if (live != ctx->s.nlive) {
    ctx->s.nlive = (int)live;
    ctx->drop_graphs();  // kernel arguments changed
  }
}

static int serve_round(SopCtx* ctx) {
  int rc = sync_checked(ctx);
  if (rc) return rc;
  const int nm = (int)ctx->caps.mols;
  std::vector<long long> steps(nm);
  std::vector<int> status(nm);
  CK(cudaMemcpy(steps.data(), ctx->s.mol_step, sizeof(long long) * nm, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(status.data(), ctx->s.mol_status, sizeof(int) * nm, cudaMemcpyDeviceToHost));
  for (int slot = 0; slot < nm; ++slot) {
    const int id = ctx->slot_job[slot];
    if (id < 0) continue;
    if (status[slot] != 0 || steps[slot] >= ctx->jobs[id].nsteps) {
      rc = retire(ctx, slot, steps, status);
      if (rc) return rc;
    }
  }
  // admission in arrival order; a job that does not fit yet lets the next
  // few (smaller) ones try
  int looked = 0;
  bool rebin = false;
  for (auto it = ctx->queue.begin(); it != ctx->queue.end() && looked < 64 && !ctx->free_slots.empty();) {
    Job& jb = ctx->jobs[*it];
    const int slot = ctx->free_slots.back();
    ctx->mols[slot] = jb.mol;
    for (int t : jb.mol.types)
      if (t != 1 && ctx->s.uniform_type) {
        ctx->s.uniform_type = 0;
        ctx->drop_graphs();  // kernel arguments changed
      }
    const bool resumed = !jb.resume.empty();
    rc = install(ctx, slot, ctx->mols[slot], resumed ? jb.resume_step : -(long long)ctx->P.nnlup);
    if (rc == SOP_ERR_CAPACITY) {
      ctx->mols[slot] = HostMol();
      ++it;
      ++looked;
      continue;
    }
    if (rc) return rc;
    if (resumed) {
      // the job continues at its checkpoint's step: its state and lists come
      // from the checkpoint, and the binning below sets the molecule's grid flags
      rc = restore_into(ctx, slot, jb.resume.data(), (long long)jb.resume.size());
      if (rc) return rc;
      jb.resume.clear();
      jb.resume.shrink_to_fit();
      rebin = true;
    }
    ctx->free_slots.pop_back();
    ctx->slot_job[slot] = *it;
    jb.slot = slot;
    jb.state = Job::ACTIVE;
    jb.mol = HostMol();
    it = ctx->queue.erase(it);
  }
  update_live(ctx);
  if (rebin) {
    launch_rebin(ctx->s, ctx->w, ctx->stream);
    CK(cudaGetLastError());
  }
  bool any = false;
  for (int id : ctx->slot_job) any |= id >= 0;
  if (any) return step_async(ctx, ctx->P.nnlup);
  return SOP_OK;
}

extern "C" {

int sop_add_molecule(void* p, const sop_molecule* m, int* mol_id) {
  if (!p || !m) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx->committed) return ctx->fail(SOP_ERR_ARG, "context already committed");
  HostMol h;
  int rc = make_hostmol(ctx, m, h);
  if (rc) return rc;
  ctx->mols.push_back(std::move(h));
  if (mol_id) *mol_id = (int)ctx->mols.size() - 1;
  return SOP_OK;
}

int sop_serve_create(const sop_params* p, long long budget_bytes, long long max_job_beads,
                     void** out) {
  if (!p || !out || budget_bytes <= 0 || max_job_beads <= 0 || max_job_beads > kMaxMolBeads)
    return SOP_ERR_ARG;
  if (p->nnlup <= 0) {
    g_lib_error = "serving needs a neighbour-list cadence (nnlup > 0)";
    return SOP_ERR_ARG;
  }
  int rc = sop_ctx_create(p, out);
  if (rc) return rc;
  SopCtx* ctx = C(*out);
  ctx->served = true;
  ctx->budget = budget_bytes;
  // graph blocks must tile the neighbour-list period
  int P = graph_steps(ctx);
  if (ctx->P.nnlup % P) ctx->P.graph_steps = std::gcd(P, ctx->P.nnlup);
  set_constants(ctx);
  const long long stride = dense_stride(ctx, max_job_beads);
  // bytes per bead slot: state (8 float4), counters and cell data (10 ints),
  // rows (3 int2), topology (2 bond, 2 angle, 8 native entries) and list rows
  // (neighbour and pair list, 16-bit entries)
  const long long per_bead = 128 + 40 + 24 + 16 + 8 + 8 * 48 + 4 * stride;
  Caps c;
  c.beads = std::max<long long>(max_job_beads, budget_bytes / per_bead);
  c.mols = std::max<long long>(64, c.beads / 50);
  c.bonds = 2 * c.beads;
  c.angles = 2 * c.beads;
  c.natives = 8 * c.beads;
  c.cells = 2 * c.beads + 64 * c.mols;
  c.max_mol_beads = max_job_beads;
  c.stride = stride;
  rc = alloc_pools(ctx, c);
  if (rc) {
    std::string msg = ctx->err;
    sop_ctx_destroy(*out);
    *out = nullptr;
    g_lib_error = msg;
    return rc;
  }
  ctx->s.uniform_type = 1;
  ctx->s.long_rows = 0;  // a served mix is mostly molecules far below kLongRowBeads
  ctx->mols.assign(c.mols, HostMol());
  ctx->slot_job.assign(c.mols, -1);
  // a served context fills up and empties as jobs come and go, so its step
  // shape is fixed rather than timed once: 4 lanes per bead, two kernels
  // (the faster form for a populated context) unless the parameters say
  const int fixed_g = lanes_for(ctx), fixed_f = split_for(ctx);
  ctx->G = fixed_g ? fixed_g : 4;
  ctx->split = fixed_f != 1;
  ctx->persist = false;
  ctx->one_block = false;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->committed = true;
  ctx->host_step = 0;
  ctx->target_step = 0;
  return SOP_OK;
}

int sop_serve_submit(void* p, const sop_molecule* m, int* job) {
  if (!p || !m) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->served) return ctx->fail(SOP_ERR_ARG, "not a served context");
  if (m->nsteps < 0) return ctx->fail(SOP_ERR_ARG, "a job needs a step budget (nsteps >= 0)");
  if (m->nbead > ctx->caps.max_mol_beads)
    return ctx->fail(SOP_ERR_BUDGET, "job larger than the context's max_job_beads");
  Job jb;
  int rc = make_hostmol(ctx, m, jb.mol);
  if (rc) return rc;
  jb.n = m->nbead;
  jb.nsteps = m->nsteps;
  jb.t_submit = now_seconds();
  ctx->jobs.push_back(std::move(jb));
  const int id = (int)ctx->jobs.size() - 1;
  ctx->queue.push_back(id);
  if (job) *job = id;
  return SOP_OK;
}

int sop_serve_advance(void* p, int rounds) {
  if (!p || rounds < 0) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->served) return ctx->fail(SOP_ERR_ARG, "not a served context");
  for (int r = 0; r < rounds; ++r) {
    int rc = serve_round(ctx);
    if (rc) return rc;
  }
  return SOP_OK;
}

int sop_serve_finished(void* p, int cap, int* jobs, int* count) {
  if (!p || cap < 0) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int k = 0;
  while (k < cap && !ctx->finished_new.empty()) {
    if (jobs) jobs[k] = ctx->finished_new.front();
    ctx->finished_new.erase(ctx->finished_new.begin());
    ++k;
  }
  if (count) *count = k;
  return SOP_OK;
}

int sop_serve_result(void* p, int job, float* unc_pos, float* vel, double* energy, int* status,
                     long long* steps, double* latency_s) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (job < 0 || job >= (int)ctx->jobs.size()) return ctx->fail(SOP_ERR_NOT_FOUND, "unknown job");
  const Job& jb = ctx->jobs[job];
  if (jb.state != Job::FINISHED) return ctx->fail(SOP_ERR_ARG, "job not finished");
  if (unc_pos) std::memcpy(unc_pos, jb.unc.data(), sizeof(float) * jb.unc.size());
  if (vel) std::memcpy(vel, jb.vel.data(), sizeof(float) * jb.vel.size());
  if (energy) std::memcpy(energy, jb.energy, sizeof(jb.energy));
  if (status) *status = jb.status;
  if (steps) *steps = jb.steps;
  if (latency_s) *latency_s = jb.t_done - jb.t_submit;
  return SOP_OK;
}

int sop_serve_stats(void* p, long long* out) {
  if (!p || !out) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  long long active = 0, beads = 0, done = 0;
  for (const Job& jb : ctx->jobs) {
    if (jb.state == Job::ACTIVE) { ++active; beads += jb.n; }
    if (jb.state == Job::FINISHED) ++done;
  }
  out[0] = (long long)ctx->queue.size();
  out[1] = active;
  out[2] = done;
  out[3] = beads;
  out[4] = ctx->caps.beads;
  out[5] = ctx->bytes;
  out[6] = ctx->budget;
  out[7] = ctx->host_step;
  return SOP_OK;
}

int sop_commit(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx->committed) return ctx->fail(SOP_ERR_ARG, "context already committed");
  cudaSetDevice(ctx->P.device);
  return commit(ctx);
}

int sop_upload_topology(void* p, const sop_molecule* m) {
  int rc = sop_add_molecule(p, m, nullptr);
  if (rc) return rc;
  return sop_commit(p);
}

int sop_upload_state(void* p, int mol, const float* pos, const float* unc_pos, const float* vel) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  long long step;
  rc = read_step(ctx, mol, &step);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  const int cur = (int)(step & 1);
  std::vector<float4> buf(hm.n);
  std::vector<float4> old(hm.n);
  CK(cudaMemcpy(old.data(), ctx->s.x[cur] + hm.start, sizeof(float4) * hm.n, cudaMemcpyDeviceToHost));
  // the new state goes to both coordinate buffers: the lists are rebuilt from
  // it at block offset -1 (before this step's force evaluation), and the
  // force evaluation reads buffer step & 1
  if (unc_pos) {
    for (int i = 0; i < hm.n; ++i)
      buf[i] = make_float4(unc_pos[3 * i], unc_pos[3 * i + 1], unc_pos[3 * i + 2], old[i].w);
    for (int b = 0; b < 2; ++b)
      CK(cudaMemcpy(ctx->s.x[b] + hm.start, buf.data(), sizeof(float4) * hm.n, cudaMemcpyHostToDevice));
  }
  const float* pp = pos ? pos : unc_pos;
  if (pp) {
    for (int i = 0; i < hm.n; ++i) buf[i] = make_float4(pp[3 * i], pp[3 * i + 1], pp[3 * i + 2], 0.f);
    for (int b = 0; b < 2; ++b)
      CK(cudaMemcpy(ctx->s.p[b] + hm.start, buf.data(), sizeof(float4) * hm.n, cudaMemcpyHostToDevice));
  }
  if (vel) {
    for (int i = 0; i < hm.n; ++i) buf[i] = make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.f);
    CK(cudaMemcpy(ctx->s.v + hm.start, buf.data(), sizeof(float4) * hm.n, cudaMemcpyHostToDevice));
  }
  // the lists of this molecule alone: the others keep theirs (built from
  // their own step's coordinates; buffer step - 1 holds their look-ahead)
  rc = nl_rebuild_checked(ctx, -1, mol);
  if (rc) return rc;
  DevSys one = ctx->s;
  one.only_mol = mol;
  launch_pl_rebuild(one, -1, ctx->stream);
  force_eval_async(ctx);  // every molecule: the same forces again for the others
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_step(void* p, long long nsteps) {
  if (!p || nsteps < 0) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = step_async(ctx, nsteps);
  if (rc) return rc;
  return sync_checked(ctx);
}

int sop_step_async(void* p, long long nsteps) {
  if (!p || nsteps < 0) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  return step_async(ctx, nsteps);
}

int sop_sync(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  if (ctx->copy_stream) CK(cudaStreamSynchronize(ctx->copy_stream));
  return SOP_OK;
}

int sop_launch_stage(void* p, int stage, int koff) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  switch (stage) {
    case 0: launch_steps(ctx, koff, 1); break;
    case 1: launch_pl_rebuild(ctx->s, koff, ctx->stream); break;
    case 2: launch_nl_rebuild(ctx->s, ctx->w, koff, ctx->stream); break;
    case 3: launch_advance(ctx->s, koff, ctx->stream); break;
    default: return ctx->fail(SOP_ERR_ARG, "unknown stage");
  }
  CK(cudaGetLastError());
  return SOP_OK;
}

int sop_update_neighbor_list(void* p, long long* nnl_att, long long* nnl_rep) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  rc = nl_rebuild_checked(ctx, 0);
  if (rc) return rc;
  if (nnl_att || nnl_rep) {
    std::vector<int> a(ctx->s.nbead), r(ctx->s.nbead);
    CK(cudaMemcpy(a.data(), ctx->s.nl_att_cnt, sizeof(int) * a.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r.data(), ctx->s.nl_cnt, sizeof(int) * r.size(), cudaMemcpyDeviceToHost));
    long long sa = 0, sr = 0;
    for (int v : a) sa += v;
    for (int v : r) sr += v;
    if (nnl_att) *nnl_att = sa / 2;
    if (nnl_rep) *nnl_rep = sr / 2;
  }
  return SOP_OK;
}

int sop_update_pair_list(void* p, long long* nil_att, long long* nil_rep) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  launch_pl_rebuild(ctx->s, 0, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  if (nil_att || nil_rep) {
    std::vector<int> a(ctx->s.nbead), r(ctx->s.nbead);
    CK(cudaMemcpy(a.data(), ctx->s.pl_att_cnt, sizeof(int) * a.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(r.data(), ctx->s.pl_cnt, sizeof(int) * r.size(), cudaMemcpyDeviceToHost));
    long long sa = 0, sr = 0;
    for (int v : a) sa += v;
    for (int v : r) sr += v;
    if (nil_att) *nil_att = sa / 2;
    if (nil_rep) *nil_rep = sr / 2;
  }
  return SOP_OK;
}

int sop_force_eval(void* p) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  force_eval_async(ctx);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_set_noise(void* p, const float* normals) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  if (normals) {
    if (!ctx->s.noise) {
      ctx->s.noise = ctx->dalloc<float4>(ctx->s.nbead);
      if (!ctx->s.noise) return ctx->fail(SOP_ERR_ALLOC, "noise buffer allocation failed");
    }
    std::vector<float4> b(ctx->s.nbead);
    for (int i = 0; i < ctx->s.nbead; ++i)
      b[i] = make_float4(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2], 0.f);
    CK(cudaMemcpy(ctx->s.noise, b.data(), sizeof(float4) * b.size(), cudaMemcpyHostToDevice));
    ctx->s.use_noise = 1;
  } else {
    ctx->s.use_noise = 0;
  }
  ctx->drop_graphs();  // kernel arguments changed
  return SOP_OK;
}

int sop_download(void* p, int mol, float* pos, float* unc_pos, float* vel, float* force) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  long long step;
  rc = read_step(ctx, mol, &step);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  const int cur = (int)(step & 1);
  if (pos && (rc = copy3(ctx, pos, ctx->s.p[cur] + hm.start, hm.n))) return rc;
  if (unc_pos && (rc = copy3(ctx, unc_pos, ctx->s.x[cur] + hm.start, hm.n))) return rc;
  if (vel && (rc = copy3(ctx, vel, ctx->s.v + hm.start, hm.n))) return rc;
  if (force && (rc = copy3(ctx, force, ctx->s.f + hm.start, hm.n))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_download_list(void* p, int mol, int which, long long cap, int* i_out, int* j_out,
                      float* r0_out, long long* count) {
  if (!p || which < 0 || which > 3) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  const int n = hm.n, o = hm.start;
  long long k = 0;
  auto emit = [&](int i, int j, float r0) {
    if (j <= i) return;
    if (k < cap) {
      if (i_out) i_out[k] = i;
      if (j_out) j_out[k] = j;
      if (r0_out) r0_out[k] = r0;
    }
    ++k;
  };
  if (which == 0 || which == 2) {
    std::vector<int2> row(n);
    std::vector<int> cnt(n);
    CK(cudaMemcpy(row.data(), ctx->s.nat_row + o, sizeof(int2) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cnt.data(), (which == 0 ? ctx->s.nl_att_cnt : ctx->s.pl_att_cnt) + o,
                  sizeof(int) * n, cudaMemcpyDeviceToHost));
    if (n > 0) {
      int lo = row[0].x, hi = row[n - 1].x + row[n - 1].y;
      size_t len = (size_t)std::max(hi - lo, 0);
      if (which == 0) {
        std::vector<int> e(len), nj(ctx->s.nbead > 0 ? len : 0);
        std::vector<float4> par(len);
        if (len) {
          CK(cudaMemcpy(e.data(), ctx->s.nl_att_e + lo, sizeof(int) * len, cudaMemcpyDeviceToHost));
          CK(cudaMemcpy(nj.data(), ctx->s.nat_j + lo, sizeof(int) * len, cudaMemcpyDeviceToHost));
          CK(cudaMemcpy(par.data(), ctx->s.nat_par + lo, sizeof(float4) * len, cudaMemcpyDeviceToHost));
        }
        for (int i = 0; i < n; ++i)
          for (int t = 0; t < cnt[i]; ++t) {
            int idx = e[row[i].x - lo + t] - lo;
            emit(i, nj[idx] - o, par[idx].x);
          }
      } else {
        std::vector<float4> q(len);
        if (len) CK(cudaMemcpy(q.data(), ctx->s.pl_att + lo, sizeof(float4) * len, cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; ++i)
          for (int t = 0; t < cnt[i]; ++t) {
            float4 v = q[row[i].x - lo + t];
            emit(i, bits_i(v.x) - o, v.y);
          }
      }
    }
  } else {
    std::vector<int> cnt(n);
    CK(cudaMemcpy(cnt.data(), (which == 1 ? ctx->s.nl_cnt : ctx->s.pl_cnt) + o, sizeof(int) * n,
                  cudaMemcpyDeviceToHost));
    const long long stride = ctx->s.nl_stride;
    std::vector<int> jj;
    int rc = read_rows(ctx, which == 1 ? 0 : 1, o, n, jj);
    if (rc) return rc;
    for (int i = 0; i < n; ++i)
      for (int t = 0; t < cnt[i]; ++t) emit(i, jj[(size_t)i * stride + t], 0.f);
  }
  if (count) *count = k;
  return SOP_OK;
}

int sop_list_sizes(void* p, long long* out) {
  if (!p || !out) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  const int* src[4] = {ctx->s.nl_att_cnt, ctx->s.nl_cnt, ctx->s.pl_att_cnt, ctx->s.pl_cnt};
  std::vector<int> h(ctx->s.nbead);
  for (int t = 0; t < 4; ++t) {
    CK(cudaMemcpy(h.data(), src[t], sizeof(int) * h.size(), cudaMemcpyDeviceToHost));
    long long sum = 0;
    for (int v : h) sum += v;
    out[t] = sum / 2;  // full rows hold each pair twice
  }
  return SOP_OK;
}

int sop_download_all(void* p, float* unc_pos) {
  if (!p || !unc_pos) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  if (!ctx->stage) {
    ctx->stage = ctx->dalloc<float4>(ctx->s.nbead);
    if (!ctx->stage) return ctx->fail(SOP_ERR_ALLOC, "staging buffer allocation failed");
  }
  // the staging buffer (nbead float4) holds the packed 3 * nbead floats
  float* packed = reinterpret_cast<float*>(ctx->stage);
  launch_gather_current(ctx->s, packed, nullptr, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(unc_pos, packed, sizeof(float) * 3 * (size_t)ctx->s.nbead,
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SOP_OK;
}

int sop_download_all_async(void* p, float* unc_pos, long long* ticket) {
  if (!p || !unc_pos || !ticket) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  if (!ctx->copy_stream) {
    CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      CK(cudaEventCreateWithFlags(&ctx->gathered[k], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->copied[k], cudaEventDisableTiming));
    }
    CK(cudaMallocHost(&ctx->h_flag, 2 * sizeof(int)));
    ctx->h_flag[0] = ctx->h_flag[1] = 0;
  }
  const int k = (int)(ctx->next_ticket & 1);
  if (!ctx->astage[k]) {
    // packed xyz (12 B per bead) and the flag word fit in nbead float4
    ctx->astage[k] = ctx->dalloc<float4>((size_t)ctx->s.nbead + 1);
    if (!ctx->astage[k]) return ctx->fail(SOP_ERR_ALLOC, "staging buffer allocation failed");
  }
  const size_t n3 = 3 * (size_t)ctx->s.nbead;
  float* packed = reinterpret_cast<float*>(ctx->astage[k]);
  int* dflag = reinterpret_cast<int*>(packed + n3);
  // the buffer's previous copy must have left it before the gather refills it
  CK(cudaStreamWaitEvent(ctx->stream, ctx->copied[k], 0));
  launch_gather_current(ctx->s, packed, dflag, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->gathered[k], ctx->stream));
  CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->gathered[k], 0));
  CK(cudaMemcpyAsync(unc_pos, packed, sizeof(float) * n3, cudaMemcpyDeviceToHost, ctx->copy_stream));
  CK(cudaMemcpyAsync(ctx->h_flag + k, dflag, sizeof(int), cudaMemcpyDeviceToHost, ctx->copy_stream));
  CK(cudaEventRecord(ctx->copied[k], ctx->copy_stream));
  *ticket = ctx->next_ticket++;
  return SOP_OK;
}

int sop_download_wait(void* p, long long ticket) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ticket < 0 || ticket >= ctx->next_ticket || !ctx->copy_stream)
    return ctx->fail(SOP_ERR_ARG, "no such download");
  // a buffer's event is re-recorded by the download two tickets later, whose
  // copy ends after this one's: waiting on it is never too early
  const int k = (int)(ticket & 1);
  CK(cudaEventSynchronize(ctx->copied[k]));
  if (ctx->h_flag[k] & FLAG_NL_OVERFLOW)
    return ctx->fail(SOP_ERR_CAPACITY,
                     "the neighbour lists overflowed before the download: sop_sync re-runs the "
                     "frozen steps, then download again");
  return SOP_OK;
}

int sop_energy(void* p, int mol, double* terms) {
  if (!p || !terms) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  launch_energy(ctx->s, hm.start, hm.n, mol, ctx->e_part, ctx->e_out,
                0.5 * ctx->P.k_bnd * ctx->P.R0 * ctx->P.R0, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->h_out, ctx->e_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int t = 0; t < 4; ++t) terms[t] = ctx->h_out[t];
  terms[4] = terms[0] + terms[1] + terms[2] + terms[3];  // rna_etot (energy.cu:76)
  return SOP_OK;
}

int sop_observables(void* p, int mol, double* out) {
  if (!p || !out) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  const HostMol& hm = ctx->mols[mol];
  launch_observables(ctx->s, hm.start, hm.n, mol, (int)hm.ni.size(), ctx->e_part, ctx->e_out,
                     ctx->stream);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->h_out, ctx->e_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  for (int t = 0; t < 4; ++t) out[t] = ctx->h_out[t];
  return SOP_OK;
}

int sop_molecule_status(void* p, int mol, int* status, long long* step) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  long long st = 0;
  int flags = 0;
  CK(cudaMemcpy(&st, ctx->s.mol_step + mol, sizeof(long long), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&flags, ctx->s.mol_status + mol, sizeof(int), cudaMemcpyDeviceToHost));
  const MolConst& mc = ctx->mc[mol];
  if (mc.nsteps >= 0 && st >= mc.nsteps) flags |= SOP_MOL_DONE;
  if (status) *status = flags;
  if (step) *step = st;
  return SOP_OK;
}

static int copy_out_ckpt(SopCtx* ctx, const std::vector<char>& blob, void* buf, long long cap,
                         long long* size) {
  if (size) *size = (long long)blob.size();
  if (!buf) return SOP_OK;
  if (cap < (long long)blob.size())
    return ctx->fail(SOP_ERR_CAPACITY, "checkpoint buffer too small (query the size with buf = NULL)");
  std::memcpy(buf, blob.data(), blob.size());
  return SOP_OK;
}

int sop_checkpoint(void* p, int mol, void* buf, long long cap, long long* size) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx->served) return ctx->fail(SOP_ERR_ARG, "served contexts use sop_serve_checkpoint");
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  std::vector<char> blob;
  rc = checkpoint_of(ctx, mol, blob);
  if (rc) return rc;
  return copy_out_ckpt(ctx, blob, buf, cap, size);
}

int sop_restore(void* p, int mol, const void* buf, long long size) {
  if (!p || !buf) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx->served) return ctx->fail(SOP_ERR_ARG, "served contexts use sop_serve_resume");
  int rc = check_mol(ctx, mol);
  if (rc) return rc;
  rc = sync_checked(ctx);
  if (rc) return rc;
  CkptHeader h;
  if (!ckpt_head(buf, size, &h)) return ctx->fail(SOP_ERR_ARG, "not a checkpoint of this format");
  const long long step = h.step;
  // one clock per context: the first restore into a context that has not
  // stepped sets it; later ones must match it
  const bool set_clock = !ctx->stepped && ctx->host_step == 0;
  if (!set_clock && step != ctx->host_step)
    return ctx->fail(SOP_ERR_ARG, "checkpoint step differs from the context's step");
  rc = restore_into(ctx, mol, static_cast<const char*>(buf), size);
  if (rc) return rc;
  // refresh each molecule's grid flags (and the cell order) from the restored
  // coordinates: binning only, no list changes
  launch_rebin(ctx->s, ctx->w, ctx->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  if (set_clock) {
    ctx->host_step = ctx->target_step = step;
    CK(cudaMemcpy(ctx->s.sys_step, &step, sizeof(long long), cudaMemcpyHostToDevice));
  }
  return SOP_OK;
}

int sop_serve_checkpoint(void* p, int job, void* buf, long long cap, long long* size) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->served) return ctx->fail(SOP_ERR_ARG, "not a served context");
  if (job < 0 || job >= (int)ctx->jobs.size()) return ctx->fail(SOP_ERR_NOT_FOUND, "unknown job");
  if (ctx->jobs[job].state != Job::ACTIVE) return ctx->fail(SOP_ERR_ARG, "job is not running");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  std::vector<char> blob;
  rc = checkpoint_of(ctx, ctx->jobs[job].slot, blob);
  if (rc) return rc;
  return copy_out_ckpt(ctx, blob, buf, cap, size);
}

int sop_serve_resume(void* p, const sop_molecule* m, const void* buf, long long size, int* job) {
  if (!p || !m || !buf) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->served) return ctx->fail(SOP_ERR_ARG, "not a served context");
  CkptHeader h;
  if (!ckpt_head(buf, size, &h)) return ctx->fail(SOP_ERR_ARG, "not a checkpoint of this format");
  if (h.n != m->nbead || h.nnat2 != 2 * m->nnat)
    return ctx->fail(SOP_ERR_ARG, "checkpoint of a different molecule");
  const long long step = h.step;
  // admission happens where the context's neighbour-list period starts, so
  // the job's own cadence lines up only for steps at that phase -- where a
  // served job's checkpoint is taken between rounds
  if (step % ctx->P.nnlup != 0)
    return ctx->fail(SOP_ERR_ARG, "a served job resumes from a step that is a multiple of nnlup");
  if (m->nsteps < step) return ctx->fail(SOP_ERR_ARG, "checkpoint beyond the job's step budget");
  int id = -1;
  int rc = sop_serve_submit(p, m, &id);
  if (rc) return rc;
  Job& jb = ctx->jobs[id];
  jb.resume.assign(static_cast<const char*>(buf), static_cast<const char*>(buf) + size);
  jb.resume_step = step;
  if (job) *job = id;
  return SOP_OK;
}

int sop_memory(void* p, int mol, long long* ctx_bytes, long long* mol_bytes) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (ctx_bytes) *ctx_bytes = ctx->bytes;
  if (mol_bytes) {
    if (mol < 0 || mol >= (int)ctx->mols.size()) return ctx->fail(SOP_ERR_NOT_FOUND, "unknown molecule");
    const HostMol& hm = ctx->mols[mol];
    long long per_bead = 7 * 16 + 4 * 10 + 16 + 3 * 8;
    long long nl = ctx->s.nl_stride * 4LL * hm.n;   // two rows of 16-bit entries
    *mol_bytes = per_bead * hm.n + nl + (long long)(hm.bi.size() + hm.ai.size()) * 16 +
                 (long long)hm.ni.size() * 2 * 40;
  }
  return SOP_OK;
}

int sop_tuning(void* p, int* lanes, float* ms) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (lanes) *lanes = ctx->G;
  if (ms) {
    const int cand[4] = {2, 4, 8, 16};
    for (int k = 0; k < 4; ++k) {
      auto it = ctx->tuning.find(cand[k]);
      ms[k] = it == ctx->tuning.end() ? 0.0f : it->second;
    }
  }
  return SOP_OK;
}

int sop_step_form(void* p, int* lanes, int* form) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (lanes) *lanes = ctx->G;
  if (form) *form = ctx->one_block ? 4 : ctx->persist ? 3 : ctx->split ? 2 : 1;
  return SOP_OK;
}

int sop_check_step_barrier(void* p, int missing, double timeout_s, int* timed_out) {
  if (!p || !timed_out || missing < 0 || !(timeout_s > 0.0) || timeout_s > 10.0)
    return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (!ctx->committed) return ctx->fail(SOP_ERR_ARG, "context not committed");
  int rc = sync_checked(ctx);
  if (rc) return rc;
  CK(launch_barrier_check(ctx->s, ctx->G, barrier_words(ctx), missing, 3,
                          (unsigned long long)(timeout_s * 1e9), ctx->stream));
  int flags = 0;
  CK(cudaMemcpyAsync(&flags, ctx->s.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *timed_out = (flags & FLAG_BARRIER_TIMEOUT) ? 1 : 0;
  if (*timed_out) {
    CK(cudaMemsetAsync(ctx->s.flags, 0, 4 * sizeof(int), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return SOP_OK;
}

int sop_step_buckets(void* p, int* tiled, int* lanes, int* forms, long long* beads, float* ms) {
  if (!p) return SOP_ERR_ARG;
  SopCtx* ctx = C(p);
  if (tiled) *tiled = ctx->tiled ? 1 : 0;
  for (int b = 0; b < kBuckets; ++b) {
    if (lanes) lanes[b] = ctx->bucket_lanes[b];
    if (forms) forms[b] = ctx->bucket_form[b];
    if (beads) beads[b] = ctx->bucket_beads[b];
  }
  if (ms) { ms[0] = ctx->ms_tiled; ms[1] = ctx->ms_whole; }
  return SOP_OK;
}

int sop_step_window(void* p, int* wcap) {
  if (!p || !wcap) return SOP_ERR_ARG;
  *wcap = C(p)->wcap;
  return SOP_OK;
}

int sop_stream(void* p, void** stream) {
  if (!p || !stream) return SOP_ERR_ARG;
  *stream = (void*)C(p)->stream;
  return SOP_OK;
}

const char* sop_last_error(void* p) {
  if (!p) return g_lib_error.c_str();
  return C(p)->err.c_str();
}

}  // extern "C"

// Host side of the C ABI (include/brownian_gb300.h): the context that owns the
// device-resident state, the constants derived from the parameters, the launch
// sequence of one MPCD step (captured once into a CUDA graph and replayed), the
// routine-level entry points, initialisation and diagnostics.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/brownian_gb300.h"
#include "traj_internal.h"
#include "kernels.cuh"

using namespace bgb;

namespace {

struct ProfEvent {
  const char *name;
  cudaEvent_t a, b;
};

struct DevAlloc {
  std::vector<void *> ptrs;
  cudaError_t err = cudaSuccess;
  template <typename T>
  T *get(size_t n) {
    void *p = nullptr;
    if (err == cudaSuccess) {
      err = cudaMalloc(&p, n * sizeof(T) + 16);
      if (err == cudaSuccess) {
        ptrs.push_back(p);
        cudaMemset(p, 0, n * sizeof(T) + 16);
      }
    }
    return (T *)p;
  }
  void release() {
    for (void *p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

}  // namespace

struct mpcd_ctx {
  mpcd_params p;
  SysF64 S;
  DevAlloc mem;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t aux = nullptr;    // second stream: colloid work beside the fluid passes
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // free-flight schedule (mpcd_step): the near particles' substeps run
  // on nst (high priority) beside the free particles' pass on the context's stream
  cudaStream_t nst = nullptr;
  cudaEvent_t ev_tab = nullptr, ev_cls = nullptr, ev_end = nullptr, ev_list = nullptr, ev_free = nullptr;
  bool flight = true;
  cudaStream_t evs = nullptr;    // third stream (FP64 form): event passes and colloid finish
  cudaEvent_t ev_start = nullptr, ev_str = nullptr, ev_aux = nullptr, ev_finp[2] = {nullptr, nullptr};

  cudaGraphExec_t step_exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [sorts][fluid buffer]
  int step_launches[2][2] = {{0, 0}, {0, 0}};
  int fbuf = 0;                  // fluid buffer holding the current state
  long long host_step = 0;       // completed steps (mirror of the device counter)
  int sort_every = 10;           // counting sort by cell every this many steps
  bool setup_done = false;
  std::string err;
  int64_t launches = 0;
  bool profile = false;
  std::vector<ProfEvent> pending;
  std::vector<cudaEvent_t> event_pool;
  bool tracing = false;          // capturing a traced step (mpcd_trace_step)
  std::vector<ProfEvent> trace;  // its launches, each between two timing events
  std::map<std::string, std::pair<int64_t, double>> prof;
  StepState *ss_host = nullptr;  // pinned
  double *insw_n = nullptr, *sqcs_n = nullptr;
  float *sq3kt_n32 = nullptr;
  double *part = nullptr;        // reduction partials
  int part_blocks = 256;
  double *staging = nullptr;     // AoS transfer buffer, allocated on first use
  double *staging2 = nullptr;    // second one (FP32 form: velocities)
  double *diag_host = nullptr;   // page-locked: what mpcd_diag reads, allocated on first use
  int phase = 0;                 // 0: between steps; 1: rotation_mpcd of the next step done
  int next_sub = 1;              // routine-level: the substep mpcd_substep expects
  int nblk = 0;                  // 256-cell blocks of the counting sort
  int n_sm = 152;                // multiprocessors of the device
  int ev_grid = 0, ev_block = 128;   // k_events launch shape (grid 0: one block per SM)
  // updown_velocity scratch, allocated on first use
  unsigned long long *ud_Tc = nullptr;
  uint16_t *ud_Tl = nullptr;
  int *ud_cnt = nullptr;
  ExchAcc *ud_acc = nullptr;
  long long ud_epoch = -1;
  int fin_grid = 0, fin_block = 32;  // k_fin launch shape (grid 0: one block per SM)
  int free_grid = 0;                 // free-flight pass blocks of 256 (0: the form's default)
  int free_after = -1;               // the substep after whose colloid finish the free pass starts
                                     // (0: after the classification; -1: the form's default)
  // routine-by-routine substep: the next routine of the substep body (0: update_pos_md)
  int rseq = 0;
  // neighbour_list_mpcd observables (allocated on first use): box of each particle,
  // occupancy of each box, candidates of each colloid
  int *box_cell = nullptr, *box_occ = nullptr, *box_nn = nullptr;
  bool box_valid = false;
};

static int fail(mpcd_ctx *c, int code, const std::string &m) {
  if (c) c->err = m;
  return code;
}

#define CUDA_OK(c, call)                                                                     \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return fail((c), MPCD_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

static long long dbits_h(double x) {
  long long b;
  memcpy(&b, &x, 8);
  return b;
}

static Dim make_dim(int L) {
  Dim d;
  d.L = (double)L;
  d.halfL = d.L / 2;
  d.lo_bits = dbits_h(ldexp(d.L, -30));
  d.L_bits = dbits_h(d.L);
  d.img_bits = dbits_h(0.49 * d.L);
  d.img1_bits = dbits_h(0.51 * d.L);
  d.img2_bits = dbits_h(1.49 * d.L);
  return d;
}

// ---------------------------------------------------------------- launching

static cudaEvent_t pool_event(mpcd_ctx *c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

template <typename... KArgs, typename... Args>
static void launch_on(mpcd_ctx *c, cudaStream_t s, const char *name, void (*k)(KArgs...), dim3 g, dim3 b,
                      Args... args) {
  ProfEvent pe{name, nullptr, nullptr};
  if (c->profile || c->tracing) {
    pe.a = pool_event(c);
    pe.b = pool_event(c);
    // (in a traced capture the records become nodes of the graph)
    cudaEventRecordWithFlags(pe.a, s, c->tracing ? cudaEventRecordExternal : cudaEventRecordDefault);
  }
  k<<<g, b, 0, s>>>(args...);
  c->launches++;
  if (c->profile || c->tracing) {
    cudaEventRecordWithFlags(pe.b, s, c->tracing ? cudaEventRecordExternal : cudaEventRecordDefault);
    (c->tracing ? c->trace : c->pending).push_back(pe);
  }
}

template <typename... KArgs, typename... Args>
static void launch(mpcd_ctx *c, const char *name, void (*k)(KArgs...), dim3 g, dim3 b, Args... args) {
  launch_on(c, c->stream, name, k, g, b, args...);
}

// a copy ordered on the context's stream (which does not synchronise with the
// legacy default stream), complete on return
static cudaError_t scopy(const mpcd_ctx *c, void *dst, const void *src, size_t n, cudaMemcpyKind kind) {
  cudaError_t e = cudaMemcpyAsync(dst, src, n, kind, c->stream);
  return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}

static unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// the pair-list grid for a list radius rl: per axis as many buckets as fit with width
// at least rl (with 1e-4 to spare for the rounding of the bucket index), at most NBK_MAX
static NListGeo nlist_geo(const mpcd_ctx *c, double rl) {
  NListGeo g;
  const int L[3] = {c->S.Lx, c->S.Ly, c->S.Lz};
  for (int a = 0; a < 3; ++a) {
    int nb = (int)floor((double)L[a] / (rl * 1.0001));
    nb = nb < 1 ? 1 : (nb > NBK_MAX ? NBK_MAX : nb);
    g.nb[a] = nb;
    g.bs[a] = (double)L[a] / nb;
  }
  g.r2 = pow(rl, 2);
  return g;
}

// the free-flight schedule's pair list at the positions at the start of the step, on
// stream s (recorded as ev_list): radius r_cutoff + 2 n_sub cmargin + 0.05, within which
// every pair that comes within r_cutoff during the step starts (each colloid moves at most
// cmargin a substep; the colloid finish fails a step in which one moves further)
static void enq_step_pairs(mpcd_ctx *c, cudaStream_t s) {
  if (!c->S.vlist) return;
  const NListGeo geo = nlist_geo(c, c->S.r_cutoff + 2.0 * c->S.n_sub * sqrt(c->S.cmargin2) + 0.05);
  launch_on(c, s, "k_cbucket", k_cbucket, 1, 1024, c->S, (const double *)nullptr, geo);
  launch_on(c, s, "k_nlist_step", k_nlist_step, blocks_for(c->S.Nc, 4), 128, c->S, geo);
  cudaEventRecord(c->ev_list, s);
}

static int colloid_grid(const mpcd_ctx *c) {
  int g = (int)blocks_for((long long)c->S.Nc * 32, 128);
  return g > 0 ? g : 1;
}

static const char *stream_name(int flags) {
  flags &= ~F_PIPE;
  return flags == (F_STREAM | F_COLLIDE) ? "k_stream"
         : flags == (F_STREAM | F_COLLIDE | F_SHELL | F_BINROT) ? "k_stream_last"
         : flags == (F_SHELL | F_BINROT) ? "k_stream_setup" : "k_stream_other";
}

// One substep's fluid passes in stream order (the FP64 form's substep kernels are
// the overlapped ones, F_PIPE, whose results do not depend on the schedule).
static void enq_stream(mpcd_ctx *c, int flags, int l, int act) {
  const int fb = c->fbuf;
  const bool f32 = c->S.precision == MPCD_FP32C;
  if (!f32 && (flags & F_STREAM)) flags |= F_PIPE;
  const char *name = stream_name(flags);
  // The colloid forces, the next cell table and the orientation work of a substep
  // need nothing the fluid passes write: they run as a kernel of their own (which
  // keeps the streaming pass at its own, low register count) on the second,
  // high-priority stream, whose few blocks start as streaming blocks retire.
  const bool fork = (flags & F_STREAM) && c->S.Nc > 0;
  if (fork) {
    cudaEventRecord(c->ev_fork, c->stream);
    cudaStreamWaitEvent(c->aux, c->ev_fork, 0);
  }
  launch(c, name, f32 ? stream_kernel32(flags) : stream_kernel(flags),
         blocks_for(c->S.N, 256 * (f32 ? stream32_per_thread(flags) : stream64_per_thread(flags))), 256, c->S, l, fb);
  if (!f32 && (flags & F_PIPE) && (flags & F_BINROT)) launch(c, "k_bin", k_bin, c->n_sm * 8, 256, c->S, fb);
  if (fork) {
    launch_on(c, c->aux, "k_aux", k_aux, c->S.Nc, 32 * c->S.aux_nw, c->S, l, act, 0);
    cudaEventRecord(c->ev_join, c->aux);
  }
  // the particles it left near a sphere surface, one per lane
  launch(c, "k_events", f32 ? event_kernel32(flags) : event_kernel(flags), c->ev_grid > 0 ? c->ev_grid : c->n_sm,
         c->ev_block, c->S, l, fb);
  if (fork) cudaStreamWaitEvent(c->stream, c->ev_join, 0);  // k_fin reads the forces and the orientation
}

static void enq_fin_on(mpcd_ctx *c, cudaStream_t s, int mode, int l) {
  if (c->S.fin_table) {
    // a block of eight warps per colloid: warp 0 the colloid, all eight its cell table
    launch_on(c, s, "k_fin", k_fin, c->S.Nc > 0 ? c->S.Nc : 1, 256, c->S, mode, l);
    return;
  }
  // one warp per colloid (warp j / grid of block j % grid): each SM's FP64 unit
  // serves the chains of a few colloids only
  int g = c->fin_grid > 0 ? c->fin_grid : c->n_sm;
  const int nc = c->S.Nc > 0 ? c->S.Nc : 1;
  if (g > nc) g = nc;
  int w = c->fin_block / 32;
  if ((long long)g * w < nc) w = (int)blocks_for(nc, g);
  if (w > 4) {
    w = 4;
    g = (int)blocks_for(nc, 4);
  }
  launch_on(c, s, "k_fin", k_fin, g, 32 * w, c->S, mode, l);
}

static void enq_fin(mpcd_ctx *c, int mode, int l) { enq_fin_on(c, c->stream, mode, l); }

static unsigned prep_blocks(const SysF64 &S) { return blocks_for(S.Cpad > S.Nc ? S.Cpad : S.Nc, 256); }

// the free-flight pass: a persistent grid beside the substeps' chain, whose kernels need room
// on the SMs next to it
static unsigned free_blocks(const mpcd_ctx *c) {
  if (c->free_grid > 0) return (unsigned)c->free_grid;
  return (unsigned)(c->n_sm * 2);
}

// the substep after whose colloid finish the FP64 free pass starts (0: after the
// classification); below n_sub
static int free_after(const mpcd_ctx *c) {
  const int a = c->free_after >= 0 ? c->free_after : 1;
  return a < c->S.n_sub ? a : 0;
}

static bool sorts_at(const mpcd_ctx *c, long long step) { return c->sort_every > 0 && step % c->sort_every == 0; }

// rotation_mpcd: per-cell map (and occupancy prefix), then the rotation, every
// sort_every steps fused with the counting-sort scatter into the other buffer
static void enq_rotation(mpcd_ctx *c, bool sort) {
  const SysF64 &S = c->S;
  const bool f32 = S.precision == MPCD_FP32C;
  launch(c, "k_cell_prep", f32 ? k_cell_prep32 : k_cell_prep, prep_blocks(S), 256, S);
  if (sort) {
    launch(c, "k_scan_blocks", k_scan_blocks, 1, 1024, S, c->nblk);
    launch(c, "k_rotate_sort", f32 ? k_rotate_sort32 : k_rotate_sort, blocks_for(S.N, 256), 256, S, c->fbuf,
           1 - c->fbuf);
    c->fbuf = 1 - c->fbuf;
  } else {
    launch(c, "k_rotate", f32 ? k_rotate32 : k_rotate, blocks_for(S.N, 256), 256, S, c->fbuf);
  }
}

// run(), cpp/run.cpp:10-26: the rear-shell test and count over the candidates the
// last substep recorded, then the compensating kick of the shell fluid
static void enq_run_shell(mpcd_ctx *c, cudaStream_t s, int fb) {
  const bool f32 = c->S.precision == MPCD_FP32C;
  launch_on(c, s, "k_run_shell", f32 ? k_run_shell32 : k_run_shell, 152 * 4, 256, c->S, fb);
}

static void enq_run_kick(mpcd_ctx *c) {
  const bool f32 = c->S.precision == MPCD_FP32C;
  launch(c, "k_run_kick", f32 ? k_run_kick32 : k_run_kick, 152 * 4, 256, c->S, c->fbuf);
}

static void enq_run_fluid(mpcd_ctx *c) {
  if (c->S.Nc == 0) return;
  enq_run_shell(c, c->stream, c->fbuf);
  enq_run_kick(c);
}

// rotation_mpcd and run of a step: the rear-shell test reads only the records, the
// positions and the colloids, none of which the cell pass or the in-place rotation
// touch, so it runs on the side stream beside them (before a sort's scatter, which
// moves the particles and rewrites their slots)
static void enq_rotation_run(mpcd_ctx *c, bool sort) {
  if (c->S.Nc == 0) {
    enq_rotation(c, sort);
    return;
  }
  cudaEventRecord(c->ev_fork, c->stream);
  cudaStreamWaitEvent(c->aux, c->ev_fork, 0);
  enq_run_shell(c, c->aux, c->fbuf);
  cudaEventRecord(c->ev_join, c->aux);
  const SysF64 &S = c->S;
  const bool f32 = S.precision == MPCD_FP32C;
  launch(c, "k_cell_prep", f32 ? k_cell_prep32 : k_cell_prep, prep_blocks(S), 256, S);
  if (sort) {
    cudaStreamWaitEvent(c->stream, c->ev_join, 0);
    launch(c, "k_scan_blocks", k_scan_blocks, 1, 1024, S, c->nblk);
    launch(c, "k_rotate_sort", f32 ? k_rotate_sort32 : k_rotate_sort, blocks_for(S.N, 256), 256, S, c->fbuf,
           1 - c->fbuf);
    c->fbuf = 1 - c->fbuf;
  } else {
    launch(c, "k_rotate", f32 ? k_rotate32 : k_rotate, blocks_for(S.N, 256), 256, S, c->fbuf);
    cudaStreamWaitEvent(c->stream, c->ev_join, 0);
  }
  enq_run_kick(c);
}

// The substeps of the FP64 form, overlapped on three streams.  Per substep l:
//   main   k_stream(l)            needs k_stream(l-1) and k_fin(l-2) (cell table of l,
//                                  positions of l-1)
//   events k_events(l), k_fin(l)  need k_stream(l); k_fin also k_aux(l)
//   aux    k_aux(l)               needs k_fin(l-1) (the positions of substep l)
// so the streaming pass of l+1, bandwidth-bound, runs beside the event pass and the
// colloid finish of l, latency-bound.  k_stream(l+1) tests against the positions
// of l with the displacement bound as margin and leaves the particles k_events(l)
// may be changing (pending) to the event passes; no data of the concurrent passes
// overlap (see the F_PIPE kernels).
static void enq_substeps_overlapped(mpcd_ctx *c) {
  const int n = c->S.n_sub;
  const bool nc = c->S.Nc > 0;
  cudaEventRecord(c->ev_start, c->stream);
  cudaStreamWaitEvent(c->evs, c->ev_start, 0);
  if (nc) cudaStreamWaitEvent(c->aux, c->ev_start, 0);
  for (int l = 1; l <= n; ++l) {
    const int flags = (l == n ? (F_STREAM | F_COLLIDE | F_SHELL | F_BINROT) : (F_STREAM | F_COLLIDE)) | F_PIPE;
    // the cell table of l and the positions of l-1 come from k_fin(l-2)
    if (l >= 3) cudaStreamWaitEvent(c->stream, c->ev_finp[l & 1], 0);
    launch(c, stream_name(flags), stream_kernel(flags), blocks_for(c->S.N, 256 * stream64_per_thread(flags)), 256,
           c->S, l, c->fbuf);
    cudaEventRecord(c->ev_str, c->stream);
    // the last substep's binning beside its event pass and colloid finish
    if (l == n) launch(c, "k_bin", k_bin, c->n_sm * 8, 256, c->S, c->fbuf);
    if (nc) {
      if (l >= 2) cudaStreamWaitEvent(c->aux, c->ev_finp[(l - 1) & 1], 0);
      launch_on(c, c->aux, "k_aux", k_aux, c->S.Nc, 32 * c->S.aux_nw, c->S, l, l >= 2 ? 1 : 0, 0);
      cudaEventRecord(c->ev_aux, c->aux);
    }
    cudaStreamWaitEvent(c->evs, c->ev_str, 0);
    launch_on(c, c->evs, "k_events", event_kernel(flags), c->ev_grid > 0 ? c->ev_grid : c->n_sm, c->ev_block, c->S,
              l, c->fbuf);
    if (nc) cudaStreamWaitEvent(c->evs, c->ev_aux, 0);
    enq_fin_on(c, c->evs, l < n ? (M_FINISH | M_ADVANCE) : (M_FINISH | M_ACT), l);
    cudaEventRecord(c->ev_finp[l & 1], c->evs);
  }
  cudaStreamWaitEvent(c->stream, c->ev_finp[n & 1], 0);
}

// A counting-sort step of the free-flight schedule: the rotation fused with the scatter into
// the other buffer in cell order (the classification then only classifies).  The scatter
// moves the particles and rewrites the slots run()'s rear-shell test reads, so it waits for
// that test (ev_join, on the side stream).
static void enq_sort_scatter(mpcd_ctx *c) {
  const SysF64 &S = c->S;
  const bool f32 = S.precision == MPCD_FP32C;
  cudaStreamWaitEvent(c->stream, c->ev_join, 0);
  launch(c, "k_scan_blocks", k_scan_blocks, 1, 1024, S, c->nblk);
  launch(c, "k_rotate_sort", f32 ? k_rotate_sort32 : k_rotate_sort, blocks_for(S.N, 256), 256, S, c->fbuf, 1 - c->fbuf);
  c->fbuf = 1 - c->fbuf;
}

// One substep of the FP32 free-flight schedule on stream s: the pass over the near list,
// the colloid side work beside it and the event pass, then the colloid finish.
static void enq_substep_near32(mpcd_ctx *c, cudaStream_t s, int l) {
  const SysF64 &S = c->S;
  const int n = S.n_sub;
  const int flags = l == n ? (F_STREAM | F_COLLIDE | F_SHELL | F_BINROT) : (F_STREAM | F_COLLIDE);
  const bool fork = S.Nc > 0;
  if (fork) {
    cudaEventRecord(c->ev_fork, s);
    cudaStreamWaitEvent(c->aux, c->ev_fork, 0);
    if (l == 1 && S.vlist) cudaStreamWaitEvent(c->aux, c->ev_list, 0);
  }
  launch_on(c, s, l == n ? "k_stream_near_last" : "k_stream_near", stream_kernel32_near(flags), c->n_sm * 8, 256, S,
            l, c->fbuf);
  if (fork) {
    launch_on(c, c->aux, "k_aux", k_aux, S.Nc, 32 * S.aux_nw, S, l, l >= 2 ? 1 : 0, S.vlist);
    cudaEventRecord(c->ev_join, c->aux);
  }
  launch_on(c, s, "k_events", event_kernel32(flags), c->ev_grid > 0 ? c->ev_grid : c->n_sm, c->ev_block, S, l,
            c->fbuf);
  if (fork) cudaStreamWaitEvent(s, c->ev_join, 0);
  enq_fin_on(c, s, l < n ? (M_FINISH | M_ADVANCE) : (M_FINISH | M_ACT), l);
}

// One step of the FP32 form in the free-flight schedule.
//   side stream: the flight table (from the colloids' positions at the start of the
//                step), then run()'s rear-shell test;
//   main:        the cell pass; the rotation with the classification (it needs the table);
//                then the free particles' whole step, beside
//   near stream: (high priority) run()'s kick (it needs the shell test; the kicked particles
//                are all near), the colloid kick and the n_sub substeps of the near list;
//   main:        the end of the step, after both.
static void enq_step_flight32(mpcd_ctx *c, bool sort) {
  const SysF64 &S = c->S;
  const int n = S.n_sub;
  cudaEventRecord(c->ev_fork, c->stream);
  cudaStreamWaitEvent(c->aux, c->ev_fork, 0);
  launch_on(c, c->aux, "k_flight_table", k_flight_table32, S.Nc > 0 ? S.Nc : 1, 128, S);
  cudaEventRecord(c->ev_tab, c->aux);
  if (S.vlist) {
    // the step's pair list on the third stream, which this schedule leaves idle; the side
    // work of the first substep waits for it
    cudaStreamWaitEvent(c->evs, c->ev_fork, 0);
    enq_step_pairs(c, c->evs);
  }
  if (S.Nc > 0) enq_run_shell(c, c->aux, c->fbuf);
  cudaEventRecord(c->ev_join, c->aux);
  launch(c, "k_cell_prep", k_cell_prep32, prep_blocks(S), 256, S);
  if (sort) enq_sort_scatter(c);
  cudaStreamWaitEvent(c->stream, c->ev_tab, 0);
  launch(c, "k_rotate_classify", classify_kernel32(!sort), blocks_for(S.N, 256 * CLASSIFY32_U), 256, S, c->fbuf);
  cudaEventRecord(c->ev_cls, c->stream);
  cudaStreamWaitEvent(c->nst, c->ev_cls, 0);
  cudaStreamWaitEvent(c->nst, c->ev_join, 0);
  if (S.Nc > 0) launch_on(c, c->nst, "k_run_kick", k_run_kick32, 152 * 4, 256, S, c->fbuf);
  enq_fin_on(c, c->nst, M_KICK | M_ADVANCE, 0);
  for (int l = 1; l <= n; ++l) enq_substep_near32(c, c->nst, l);
  cudaEventRecord(c->ev_end, c->nst);
  launch(c, "k_free_flight", k_free_flight32, free_blocks(c), 256, S, c->fbuf);
  cudaStreamWaitEvent(c->stream, c->ev_end, 0);
  launch(c, "k_end_step", k_end_step, 1, 256, S);
}

// One step of the FP64 form in the free-flight schedule:
// as the FP32 form's, with the FP64 substeps overlapped as in enq_substeps_overlapped
// (the near list's streaming passes on the near stream; the event pass fused with the
// colloid side work, then the colloid finish, on the event stream) and the near
// particles' binning after the last streaming pass.
static void enq_step_flight64(mpcd_ctx *c, bool sort) {
  const SysF64 &S = c->S;
  const int n = S.n_sub;
  const bool nc = S.Nc > 0;
  cudaEventRecord(c->ev_fork, c->stream);
  cudaStreamWaitEvent(c->aux, c->ev_fork, 0);
  launch_on(c, c->aux, "k_flight_table", k_flight_table32, nc ? S.Nc : 1, 128, S);
  cudaEventRecord(c->ev_tab, c->aux);
  if (S.vlist) {
    // the step's pair list on the event stream before its substeps, whose side work reads it
    cudaStreamWaitEvent(c->evs, c->ev_fork, 0);
    enq_step_pairs(c, c->evs);
  }
  if (nc) enq_run_shell(c, c->aux, c->fbuf);
  cudaEventRecord(c->ev_join, c->aux);
  launch(c, "k_cell_prep", k_cell_prep, prep_blocks(S), 256, S);
  if (sort) enq_sort_scatter(c);
  cudaStreamWaitEvent(c->stream, c->ev_tab, 0);
  launch(c, "k_rotate_classify", classify_kernel(!sort), blocks_for(S.N, 256), 256, S, c->fbuf);
  cudaEventRecord(c->ev_cls, c->stream);
  cudaStreamWaitEvent(c->nst, c->ev_cls, 0);
  cudaStreamWaitEvent(c->nst, c->ev_join, 0);
  if (nc) launch_on(c, c->nst, "k_run_kick", k_run_kick, 152 * 4, 256, S, c->fbuf);
  enq_fin_on(c, c->nst, M_KICK | M_ADVANCE, 0);
  cudaEventRecord(c->ev_start, c->nst);
  cudaStreamWaitEvent(c->evs, c->ev_start, 0);
  const int nevb = c->ev_grid > 0 ? c->ev_grid : c->n_sm;
  for (int l = 1; l <= n; ++l) {
    const int flags = (l == n ? (F_STREAM | F_COLLIDE | F_SHELL | F_BINROT) : (F_STREAM | F_COLLIDE)) | F_PIPE;
    if (l >= 3) cudaStreamWaitEvent(c->nst, c->ev_finp[l & 1], 0);
    launch_on(c, c->nst, l == n ? "k_stream_near_last" : "k_stream_near", stream_kernel_near(flags), c->n_sm * 5, 256,
              S, l, c->fbuf);
    cudaEventRecord(c->ev_str, c->nst);
    if (l == n) launch_on(c, c->nst, "k_bin_near", k_bin_near, c->n_sm * 4, 256, S, c->fbuf);
    // the event pass with the substep's colloid side work (which needs the finish of l-1,
    // earlier on this stream)
    cudaStreamWaitEvent(c->evs, c->ev_str, 0);
    launch_on(c, c->evs, "k_events_aux", event_aux_kernel(flags), nevb + (S.Nc + 1) / 2, 128, S, l, c->fbuf, nevb,
              l >= 2 ? 1 : 0);
    enq_fin_on(c, c->evs, l < n ? (M_FINISH | M_ADVANCE) : (M_FINISH | M_ACT), l);
    cudaEventRecord(c->ev_finp[l & 1], c->evs);
    if (l == free_after(c)) cudaEventRecord(c->ev_free, c->evs);
  }
  cudaStreamWaitEvent(c->nst, c->ev_finp[n & 1], 0);
  cudaEventRecord(c->ev_end, c->nst);
  // the free pass after the first substep's finish (by default): the chain's first event pass
  // then has the SMs to itself (the free pass holds half of every SM's registers)
  if (free_after(c) >= 1) cudaStreamWaitEvent(c->stream, c->ev_free, 0);
  launch(c, "k_free_flight", k_free_flight, free_blocks(c), 256, S, c->fbuf);
  cudaStreamWaitEvent(c->stream, c->ev_end, 0);
  launch(c, "k_end_step", k_end_step, 1, 256, S);
}

// one MPCD step: rotation_mpcd, run, n_sub substeps (cpp/active_brownian.cpp:25-38)
static void enq_step(mpcd_ctx *c, bool sort) {
  const int n = c->S.n_sub;
  if (c->flight) {
    if (c->S.precision == MPCD_FP32C) enq_step_flight32(c, sort);
    else enq_step_flight64(c, sort);
    return;
  }
  enq_rotation_run(c, sort);
  enq_fin(c, M_KICK | M_ADVANCE, 0);
  if (c->S.precision == MPCD_FP64) {
    enq_substeps_overlapped(c);
  } else {
    for (int l = 1; l <= n; ++l) {
      // the orientation update of substep l-1 rides on the streaming pass of substep l
      enq_stream(c, l == n ? (F_STREAM | F_COLLIDE | F_SHELL | F_BINROT) : (F_STREAM | F_COLLIDE), l, l >= 2);
      enq_fin(c, l < n ? (M_FINISH | M_ADVANCE) : (M_FINISH | M_ACT), l);
    }
  }
  launch(c, "k_end_step", k_end_step, 1, 256, c->S);
}

static int collect_profile(mpcd_ctx *c) {
  if (c->pending.empty()) return MPCD_OK;
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  for (auto &pe : c->pending) {
    float ms = 0;
    cudaEventElapsedTime(&ms, pe.a, pe.b);
    auto &slot = c->prof[pe.name];
    slot.first += 1;
    slot.second += ms;
    c->event_pool.push_back(pe.a);
    c->event_pool.push_back(pe.b);
  }
  c->pending.clear();
  return MPCD_OK;
}

static const char *err_text(int bits) {
  if (bits & ERRB_TTABLE) return "more colloids reach one cell than the fluid-to-colloid table holds";
  if (bits & ERRB_SHELL) return "run() candidate records overflowed";
  if (bits & ERRB_VRANGE) return "a fluid velocity exceeded vmax (range of the exact cell sums)";
  if (bits & ERRB_OCCUPANCY) return "a cell holds more than max_per_cell particles";
  if (bits & ERRB_DISPLACE)
    return "a wall collision displaced a particle, or a colloid moved in a substep, beyond the margin of the cell "
           "tables and the free-flight classification";
  if (bits & ERRB_SHELLSLOTS) return "a particle lies in more rear shells than a record holds";
  if (bits & ERRB_DELTA) return "a colloid momentum exchange left the range of the exact sums";
  if (bits & ERRB_EVENTS) return "the wall-collision event lists overflowed";
  if (bits & ERRB_NBR) return "a colloid has more pair-list partners than the list holds";
  return "device error";
}

// synchronise, read the device step state, turn error bits into a status
static int check_device(mpcd_ctx *c) {
  CUDA_OK(c, cudaMemcpyAsync(c->ss_host, c->S.ss, sizeof(StepState), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  CUDA_OK(c, cudaGetLastError());
  if (c->profile) collect_profile(c);
  int bits = c->ss_host->err;
  if (bits) {
    int code = (bits & (ERRB_VRANGE | ERRB_DELTA)) ? MPCD_ERR_RANGE : MPCD_ERR_CAPACITY;
    char buf[160];
    snprintf(buf, sizeof buf, "device error bits 0x%x: %s", bits, err_text(bits));
    return fail(c, code, buf);
  }
  return MPCD_OK;
}

static int drop_graph(mpcd_ctx *c) {
  for (int s = 0; s < 2; ++s)
    for (int b = 0; b < 2; ++b)
      if (c->step_exec[s][b]) {
        cudaGraphExecDestroy(c->step_exec[s][b]);
        c->step_exec[s][b] = nullptr;
      }
  return MPCD_OK;
}

// ---------------------------------------------------------------- lifetime

extern "C" int mpcd_create(const mpcd_params *pp, mpcd_ctx **out) {
  if (!pp || !out) return MPCD_ERR_PARAM;
  *out = nullptr;
  const mpcd_params &p = *pp;
  if (p.Lx < 7 || p.Ly < 7 || p.Lz < 7) return MPCD_ERR_PARAM;  // the 7x7x7 block must not wrap onto itself
  if (p.n_fluid < 1 || p.n_colloid < 0 || p.n_colloid > 65535 || p.n_sub < 1) return MPCD_ERR_PARAM;
  if (!(p.ndt > 0) || !(p.kbt > 0) || !(p.mass_fl > 0)) return MPCD_ERR_PARAM;
  if (p.n_colloid > 0 && (!(p.mass_colloid > 0) || !(p.I_colloid > 0) || !(p.sigma > 0) || !(p.sig_colloid > 0)))
    return MPCD_ERR_PARAM;
  if (p.precision != MPCD_FP64 && p.precision != MPCD_FP32C) return MPCD_ERR_PARAM;
  if (p.physics != MPCD_PHYSICS_REFERENCE && p.physics != MPCD_PHYSICS_FIXED) return MPCD_ERR_PARAM;
  if (p.precision == MPCD_FP32C && (p.Lx > 1023 || p.Ly > 1023 || p.Lz > 1023)) return MPCD_ERR_PARAM;
  long long C = (long long)p.Lx * p.Ly * p.Lz;
  if (C > (1ll << 30)) return MPCD_ERR_PARAM;

  mpcd_ctx *c = new mpcd_ctx();
  c->p = p;
  SysF64 &S = c->S;
  memset(&S, 0, sizeof S);
  S.N = p.n_fluid;
  S.Nc = p.n_colloid;
  S.Lx = p.Lx; S.Ly = p.Ly; S.Lz = p.Lz;
  S.C = (int)C;
  S.Cpad = S.C + p.Lx * p.Ly + 2 * p.Lx + 4;
  S.n_sub = p.n_sub;
  S.dx = make_dim(p.Lx); S.dy = make_dim(p.Ly); S.dz = make_dim(p.Lz);
  S.Lxf = (float)p.Lx; S.Lyf = (float)p.Ly; S.Lzf = (float)p.Lz;
  S.key = make_uint2((uint32_t)p.seed, (uint32_t)(p.seed >> 32));
  // constants, evaluated with the host libm exactly as the reference writes them
  const double dt = p.ndt / (double)p.n_sub;
  S.dt = dt;
  S.inv_dt = 1.0 / dt;
  S.mass_fl = p.mass_fl; S.mass_colloid = p.mass_colloid; S.I_colloid = p.I_colloid; S.kbt = p.kbt;
  S.sig2q = pow(p.sigma, 2) * 0.25;                       // cpp/fluid_colloid_collision.cpp:35
  S.rsh2 = pow(p.sigma * 0.5 + 0.5, 2);                   // cpp/run.cpp:18
  S.sig_colloid = p.sig_colloid; S.eps = p.eps;
  S.r_cutoff = pow(2, 1.0 / 6.0) * p.sig_colloid;         // cpp/update.cpp:3
  S.fc = 4.0 * p.eps * (12.0 * (pow(p.sig_colloid, 12) / pow(S.r_cutoff, 13)) -
                        6.0 * (pow(p.sig_colloid, 6) / pow(S.r_cutoff, 7)));
  S.ufc = 4.0 * p.eps * (pow(p.sig_colloid / S.r_cutoff, 12) - pow(p.sig_colloid / S.r_cutoff, 6)) + S.fc * S.r_cutoff;
  S.sig12 = pow(p.sig_colloid, 12);
  S.sig6 = pow(p.sig_colloid, 6);
  S.rcf = (float)S.r_cutoff * 1.0001f + 1e-4f;
  const double dt2 = dt * dt;
  S.ddt = 0.5 * dt2 / p.mass_colloid;                      // cpp/update.cpp:48
  S.dtb2 = dt / (p.mass_colloid * 2);                      // cpp/update.cpp:63
  S.v0 = p.v0; S.Dr = p.Dr;
  S.rotdiff_s = sqrt(2.0 * p.Dr * dt);
  const double theta = 2 * asin(1) * (p.theta_deg / 180.0); // cpp/rotation_mpcd.cpp:19
  S.ct = cos(theta); S.st = sin(theta); S.ict = 1 - cos(theta);
  S.two_pi = 4.0 * asin(1.0);
  S.sqrt_kt_m = sqrt(p.kbt / p.mass_fl);
  S.m_beta = p.mass_fl / p.kbt;
  S.inv_m_beta = p.kbt / p.mass_fl;
  S.inv_mc = 1.0 / p.mass_colloid;
  S.inv_ic = 1.0 / p.I_colloid;
  S.cs = 3.0 * p.kbt * dt2 / p.mass_fl;
  // run() gives each particle of a colloid's rear shell M v0 / (m cnt): with a shell of
  // one particle (a colloid whose rear is blocked by another) that is M v0 / m.  The
  // default speed bound of the exact cell sums covers it, and the cell-table reach
  // covers a wall collision's displacement dt/2 (|v| + |v'|) at such speeds.
  const double kick = p.n_colloid > 0 ? fabs(p.v0) * p.mass_colloid / p.mass_fl : 0.0;
  const double vth = sqrt(p.kbt / p.mass_fl);
  const double vmax = p.vmax > 0 ? p.vmax : 24.0 * vth + 2.0 * kick;
  // cell-table reach: sphere (or run() shell) + a wall collision's displacement
  // (0.1 covers speeds near 20 kT units) + a colloid's move in one substep + FP32
  // slack; both displacements are checked on the device.  The colloid bound is
  // dt (20 sigma_V + 20 |v0|), sigma_V = sqrt(3 kT / M) the colloid's thermal speed,
  // within [0.005, 0.05]: the FP64 form's streaming pass tests against the previous
  // substep's colloid positions with it as margin, and every particle within it of
  // a sphere goes to the (latency-bound) event passes, so it is kept tight.
  const double kt_c = fmax(p.kbt, p.kbt1);
  const double vcol = p.n_colloid > 0 ? 20.0 * sqrt(3.0 * kt_c / p.mass_colloid) + 20.0 * fabs(p.v0) : 0.0;
  const double pmargin = fmax(0.1, 0.5 * dt * (2.0 * kick + 6.0 * vth));
  const double cmargin = fmin(0.05, fmax(0.005, dt * vcol));
  S.r_coll = (float)(p.sigma * 0.5);
  S.r_shell = (float)(p.sigma * 0.5 + 0.5);
  S.rT_coll = (float)(p.sigma * 0.5 + pmargin + cmargin + 0.01);
  S.rT_shell = (float)(p.sigma * 0.5 + 0.5 + pmargin + cmargin + 0.01);
  S.disp_margin2 = pmargin * pmargin;
  S.cmargin2 = cmargin * cmargin;
  S.cmarginf = (float)cmargin;
  S.max_per_cell = p.max_per_cell > 0 ? p.max_per_cell : 128;
  c->sort_every = p.sort_every > 0 ? p.sort_every : (p.sort_every < 0 ? 0 : 10);
  S.precision = p.precision;
  // the FP64 form builds the cell tables in the colloid finish: its side kernel
  // needs two warps per colloid (forces; orientation), the FP32 form's four
  S.fin_table = p.precision == MPCD_FP64 ? 1 : 0;
  S.physics = p.physics == MPCD_PHYSICS_FIXED ? 1 : 0;
  S.aux_nw = S.fin_table ? 2 : 4;
  S.dtf = (float)dt;
  S.kick32 = (float)(p.mass_colloid * p.v0 / p.mass_fl);
  S.vmaxf = (float)vmax;
  // free flight: a particle moving further than 5 thermal speeds' worth in a step is near
  S.flight_rv = (float)(5.0 * vth * p.ndt);
  // the free-flight steps' forces from a pair list built at the start of each step
  S.vlist = p.n_colloid > 1 ? 1 : 0;
  // the FP64 form sums displacements w = v dt, the FP32 form velocities
  const double wmax = p.precision == MPCD_FP64 ? vmax * dt : vmax;
  // one scale for the sums of w and |w|^2: max_per_cell * max(wmax, 3 wmax^2) * 2^kw < 2^62
  const double wbound = wmax > 3.0 * wmax * wmax ? wmax : 3.0 * wmax * wmax;
  S.kw = 62 - (int)ceil(log2((double)S.max_per_cell * wbound));
  if (S.kw > 62) S.kw = 62;
  S.inv_sw = ldexp(1.0, -S.kw);
  S.wlim_bits = dbits_h(wmax);

  DevAlloc &m = c->mem;
  const size_t N = S.N, Nc = S.Nc > 0 ? S.Nc : 1;
  for (int b = 0; b < 2; ++b) {
    if (p.precision == MPCD_FP64) {
      for (int k = 0; k < 6; ++k) S.fl[b][k] = m.get<double>(N);
    } else {
      S.q[b] = m.get<uint4>(N);
      for (int k = 0; k < 3; ++k) S.v32[b][k] = m.get<float>(N);
    }
    S.pid[b] = m.get<int>(N);
  }
  S.newpos = m.get<int>(N);
  S.rotcell = m.get<int>(N);
  c->nblk = (int)blocks_for(S.Cpad, 256);
  S.cell_off = m.get<int>(S.Cpad);
  S.cursor = m.get<int>(S.Cpad);
  S.blk_off = m.get<int>(prep_blocks(S) + 1);
  S.acc = m.get<CellAcc>(S.Cpad);
  if (p.precision == MPCD_FP64) S.cell_ab = m.get<double>((size_t)S.C * 12);
  else S.cell_ab32 = m.get<float>((size_t)S.C * 12);
  for (int b = 0; b < 2; ++b) {
    S.X[b] = m.get<double>(3 * Nc);
    S.Xf[b] = m.get<float4>(Nc);
    S.Xcq[b] = m.get<float4>(Nc);
    S.Xco[b] = m.get<float4>(Nc);
    S.cbox[b] = m.get<int>(Nc);
    S.Tcnt[b] = m.get<unsigned long long>(S.C);
    S.Tlist[b] = m.get<uint16_t>((size_t)S.C * TCAP);
  }
  S.V = m.get<double>(3 * Nc); S.W = m.get<double>(3 * Nc); S.ra = m.get<double>(3 * Nc); S.f = m.get<double>(3 * Nc);
  S.fnew = m.get<double>(3 * Nc);
  S.xi = m.get<double>(3 * Nc);
  S.exch = m.get<ExchAcc>(Nc);
  S.xacc = m.get<double>(6 * Nc);
  S.shell_cnt = m.get<int>(Nc);
  S.pot_part = m.get<double>(Nc);
  S.fold = m.get<double>(3 * Nc);
  S.nbr_n = m.get<int>(Nc);
  S.nbr = m.get<uint16_t>(Nc * NBR_CAP);
  S.bkt_start = m.get<int>((size_t)NBK_MAX * NBK_MAX * NBK_MAX + 1);
  S.bkt_cur = m.get<int>((size_t)NBK_MAX * NBK_MAX * NBK_MAX);
  S.bkt_list = m.get<int>(Nc);
  // run() candidates: particles within sigma/2 + 1/2 of a colloid, with room to spare
  const double rsh = p.sigma * 0.5 + 0.5, density = (double)S.N / (double)S.C;
  double est = (double)S.Nc * (4.0 / 3.0 * M_PI * rsh * rsh * rsh * density * 2.0 + 64.0);
  S.shell_cap = (int)(est < (double)S.N ? est : (double)S.N) + 1024;
  S.shell = m.get<ShellRec>(S.shell_cap);
  S.events_cap = S.N / 16 + 65536;
  S.events = m.get<int>(S.events_cap);
  S.near = m.get<int>(N);
  S.fnear = m.get<uint8_t>(N);
  S.ftab = m.get<FlightCell>(S.C);
  if (S.precision == MPCD_FP64) {
    S.newrec[0] = m.get<EventRec>(S.events_cap);
    S.newrec[1] = m.get<EventRec>(S.events_cap);
    S.pend_cap = S.events_cap;
    S.prec = m.get<EventRec>(S.pend_cap);
    S.pend = m.get<uint8_t>(S.N);
  }
  S.ss = m.get<StepState>(1);
  c->insw_n = m.get<double>(S.max_per_cell + 1);
  S.insw_n = c->insw_n;
  c->sqcs_n = m.get<double>(S.max_per_cell + 1);
  S.sqcs_n = c->sqcs_n;
  c->sq3kt_n32 = m.get<float>(S.max_per_cell + 1);
  S.sq3kt_n32 = c->sq3kt_n32;
  c->part = m.get<double>((size_t)c->part_blocks * 8);
  if (m.err != cudaSuccess) {
    std::string e = cudaGetErrorString(m.err);
    m.release();
    delete c;
    return m.err == cudaErrorMemoryAllocation ? MPCD_ERR_NOMEM : MPCD_ERR_CUDA;
  }
  std::vector<double> insw(S.max_per_cell + 1, 0.0), sqcs(S.max_per_cell + 1, 0.0);
  std::vector<float> sq32(S.max_per_cell + 1, 0.f);
  for (int n = 1; n <= S.max_per_cell; ++n) {
    insw[n] = ldexp(1.0 / n, -S.kw);
    sqcs[n] = sqrt(S.cs * (double)(n - 1));
    sq32[n] = (float)sqrt(3.0 * p.kbt * (double)(n - 1) / p.mass_fl);
  }
  scopy(c, c->insw_n, insw.data(), sizeof(double) * insw.size(), cudaMemcpyHostToDevice);
  scopy(c, c->sqcs_n, sqcs.data(), sizeof(double) * sqcs.size(), cudaMemcpyHostToDevice);
  scopy(c, c->sq3kt_n32, sq32.data(), sizeof(float) * sq32.size(), cudaMemcpyHostToDevice);
  if (cudaMallocHost(&c->ss_host, sizeof(StepState)) != cudaSuccess) {
    m.release();
    delete c;
    return MPCD_ERR_NOMEM;
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    m.release();
    cudaFreeHost(c->ss_host);
    delete c;
    return MPCD_ERR_CUDA;
  }
  c->own_stream = true;
  // the side stream has the highest priority: its few blocks are scheduled as soon
  // as streaming blocks retire instead of after the whole streaming pass
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if (cudaStreamCreateWithPriority(&c->aux, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->evs, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->nst, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_cls, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_end, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_list, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_free, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_tab, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_str, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_aux, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_finp[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_finp[1], cudaEventDisableTiming) != cudaSuccess) {
    mpcd_destroy(c);
    return MPCD_ERR_CUDA;
  }
  {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && nsm > 0)
      c->n_sm = nsm;
  }
  cudaDeviceSynchronize();
  *out = c;
  return MPCD_OK;
}

extern "C" int mpcd_destroy(mpcd_ctx *c) {
  if (!c) return MPCD_ERR_PARAM;
  cudaStreamSynchronize(c->stream);
  drop_graph(c);
  for (auto &pe : c->pending) { cudaEventDestroy(pe.a); cudaEventDestroy(pe.b); }
  for (auto e : c->event_pool) cudaEventDestroy(e);
  c->mem.release();
  if (c->staging) cudaFree(c->staging);
  if (c->staging2) cudaFree(c->staging2);
  if (c->ss_host) cudaFreeHost(c->ss_host);
  if (c->diag_host) cudaFreeHost(c->diag_host);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  if (c->aux) cudaStreamDestroy(c->aux);
  if (c->evs) cudaStreamDestroy(c->evs);
  if (c->nst) cudaStreamDestroy(c->nst);
  for (void *q : {(void *)c->ud_Tc, (void *)c->ud_Tl, (void *)c->ud_cnt, (void *)c->ud_acc, (void *)c->box_cell,
                  (void *)c->box_occ, (void *)c->box_nn})
    if (q) cudaFree(q);
  for (cudaEvent_t e : {c->ev_fork, c->ev_join, c->ev_tab, c->ev_cls, c->ev_end, c->ev_list, c->ev_free, c->ev_start, c->ev_str,
                        c->ev_aux, c->ev_finp[0], c->ev_finp[1]})
    if (e) cudaEventDestroy(e);
  delete c;
  return MPCD_OK;
}

extern "C" const char *mpcd_last_error(const mpcd_ctx *c) { return c ? c->err.c_str() : "null context"; }

extern "C" int mpcd_set_stream(mpcd_ctx *c, void *stream) {
  if (!c) return MPCD_ERR_PARAM;
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  if (c->own_stream) cudaStreamDestroy(c->stream);
  drop_graph(c);
  if (stream) {
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
  } else {
    CUDA_OK(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  return MPCD_OK;
}

// ---------------------------------------------------------------- state

// the colloid position buffer holding the present positions: that of the last substep
// of the last completed step, or inside a step begun routine by routine, that of the
// substep the routines have reached
static int cur_buf(const mpcd_ctx *c) {
  long long g = c->ss_host->step * c->S.n_sub - 1;
  if (c->phase == 1 && (c->next_sub > 1 || c->rseq > 0)) {
    const int l = c->rseq > 0 ? c->next_sub : c->next_sub - 1;
    g = c->host_step * c->S.n_sub + (l - 1);
  }
  return (int)(g & 1);
}

static int read_ss(mpcd_ctx *c) {
  CUDA_OK(c, cudaMemcpyAsync(c->ss_host, c->S.ss, sizeof(StepState), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  return MPCD_OK;
}

static int upload_colloid_pos(mpcd_ctx *c, const double *xyz) {
  const SysF64 &S = c->S;
  int b = cur_buf(c);
  std::vector<float4> xf(S.Nc);
  std::vector<int> cb(S.Nc);
  for (int j = 0; j < S.Nc; ++j) {
    xf[j] = make_float4((float)xyz[3 * j], (float)xyz[3 * j + 1], (float)xyz[3 * j + 2], 0.f);
    // int(x) + Lx*int(y) + Lx*Ly*int(z) of cpp/parameters.hpp:59
    cb[j] = (int)xyz[3 * j] + S.Lx * ((int)xyz[3 * j + 1] + S.Ly * (int)xyz[3 * j + 2]);
  }
  CUDA_OK(c, cudaMemcpyAsync(S.X[b], xyz, sizeof(double) * 3 * S.Nc, cudaMemcpyHostToDevice, c->stream));
  CUDA_OK(c, cudaMemcpyAsync(S.Xf[b], xf.data(), sizeof(float4) * S.Nc, cudaMemcpyHostToDevice, c->stream));
  CUDA_OK(c, cudaMemcpyAsync(S.cbox[b], cb.data(), sizeof(int) * S.Nc, cudaMemcpyHostToDevice, c->stream));
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  return MPCD_OK;
}

static int ensure_staging(mpcd_ctx *c, bool two = false) {
  if (!c->staging) {
    cudaError_t e = cudaMalloc(&c->staging, sizeof(double) * 3 * (size_t)c->S.N);
    if (e != cudaSuccess) return fail(c, MPCD_ERR_NOMEM, "staging buffer");
  }
  if (two && !c->staging2) {
    cudaError_t e = cudaMalloc(&c->staging2, sizeof(double) * 3 * (size_t)c->S.N);
    if (e != cudaSuccess) return fail(c, MPCD_ERR_NOMEM, "staging buffer");
  }
  return MPCD_OK;
}

// host AoS xyz -> device SoA: one copy of the caller's buffer (a DMA when it is
// pinned), then a transpose on the device
static int upload_soa(mpcd_ctx *c, const double *aos, double *dx, double *dy, double *dz, int *id, int *newpos,
                      double scale) {
  int r;
  if ((r = ensure_staging(c))) return r;
  const int N = c->S.N;
  CUDA_OK(c, cudaMemcpyAsync(c->staging, aos, sizeof(double) * 3 * (size_t)N, cudaMemcpyHostToDevice, c->stream));
  launch(c, "k_aos_to_soa", k_aos_to_soa, blocks_for(N, 256), 256, (const double *)c->staging, dx, dy, dz, id, newpos,
         N, scale);
  return MPCD_OK;
}

static int download_soa(mpcd_ctx *c, double *aos, const double *dx, const double *dy, const double *dz, const int *id,
                        double div) {
  int r;
  if ((r = ensure_staging(c))) return r;
  const int N = c->S.N;
  launch(c, "k_soa_to_aos", k_soa_to_aos, blocks_for(N, 256), 256, c->staging, dx, dy, dz, id, N, div);
  CUDA_OK(c, cudaMemcpyAsync(aos, c->staging, sizeof(double) * 3 * (size_t)N, cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  return MPCD_OK;
}

// the fluid buffer holding the current state
static Fluid cur_fluid(const mpcd_ctx *c) { return fluid_at(c->S, c->fbuf); }

static int invalidate_tables(mpcd_ctx *c) {
  const SysF64 &S = c->S;
  for (int b = 0; b < 2; ++b) CUDA_OK(c, cudaMemsetAsync(S.Tcnt[b], 0, sizeof(unsigned long long) * S.C, c->stream));
  CUDA_OK(c, cudaMemsetAsync(S.acc, 0, sizeof(CellAcc) * S.Cpad, c->stream));
  if (S.Nc) CUDA_OK(c, cudaMemsetAsync(S.exch, 0, sizeof(ExchAcc) * S.Nc, c->stream));
  if (S.ftab) CUDA_OK(c, cudaMemsetAsync(S.ftab, 0, sizeof(FlightCell) * S.C, c->stream));
  c->setup_done = false;
  c->phase = 0;
  c->next_sub = 1;
  c->rseq = 0;
  c->box_valid = false;
  return MPCD_OK;
}

extern "C" int mpcd_set_state(mpcd_ctx *c, const double *pos_fl, const double *vel_fl, const double *pos_colloid,
                              const double *vel_colloid, const double *ang_vel_colloid, const double *ra) {
  if (!c) return MPCD_ERR_PARAM;
  int r;
  if ((r = read_ss(c))) return r;
  const SysF64 &S = c->S;
  if ((pos_fl == nullptr) != (vel_fl == nullptr))
    return fail(c, MPCD_ERR_PARAM, "pos_fl and vel_fl are set together (the device keeps particles in cell order)");
  c->phase = 0;
  if (pos_fl && S.precision == MPCD_FP32C) {
    if ((r = ensure_staging(c, true))) return r;
    const size_t nb = sizeof(double) * 3 * (size_t)S.N;
    CUDA_OK(c, cudaMemcpyAsync(c->staging, pos_fl, nb, cudaMemcpyHostToDevice, c->stream));
    CUDA_OK(c, cudaMemcpyAsync(c->staging2, vel_fl, nb, cudaMemcpyHostToDevice, c->stream));
    launch(c, "k_aos_to_q", k_aos_to_q, blocks_for(S.N, 256), 256, S, (const double *)c->staging,
           (const double *)c->staging2, c->fbuf);
  } else if (pos_fl) {
    Fluid F = cur_fluid(c);
    if ((r = upload_soa(c, pos_fl, F.x, F.y, F.z, F.id, S.newpos, 0.0))) return r;
    if ((r = upload_soa(c, vel_fl, F.wx, F.wy, F.wz, nullptr, nullptr, S.dt))) return r;  // w = fl(v*dt)
  }
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  if (S.Nc) {
    if (pos_colloid && (r = upload_colloid_pos(c, pos_colloid))) return r;
    if (vel_colloid) CUDA_OK(c, scopy(c, S.V, vel_colloid, sizeof(double) * 3 * S.Nc, cudaMemcpyHostToDevice));
    if (ang_vel_colloid) CUDA_OK(c, scopy(c, S.W, ang_vel_colloid, sizeof(double) * 3 * S.Nc, cudaMemcpyHostToDevice));
    if (ra) CUDA_OK(c, scopy(c, S.ra, ra, sizeof(double) * 3 * S.Nc, cudaMemcpyHostToDevice));
  }
  return invalidate_tables(c);
}

extern "C" int mpcd_get_state(mpcd_ctx *c, double *pos_fl, double *vel_fl, double *pos_colloid, double *vel_colloid,
                              double *ang_vel_colloid, double *ra, double *f) {
  if (!c) return MPCD_ERR_PARAM;
  int r;
  if ((r = read_ss(c))) return r;
  const SysF64 &S = c->S;
  if (S.precision == MPCD_FP32C && (pos_fl || vel_fl)) {
    if ((r = ensure_staging(c, true))) return r;
    const size_t nb = sizeof(double) * 3 * (size_t)S.N;
    launch(c, "k_q_to_aos", k_q_to_aos, blocks_for(S.N, 256), 256, S, c->staging, c->staging2, c->fbuf);
    if (pos_fl) CUDA_OK(c, cudaMemcpyAsync(pos_fl, c->staging, nb, cudaMemcpyDeviceToHost, c->stream));
    if (vel_fl) CUDA_OK(c, cudaMemcpyAsync(vel_fl, c->staging2, nb, cudaMemcpyDeviceToHost, c->stream));
    CUDA_OK(c, cudaStreamSynchronize(c->stream));
  } else {
    Fluid F = cur_fluid(c);
    if (pos_fl && (r = download_soa(c, pos_fl, F.x, F.y, F.z, F.id, 0.0))) return r;
    if (vel_fl && (r = download_soa(c, vel_fl, F.wx, F.wy, F.wz, F.id, S.dt))) return r;  // v = w/dt
  }
  if (S.Nc) {
    int b = cur_buf(c);
    if (pos_colloid) CUDA_OK(c, scopy(c, pos_colloid, S.X[b], sizeof(double) * 3 * S.Nc, cudaMemcpyDeviceToHost));
    if (vel_colloid) CUDA_OK(c, scopy(c, vel_colloid, S.V, sizeof(double) * 3 * S.Nc, cudaMemcpyDeviceToHost));
    if (ang_vel_colloid) CUDA_OK(c, scopy(c, ang_vel_colloid, S.W, sizeof(double) * 3 * S.Nc, cudaMemcpyDeviceToHost));
    if (ra) CUDA_OK(c, scopy(c, ra, S.ra, sizeof(double) * 3 * S.Nc, cudaMemcpyDeviceToHost));
    if (f) CUDA_OK(c, scopy(c, f, S.f, sizeof(double) * 3 * S.Nc, cudaMemcpyDeviceToHost));
  }
  return MPCD_OK;
}

extern "C" int mpcd_set_step(mpcd_ctx *c, int64_t step) {
  if (!c || step < 0) return MPCD_ERR_PARAM;
  int r;
  if ((r = read_ss(c))) return r;
  if (c->S.Nc && c->ss_host->step != step) {
    // the colloid positions live in the buffer of the last finished substep; move them
    int from = cur_buf(c);
    int to = (int)((step * c->S.n_sub - 1) & 1);
    if (from != to) {
      const SysF64 &S = c->S;
      CUDA_OK(c, scopy(c, S.X[to], S.X[from], sizeof(double) * 3 * S.Nc, cudaMemcpyDeviceToDevice));
      CUDA_OK(c, scopy(c, S.Xf[to], S.Xf[from], sizeof(float4) * S.Nc, cudaMemcpyDeviceToDevice));
      CUDA_OK(c, scopy(c, S.cbox[to], S.cbox[from], sizeof(int) * S.Nc, cudaMemcpyDeviceToDevice));
    }
  }
  c->ss_host->step = step;
  CUDA_OK(c, scopy(c, &c->S.ss->step, &step, sizeof(long long), cudaMemcpyHostToDevice));
  return invalidate_tables(c);
}

extern "C" int mpcd_set_launch(mpcd_ctx *c, int which, int grid, int block) {
  if (!c) return MPCD_ERR_PARAM;
  if (which == MPCD_LAUNCH_AUX) {
    if (grid > 0 && block != 64 && block != 128 && block != 256)
      return fail(c, MPCD_ERR_PARAM, "colloid side work: 64, 128 or 256 threads per colloid");
    c->S.aux_nw = grid > 0 ? block / 32 : (c->S.fin_table ? 2 : 4);
    return drop_graph(c);
  }
  if (which == MPCD_LAUNCH_FREE) {
    if (grid > 65535) return fail(c, MPCD_ERR_PARAM, "free-flight pass: grid <= 65535");
    if (grid > 0 && (block < 0 || block > c->S.n_sub - 1))
      return fail(c, MPCD_ERR_PARAM, "free-flight pass: block = the substep it follows, 0..n_sub-1");
    c->free_grid = grid > 0 ? grid : 0;
    c->free_after = grid > 0 ? block : -1;
    return drop_graph(c);
  }
  if (grid > 65535 || (grid > 0 && (block < 32 || block > 128 || block % 32)))
    return fail(c, MPCD_ERR_PARAM, "launch shape: block a multiple of 32 in [32, 128], grid <= 65535");
  if (which == MPCD_LAUNCH_EVENTS) {
    c->ev_grid = grid > 0 ? grid : 0;
    c->ev_block = grid > 0 ? block : 128;
  } else if (which == MPCD_LAUNCH_FIN) {
    c->fin_grid = grid > 0 ? grid : 0;
    c->fin_block = grid > 0 ? block : 32;
  } else {
    return fail(c, MPCD_ERR_PARAM, "unknown launch");
  }
  return drop_graph(c);
}

extern "C" int mpcd_set_flight(mpcd_ctx *c, int on) {
  if (!c) return MPCD_ERR_PARAM;
  c->flight = on != 0;
  return drop_graph(c);
}

extern "C" int mpcd_get_flight(mpcd_ctx *c, int32_t *near) {
  if (!c || !near) return MPCD_ERR_PARAM;
  int r;
  if ((r = read_ss(c))) return r;
  *near = c->ss_host->nnear;
  return MPCD_OK;
}

extern "C" int64_t mpcd_get_step(const mpcd_ctx *c) {
  if (!c) return -1;
  long long s = 0;
  cudaStreamSynchronize(c->stream);
  scopy(c, &s, &c->S.ss->step, sizeof s, cudaMemcpyDeviceToHost);
  return s;
}

// ---------------------------------------------------------------- routines

extern "C" int mpcd_setup(mpcd_ctx *c) {
  if (!c) return MPCD_ERR_PARAM;
  int r;
  if ((r = read_ss(c))) return r;
  if ((r = invalidate_tables(c))) return r;
  const int zero = 0;
  CUDA_OK(c, cudaMemcpyAsync(&c->S.ss->err, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  // create_box + neighbour_list_md + compute_force_md: forces at the current positions,
  // cell table around each colloid (cpp/active_brownian.cpp:17-20)
  // no particle is pending between steps (a step cut short by an error may have left marks)
  if (c->S.pend) CUDA_OK(c, cudaMemsetAsync(c->S.pend, 0, (size_t)c->S.N, c->stream));
  if (c->S.Nc) CUDA_OK(c, cudaMemsetAsync(c->S.shell_cnt, 0, sizeof(int) * (size_t)c->S.Nc, c->stream));
  launch(c, "k_colloid_setup", k_colloid_setup, colloid_grid(c), 128, c->S);
  // neighbour_list_mpcd seen from the fluid: run() candidates of the first step, and the
  // SRD binning of its rotation_mpcd
  c->host_step = c->ss_host->step;
  enq_stream(c, F_SHELL | F_BINROT, 0, 0);
  if ((r = check_device(c))) return r;
  c->setup_done = true;
  c->phase = 0;
  c->next_sub = 1;
  return MPCD_OK;
}

static int need_setup(mpcd_ctx *c) {
  if (!c) return MPCD_ERR_PARAM;
  if (!c->setup_done) return fail(c, MPCD_ERR_STATE, "mpcd_setup must follow set_state/initialize");
  return MPCD_OK;
}

extern "C" int mpcd_rotation_mpcd(mpcd_ctx *c) {
  int r;
  if ((r = need_setup(c))) return r;
  if (c->phase != 0) return fail(c, MPCD_ERR_STATE, "rotation_mpcd starts a step: finish the substeps of this one");
  enq_rotation(c, sorts_at(c, c->host_step));
  c->phase = 1;
  c->next_sub = 0;
  return check_device(c);
}

extern "C" int mpcd_run(mpcd_ctx *c) {
  int r;
  if ((r = need_setup(c))) return r;
  if (c->phase != 1 || c->next_sub != 0) return fail(c, MPCD_ERR_STATE, "run follows rotation_mpcd of the same step");
  enq_run_fluid(c);
  enq_fin(c, M_KICK, 0);
  c->next_sub = 1;
  return check_device(c);
}

extern "C" int mpcd_substep(mpcd_ctx *c, int l) {
  int r;
  if ((r = need_setup(c))) return r;
  const int n = c->S.n_sub;
  if (l < 1 || l > n) return fail(c, MPCD_ERR_PARAM, "substep out of range");
  if (c->phase != 1 || c->next_sub != l)
    return fail(c, MPCD_ERR_STATE, "substeps follow rotation_mpcd and run, in order 1..n_sub");
  if (c->rseq != 0)
    return fail(c, MPCD_ERR_STATE, "a substep begun routine by routine is unfinished (update_velocity_colloid closes it)");
  enq_fin(c, M_ADVANCE, l - 1);   // update_pos_md, neighbour_list_md
  // update_pos_mpcd, neighbour_list_mpcd, fluid_colloid_collision (fluid side), and
  // compute_force_md at the new colloid positions
  enq_stream(c, l == n ? (F_STREAM | F_COLLIDE | F_SHELL | F_BINROT) : (F_STREAM | F_COLLIDE), l, 0);
  // end of fluid_colloid_collision, update_activity_direction, update_velocity_colloid
  enq_fin(c, M_FINISH | M_ACT, l);
  c->next_sub = l + 1;
  if (l == n) {
    launch(c, "k_end_step", k_end_step, 1, 256, c->S);
    c->phase = 0;
    c->host_step += 1;
  }
  return check_device(c);
}

// nsteps steps enqueued on the context's stream (graph replays), nothing waited for
static int enq_steps(mpcd_ctx *c, int nsteps) {
  int r;
  if ((r = need_setup(c))) return r;
  if (nsteps < 0) return MPCD_ERR_PARAM;
  if (c->phase != 0) return fail(c, MPCD_ERR_STATE, "a step begun routine by routine is unfinished");
  if (c->profile) {
    for (int s = 0; s < nsteps; ++s) {
      enq_step(c, sorts_at(c, c->host_step));
      c->host_step += 1;
    }
    return MPCD_OK;
  }
  for (int s = 0; s < nsteps; ++s) {
    // one graph per (sorts this step, fluid buffer): the kernels' buffer arguments
    // are fixed at capture
    const int sort = sorts_at(c, c->host_step) ? 1 : 0, b = c->fbuf;
    if (!c->step_exec[sort][b]) {
      cudaGraph_t g;
      int64_t before = c->launches;
      CUDA_OK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      enq_step(c, sort != 0);
      CUDA_OK(c, cudaStreamEndCapture(c->stream, &g));
      c->fbuf = b;  // capture only recorded the launches
      c->step_launches[sort][b] = (int)(c->launches - before);
      c->launches = before;
      cudaError_t e = cudaGraphInstantiate(&c->step_exec[sort][b], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return fail(c, MPCD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    CUDA_OK(c, cudaGraphLaunch(c->step_exec[sort][b], c->stream));
    c->launches += c->step_launches[sort][b];
    if (sort) c->fbuf = 1 - b;
    c->host_step += 1;
  }
  return MPCD_OK;
}

extern "C" int mpcd_step(mpcd_ctx *c, int nsteps) {
  int r;
  if ((r = enq_steps(c, nsteps))) return r;
  return check_device(c);
}

extern "C" int mpcd_step_async(mpcd_ctx *c, int nsteps) { return enq_steps(c, nsteps); }

extern "C" int mpcd_sync(mpcd_ctx *c) {
  if (!c) return MPCD_ERR_PARAM;
  return check_device(c);
}

// ---------------------------------------------------------------- diagnostics

extern "C" int mpcd_diag(mpcd_ctx *c, mpcd_diag_t *out) {
  int r;
  if (!out) return MPCD_ERR_PARAM;
  if ((r = need_setup(c))) return r;
  const SysF64 &S = c->S;
  const size_t np = (size_t)c->part_blocks * 5, nc = (size_t)S.Nc;
  if (!c->diag_host && cudaMallocHost(&c->diag_host, sizeof(double) * (np + 7 * nc + 1)) != cudaSuccess) {
    c->diag_host = nullptr;
    return fail(c, MPCD_ERR_NOMEM, "page-locked diagnostics buffer");
  }
  launch(c, "k_diag_fluid", k_diag_fluid, c->part_blocks, 256, S, c->part);
  if (S.Nc) launch(c, "k_colloid_pot", k_colloid_pot, colloid_grid(c), 128, S, cur_buf(c));
  // everything the diagnostics read in one round trip: the step state (error bits, event
  // count), the fluid partial sums and the colloid arrays into page-locked memory, then the
  // event count reset, then one synchronisation
  double *h = c->diag_host;
  CUDA_OK(c, cudaMemcpyAsync(c->ss_host, S.ss, sizeof(StepState), cudaMemcpyDeviceToHost, c->stream));
  CUDA_OK(c, cudaMemcpyAsync(h, c->part, sizeof(double) * np, cudaMemcpyDeviceToHost, c->stream));
  if (nc) {
    CUDA_OK(c, cudaMemcpyAsync(h + np, S.V, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    CUDA_OK(c, cudaMemcpyAsync(h + np + 3 * nc, S.W, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    CUDA_OK(c, cudaMemcpyAsync(h + np + 6 * nc, S.pot_part, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_OK(c, cudaMemsetAsync(&S.ss->ev_total, 0, sizeof(long long), c->stream));
  CUDA_OK(c, cudaStreamSynchronize(c->stream));
  CUDA_OK(c, cudaGetLastError());
  if (c->profile) collect_profile(c);
  if (int bits = c->ss_host->err) {
    char buf[200];
    snprintf(buf, sizeof buf, "device error bits 0x%x: %s", bits, err_text(bits));
    return fail(c, (bits & (ERRB_VRANGE | ERRB_DELTA)) ? MPCD_ERR_RANGE : MPCD_ERR_CAPACITY, buf);
  }
  const double *part = h;
  double sw[3] = {0, 0, 0}, s2 = 0, n = 0;
  for (int b = 0; b < c->part_blocks; ++b) {
    for (int k = 0; k < 3; ++k) sw[k] += part[5 * b + k];
    s2 += part[5 * b + 3];
    n += part[5 * b + 4];
  }
  memset(out, 0, sizeof *out);
  out->step = c->ss_host->step;
  const double m = c->p.mass_fl;
  const double per = S.precision == MPCD_FP64 ? S.dt : 1.0;  // the FP64 form sums w = v dt
  for (int k = 0; k < 3; ++k) out->momentum_fluid[k] = m * sw[k] / per;
  out->ke_fluid = 0.5 * m * s2 / (per * per);
  out->temperature_fluid = n > 0 ? 2.0 * out->ke_fluid / (3.0 * n) / c->p.kbt : 0;
  // wall-collision candidates handled exactly, summed since the last call
  out->events = c->ss_host->ev_total;
  out->shell_records = c->ss_host->nshell;
  double mom[3] = {out->momentum_fluid[0], out->momentum_fluid[1], out->momentum_fluid[2]};
  if (S.Nc) {
    const double *V = h + np, *W = h + np + 3 * nc, *pot = h + np + 6 * nc;
    double ke = 0, ake = 0, pe = 0;
    for (int j = 0; j < S.Nc; ++j) {
      ke += V[3 * j] * V[3 * j] + V[3 * j + 1] * V[3 * j + 1] + V[3 * j + 2] * V[3 * j + 2];
      ake += W[3 * j] * W[3 * j] + W[3 * j + 1] * W[3 * j + 1] + W[3 * j + 2] * W[3 * j + 2];
      for (int k = 0; k < 3; ++k) mom[k] += V[3 * j + k] * c->p.mass_colloid;
      pe += pot[j];
    }
    out->ke_colloid = 0.5 * c->p.mass_colloid * ke;
    out->ang_ke_colloid = 0.5 * c->p.I_colloid * ake;
    out->potential_colloid = pe;
    out->energy_colloid = pe + out->ke_colloid + out->ang_ke_colloid;
  }
  for (int k = 0; k < 3; ++k) out->momentum[k] = mom[k];
  return MPCD_OK;
}

// ---------------------------------------------------------------- observables

extern "C" int mpcd_get_rotation_binning(mpcd_ctx *c, int32_t *cell_of, int32_t *occupancy, double *shift) {
  int r;
  if ((r = need_setup(c))) return r;
  const SysF64 &S = c->S;
  if ((r = read_ss(c))) return r;
  if (c->phase != 0) return fail(c, MPCD_ERR_STATE, "the binning is that of the next step; call between steps");
  std::vector<int> rc(S.N), id(S.N);
  CUDA_OK(c, scopy(c, rc.data(), S.rotcell, sizeof(int) * S.N, cudaMemcpyDeviceToHost));
  CUDA_OK(c, scopy(c, id.data(), cur_fluid(c).id, sizeof(int) * S.N, cudaMemcpyDeviceToHost));
  if (cell_of)
    for (int i = 0; i < S.N; ++i) cell_of[id[i]] = rc[i] + 1;
  if (occupancy) {
    for (int b = 0; b < S.C; ++b) occupancy[b] = 0;
    for (int i = 0; i < S.N; ++i)
      if (rc[i] < S.C) occupancy[rc[i]]++;
  }
  if (shift)
    for (int k = 0; k < 3; ++k) shift[k] = c->ss_host->rr[k];
  return MPCD_OK;
}

extern "C" int mpcd_get_shell_count(mpcd_ctx *c, int32_t *cnt) {
  if (!c || !cnt) return MPCD_ERR_PARAM;
  if (c->S.Nc) CUDA_OK(c, scopy(c, cnt, c->S.shell_cnt, sizeof(int) * c->S.Nc, cudaMemcpyDeviceToHost));
  return MPCD_OK;
}

// ---------------------------------------------------------------- profiling

extern "C" int mpcd_profile_enable(mpcd_ctx *c, int on) {
  if (!c) return MPCD_ERR_PARAM;
  if (!on) collect_profile(c);
  c->profile = on != 0;
  if (on) c->prof.clear();
  return MPCD_OK;
}

extern "C" int mpcd_profile_read(mpcd_ctx *c, char names[][48], int64_t *launches, double *total_ms, int cap) {
  if (!c) return MPCD_ERR_PARAM;
  collect_profile(c);
  int i = 0;
  for (auto &kv : c->prof) {
    if (i < cap) {
      snprintf(names[i], 48, "%s", kv.first.c_str());
      launches[i] = kv.second.first;
      total_ms[i] = kv.second.second;
    }
    ++i;
  }
  return i;
}

extern "C" int64_t mpcd_launch_count(const mpcd_ctx *c) { return c ? c->launches : -1; }

// One step as a graph with a timing event before and after every launch (event-record
// nodes), replayed once: each launch's start and end in ms from the step's start.
extern "C" int mpcd_trace_step(mpcd_ctx *c, char names[][48], double *t0_ms, double *t1_ms, int cap) {
  int r;
  if ((r = need_setup(c))) return r;
  if (c->phase != 0) return fail(c, MPCD_ERR_STATE, "a step begun routine by routine is unfinished");
  if (c->profile) return fail(c, MPCD_ERR_STATE, "profiling is on");
  const int sort = sorts_at(c, c->host_step) ? 1 : 0, b = c->fbuf;
  cudaEvent_t start = pool_event(c);
  cudaGraph_t g;
  cudaGraphExec_t x = nullptr;
  c->trace.clear();
  CUDA_OK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  cudaEventRecordWithFlags(start, c->stream, cudaEventRecordExternal);
  c->tracing = true;
  const int64_t before = c->launches;
  enq_step(c, sort != 0);
  c->tracing = false;
  c->launches = before;
  c->fbuf = b;
  CUDA_OK(c, cudaStreamEndCapture(c->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(c, MPCD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  e = cudaGraphLaunch(x, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaGraphExecDestroy(x);
  if (e != cudaSuccess) return fail(c, MPCD_ERR_CUDA, std::string("traced step: ") + cudaGetErrorString(e));
  c->launches += (int64_t)c->trace.size();
  if (sort) c->fbuf = 1 - b;
  c->host_step += 1;
  int i = 0;
  for (auto &pe : c->trace) {
    if (i < cap) {
      float a = 0, z = 0;
      cudaEventElapsedTime(&a, start, pe.a);
      cudaEventElapsedTime(&z, start, pe.b);
      snprintf(names[i], 48, "%s", pe.name);
      t0_ms[i] = a;
      t1_ms[i] = z;
    }
    c->event_pool.push_back(pe.a);
    c->event_pool.push_back(pe.b);
    ++i;
  }
  c->event_pool.push_back(start);
  c->trace.clear();
  if ((r = check_device(c))) return r;
  return i;
}

// initialisation lives in init.cu; it needs the context internals
#include "init_host.inc"

// the substep body routine by routine
#include "routines_host.inc"

extern "C" int mpcd_exchange_read(mpcd_ctx *c, double *out, int reset) {
  if (!c) return MPCD_ERR_PARAM;
  int r;
  if ((r = read_ss(c))) return r;
  if (!c->S.Nc) return MPCD_OK;
  const size_t nb = sizeof(double) * 6 * (size_t)c->S.Nc;
  if (out) CUDA_OK(c, scopy(c, out, c->S.xacc, nb, cudaMemcpyDeviceToHost));
  if (reset) {
    CUDA_OK(c, cudaMemsetAsync(c->S.xacc, 0, nb, c->stream));
    CUDA_OK(c, cudaStreamSynchronize(c->stream));
  }
  return MPCD_OK;
}

// updown_velocity (cpp/run.cpp:28-50) on the current state: per colloid the
// number of fluid particles in its run() shell and in its inner shell (rear side,
// r.V <= 0) and the sums of their velocities
extern "C" int mpcd_updown_velocity(mpcd_ctx *c, int32_t *cnt, int32_t *up_cnt, double *vel_sum,
                                    double *up_vel_sum) {
  int r;
  if ((r = need_setup(c))) return r;
  const SysF64 &S = c->S;
  if (!S.Nc) return MPCD_OK;
  if (!c->ud_Tc) {
    if (cudaMalloc(&c->ud_Tc, sizeof(unsigned long long) * (size_t)S.C) != cudaSuccess ||
        cudaMalloc(&c->ud_Tl, sizeof(uint16_t) * (size_t)S.C * TCAP) != cudaSuccess ||
        cudaMalloc(&c->ud_cnt, sizeof(int) * 2 * (size_t)S.Nc) != cudaSuccess ||
        cudaMalloc(&c->ud_acc, sizeof(ExchAcc) * (size_t)S.Nc) != cudaSuccess)
      return fail(c, MPCD_ERR_NOMEM, "updown_velocity scratch");
    CUDA_OK(c, cudaMemsetAsync(c->ud_Tc, 0, sizeof(unsigned long long) * (size_t)S.C, c->stream));
  }
  CUDA_OK(c, cudaMemsetAsync(c->ud_cnt, 0, sizeof(int) * 2 * (size_t)S.Nc, c->stream));
  CUDA_OK(c, cudaMemsetAsync(c->ud_acc, 0, sizeof(ExchAcc) * (size_t)S.Nc, c->stream));
  const long long e = ++c->ud_epoch;  // a stale entry of an earlier call reads as empty
  const double sh_up = c->p.sigma * 0.5 + 0.1;
  const double rup2 = pow(sh_up, 2);  // cpp/run.cpp:39
  launch(c, "k_updown_table", k_updown_table, colloid_grid(c), 128, S, c->ud_Tc, c->ud_Tl, e,
         (float)(c->p.sigma * 0.5 + 0.5 + 0.01));
  launch(c, "k_updown", k_updown, c->n_sm * 8, 256, S, c->fbuf, (const unsigned long long *)c->ud_Tc,
         (const uint16_t *)c->ud_Tl, e, rup2, c->ud_cnt, c->ud_acc);
  if ((r = check_device(c))) return r;
  std::vector<int> hc(2 * (size_t)S.Nc);
  std::vector<ExchAcc> ha(S.Nc);
  CUDA_OK(c, scopy(c, hc.data(), c->ud_cnt, sizeof(int) * hc.size(), cudaMemcpyDeviceToHost));
  CUDA_OK(c, scopy(c, ha.data(), c->ud_acc, sizeof(ExchAcc) * ha.size(), cudaMemcpyDeviceToHost));
  for (int j = 0; j < S.Nc; ++j) {
    if (cnt) cnt[j] = hc[2 * j];
    if (up_cnt) up_cnt[j] = hc[2 * j + 1];
    for (int k = 0; k < 3; ++k) {
      const double a = (double)ha[j].hi[k] * 0x1p-20 + (double)ha[j].lo[k] * 0x1p-72;
      const double u = (double)ha[j].hi[3 + k] * 0x1p-20 + (double)ha[j].lo[3 + k] * 0x1p-72;
      if (vel_sum) vel_sum[3 * j + k] = a;
      if (up_vel_sum) up_vel_sum[3 * j + k] = u;
    }
  }
  return MPCD_OK;
}

// a trajectory frame of this context's colloids (between steps)
extern "C" int mpcd_traj_record(mpcd_traj *t, mpcd_ctx *c) {
  int r;
  if ((r = need_setup(c))) return r;
  if (!t || traj_colloids(t) != c->S.Nc || c->S.Nc < 1) return fail(c, MPCD_ERR_PARAM, "trajectory size");
  if (c->phase != 0) return fail(c, MPCD_ERR_STATE, "frames are taken between steps");
  const int b = (int)((c->host_step * c->S.n_sub - 1) & 1);
  r = traj_record_f64(t, c->S.X[b], c->S.V, c->S.ra, c->stream);
  return r ? fail(c, r, mpcd_traj_last_error(t)) : MPCD_OK;
}

#include "ensemble.inc"

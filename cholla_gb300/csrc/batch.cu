// batch.cu -- the batch handle API: many independent 3D boxes of one scheme, each with its own
// state, scratch, time step and time, advanced together (kernels in hydro_fast.cu).  The jobs
// are cut into chunks of BATCH_CHUNK; each chunk is one chain of launches whose kernels carry
// the chunk in their parameters, one block per tile of all its jobs; large jobs run the
// single-box step in a chain of their own.  The chains run side by side (forked streams); a
// job set that holds for two steps is captured into a CUDA graph and replayed (jobs join and
// leave between steps).
//
// No counterpart in the reference: it holds one box shape per process (its scratch and launch
// parameters are file-scope globals, src/global/global_cuda.cu:1-16, VL_3D_cuda.cu:141).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cholla_gb300.h"
#include "common.cuh"
#include "ghost.cuh"
#include "kernels.h"

struct cgb_batch {
  cgb_scheme scheme;
  double c_cfl = 0.3;
  cudaStream_t stream = nullptr;
  std::vector<cgb::BatchJob> jobs;  // index = position in the batch
  struct Slot {
    int id;
    void *mem;          // one stream-ordered allocation: W, GEp, Epre, dti, status, dt_t
    bool held = false;  // left out of the steps until released
    int flags[6];       // boundary flags as given
  };
  std::vector<Slot> slots;  // parallel to jobs
  int next_id = 1;
  bool dirty  = true;                   // the job set changed since the graph was captured
  int chains  = 1;                      // at least this many chains of launches
  int tiles   = 0;                      // sweep tile set of the shared-kernel chains (0 / 1)
  long long solo_cells = 2LL << 20;     // jobs of at least this many padded cells run solo
  cudaGraphExec_t graph = nullptr;
  std::vector<cudaStream_t> aux;        // capture streams of chunks 1, 2, ...
  std::vector<cudaEvent_t> ev;          // fork (0) and joins of the capture
  cudaMemPool_t pool = nullptr;         // job scratch; keeps freed memory for the next job
  struct Plan {
    std::vector<cgb::BatchChunk> chunks;  // shared-kernel chains
    std::vector<size_t> solo;             // jobs run by the single-box step, one chain each
  } plan;
  int stable      = 0;                  // steps since the job set last changed
  long long steps = 0;
  std::mutex mu;
};

namespace
{
thread_local std::string g_batch_err;

int bfail(int code, const std::string &m)
{
  g_batch_err = m;
  return code;
}
int bcuda(cudaError_t e, const char *where) { return bfail(CGB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e)); }

size_t al256(size_t v) { return (v + 255) & ~size_t(255); }

// work of a job for balancing the chains: padded cells (every kernel's tiles scale with them)
double job_work(const cgb::BatchJob &J) { return (double)J.b.n; }

// The batch's jobs as chunks of at most BATCH_CHUNK jobs with per-kind tile offsets, at least
// `chains` of them (each chunk is a chain of launches; the chains run side by side), filled
// largest job first into the chunk with the least work so far.
std::vector<cgb::BatchChunk> build_chunks(const std::vector<cgb::BatchJob> &jobs, int chains, int set)
{
  size_t const nj = jobs.size();
  size_t nc       = (nj + cgb::BATCH_CHUNK - 1) / cgb::BATCH_CHUNK;
  nc              = std::max(nc, std::min(nj, (size_t)std::max(chains, 1)));
  std::vector<size_t> order(nj);
  for (size_t i = 0; i < nj; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t a, size_t b) { return job_work(jobs[a]) > job_work(jobs[b]); });
  std::vector<cgb::BatchChunk> out(nc);
  std::vector<double> load(nc, 0.0);
  for (auto &C : out) std::memset(&C, 0, sizeof(C));
  for (size_t i : order) {
    size_t best = nc;
    for (size_t c = 0; c < nc; c++)
      if (out[c].njobs < cgb::BATCH_CHUNK && (best == nc || load[c] < load[best])) best = c;
    cgb::BatchChunk &C = out[best];
    C.jobs[C.njobs++]  = jobs[i];
    load[best] += job_work(jobs[i]);
  }
  for (auto &C : out) {
    for (int j = 0; j < C.njobs; j++) {
      int tiles[cgb::BK_NUM];
      cgb::batch_tiles(C.jobs[j].b, tiles, set);
      for (int k = 0; k < cgb::BK_NUM; k++) {
        C.off[k][j] = C.total[k];
        C.total[k] += tiles[k];
      }
    }
    for (int k = 0; k < cgb::BK_NUM; k++) C.off[k][C.njobs] = C.total[k];
  }
  return out;
}
// the running jobs as chains: large ones solo, the rest in chunks; streams and events for them
cudaError_t make_plan(cgb_batch &bt)
{
  std::vector<cgb::BatchJob> shared;
  bt.plan.solo.clear();
  for (size_t i = 0; i < bt.jobs.size(); i++) {
    if (bt.slots[i].held) continue;
    if (bt.jobs[i].b.n >= bt.solo_cells)
      bt.plan.solo.push_back(i);
    else
      shared.push_back(bt.jobs[i]);
  }
  bt.plan.chunks  = build_chunks(shared, bt.chains, bt.tiles);
  size_t const nc = bt.plan.chunks.size() + bt.plan.solo.size();
  cudaError_t e;
  while (bt.aux.size() + 1 < nc) {
    cudaStream_t a;
    if ((e = cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking)) != cudaSuccess) return e;
    bt.aux.push_back(a);
  }
  while (bt.ev.size() < nc) {
    cudaEvent_t v;
    if ((e = cudaEventCreateWithFlags(&v, cudaEventDisableTiming)) != cudaSuccess) return e;
    bt.ev.push_back(v);
  }
  return cudaSuccess;
}

// One step of every chain of the plan, queued on the batch stream: chain 0 on it, chain c > 0
// on aux[c - 1], forked from and joined back to it by events (the same calls build the graph
// under capture).  Chains 0 .. chunks-1 are the chunks; the solo jobs follow, each the
// single-box step (ghost fill, dt, step with the CFL reduction for the next) as the box
// engine runs it.
cudaError_t launch_plan(cgb_batch &bt)
{
  cgb_scheme const &s = bt.scheme;
  int const mixed     = s.precision == CGB_MIXED ? 1 : 0;
  auto const &chunks  = bt.plan.chunks;
  size_t const nc     = chunks.size() + bt.plan.solo.size();
  cudaError_t e       = nc > 1 ? cudaEventRecord(bt.ev[0], bt.stream) : cudaSuccess;
  for (size_t c = 1; c < nc && e == cudaSuccess; c++) e = cudaStreamWaitEvent(bt.aux[c - 1], bt.ev[0], 0);
  for (size_t c = 0; c < nc && e == cudaSuccess; c++) {
    cudaStream_t const st = c ? bt.aux[c - 1] : bt.stream;
    if (c < chunks.size()) {
      e = cgb::batch_chunk_step(chunks[c], s.reconstruction, s.riemann_solver, mixed, s.dual_energy, s.n_scalars,
                                bt.c_cfl, s.U_floor, s.temperature_floor, bt.tiles, st);
      continue;
    }
    size_t const i         = bt.plan.solo[c - chunks.size()];
    cgb::BatchJob const &J = bt.jobs[i];
    cgb::Scratch sc{};
    sc.W = J.W, sc.GEp = J.GEp, sc.Epre = J.Epre, sc.dti = J.dti, sc.status = J.status;
    e = cgb::set_boundaries(J.b, J.U, bt.slots[i].flags, st);
    if (e == cudaSuccess) e = cgb::cfl_dt(J.dti, J.dt_t, bt.c_cfl, J.t_end, st);
    if (e == cudaSuccess)
      e = cgb::hydro_step(J.b, s.reconstruction, s.riemann_solver, s.precision, J.U, sc, 0.0, J.dt_t, s.U_floor,
                          s.temperature_floor, 1, st, nullptr, 1);
  }
  for (size_t c = 1; c < nc && e == cudaSuccess; c++) {
    e = cudaEventRecord(bt.ev[c], bt.aux[c - 1]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(bt.stream, bt.ev[c], 0);
  }
  return e;
}
}  // namespace

extern "C" {

const char *cgb_batch_last_error(void) { return g_batch_err.c_str(); }

int cgb_batch_create(cgb_batch **out, const cgb_scheme *scheme, double c_cfl, void *stream)
{
  if (!out || !scheme) return bfail(CGB_ERR_ARGS, "null argument");
  *out                 = nullptr;
  cgb_scheme const &s = *scheme;
  if (s.reconstruction < CGB_PCM || s.reconstruction > CGB_PPMP || s.riemann_solver < CGB_HLLC ||
      s.riemann_solver > CGB_EXACT)
    return bfail(CGB_ERR_ARGS, "bad reconstruction or riemann solver");
  if (s.mhd || s.riemann_solver == CGB_HLLD) return bfail(CGB_ERR_UNSUPPORTED, "batches are hydro only");
  if (s.precision != CGB_MIXED && s.precision != CGB_FP64_FAST)
    return bfail(CGB_ERR_UNSUPPORTED, "batches run the fast FP64 or the mixed-precision form");
  if (s.n_scalars < 0 || s.n_scalars > cgb::NS_MAX || !(s.gamma > 1.0)) return bfail(CGB_ERR_ARGS, "bad scheme");
  if (!(c_cfl > 0)) return bfail(CGB_ERR_ARGS, "c_cfl must be positive");
  if (!stream) return bfail(CGB_ERR_ARGS, "a batch needs its own (non-default) stream");
  cgb_batch *bt = new cgb_batch();
  bt->scheme    = s;
  bt->c_cfl     = c_cfl;
  bt->stream    = (cudaStream_t)stream;
  // a pool of its own, which holds on to the memory of retired jobs (no unmap / remap between
  // a job leaving and the next one joining)
  int dev = 0;
  cudaMemPoolProps props{};
  props.allocType     = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  cudaError_t e       = cudaGetDevice(&dev);
  props.location.id   = dev;
  if (e == cudaSuccess) e = cudaMemPoolCreate(&bt->pool, &props);
  unsigned long long keep = ~0ULL;
  if (e == cudaSuccess) e = cudaMemPoolSetAttribute(bt->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (bt->pool) cudaMemPoolDestroy(bt->pool);
    delete bt;
    return bcuda(e, "batch memory pool");
  }
  *out = bt;
  return CGB_OK;
}

int cgb_batch_destroy(cgb_batch *bt)
{
  if (!bt) return CGB_OK;
  cudaStreamSynchronize(bt->stream);
  for (auto &sl : bt->slots) cudaFreeAsync(sl.mem, bt->stream);
  cudaStreamSynchronize(bt->stream);
  if (bt->pool) cudaMemPoolDestroy(bt->pool);
  if (bt->graph) cudaGraphExecDestroy(bt->graph);
  for (cudaStream_t a : bt->aux) cudaStreamDestroy(a);
  for (cudaEvent_t e : bt->ev) cudaEventDestroy(e);
  delete bt;
  return CGB_OK;
}

// Bytes of library scratch a job of this shape takes (the state itself is the caller's).
long long cgb_batch_job_bytes(const cgb_batch *bt, int nx, int ny, int nz)
{
  if (!bt) return -1;
  cgb::Box b{};
  b.nx = nx, b.ny = ny, b.nz = nz, b.ns = bt->scheme.n_scalars, b.de = bt->scheme.dual_energy ? 1 : 0;
  b.nf = 5 + b.ns + b.de, b.n = (long long)nx * ny * nz;
  return (long long)(al256(cgb::batch_w_bytes(b)) + 2 * al256((size_t)b.n * 8) + 3 * 256);
}

// Add a box to the batch: its state d_conserved (caller-owned, kept resident), shape, cell size,
// boundary flags and end time (t_end <= 0: none).  The job's first dt comes from a CFL reduction
// of the state queued now; it joins the next step.  *job_id identifies it afterwards.
int cgb_batch_add(cgb_batch *bt, double *d_conserved, int nx, int ny, int nz, int n_ghost, double dx, double dy,
                  double dz, const int flags[6], double t_end, int *job_id)
{
  if (!bt || !d_conserved || !flags || !job_id) return bfail(CGB_ERR_ARGS, "null argument");
  std::lock_guard<std::mutex> lk(bt->mu);
  if ((int)bt->jobs.size() >= cgb::BATCH_MAX_JOBS) return bfail(CGB_ERR_ARGS, "batch is full");
  cgb_scheme const &s = bt->scheme;
  int const H = (s.reconstruction == CGB_PPMC || s.reconstruction == CGB_PPMP)   ? 4
                : (s.reconstruction == CGB_PLMC || s.reconstruction == CGB_PLMP) ? 3
                                                                                 : 2;
  if (ny < 2 || nz < 2) return bfail(CGB_ERR_ARGS, "batches hold 3D boxes");
  if (n_ghost < H || nx < 2 * n_ghost + 1 || ny < 2 * n_ghost + 1 || nz < 2 * n_ghost + 1)
    return bfail(CGB_ERR_ARGS, "box too small for the reconstruction stencil");
  if (!(dx > 0 && dy > 0 && dz > 0)) return bfail(CGB_ERR_ARGS, "cell sizes must be positive");
  for (int i = 0; i < 6; i++)
    if (flags[i] < 0 || flags[i] > 5) return bfail(CGB_ERR_ARGS, "boundary flags must be 0..5");
  cgb::BatchJob J{};
  cgb::Box &b = J.b;
  b.nx = nx, b.ny = ny, b.nz = nz, b.ng = n_ghost, b.ns = s.n_scalars, b.de = s.dual_energy ? 1 : 0, b.mhd = 0;
  b.nf = 5 + b.ns + b.de, b.floor_on = s.density_floor ? 1 : 0, b.n = (long long)nx * ny * nz;
  b.gamma = s.gamma, b.dx = dx, b.dy = dy, b.dz = dz, b.density_floor = 0.0;
  size_t const wb = al256(cgb::batch_w_bytes(b)), cb = al256((size_t)b.n * 8);
  size_t const bytes = wb + 2 * cb + 3 * 256;
  void *mem          = nullptr;
  cudaError_t e      = cgb::dev_malloc_pool_async(&mem, bytes, bt->pool, bt->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return bfail(CGB_ERR_NOMEM, "job scratch allocation failed");
  }
  unsigned char *p = (unsigned char *)mem;
  J.U              = d_conserved;
  J.W              = p;
  J.GEp            = (double *)(p + wb);
  J.Epre           = (double *)(p + wb + cb);
  J.dti            = (unsigned long long *)(p + wb + 2 * cb);
  J.status         = (int *)(p + wb + 2 * cb + 256);
  J.dt_t           = (double *)(p + wb + 2 * cb + 512);
  J.t_end          = t_end;
  J.b              = cgb::with_inverses(b);
  cgb::Flags const fl = cgb::ghost_flags(b, flags);
  for (int i = 0; i < 6; i++) J.flags[i] = fl.f[i];
  // zero W (the predictor's unwritten edge cells are read, and discarded, by the sweeps),
  // then the first CFL reduction of the state as it is (real cells only)
  if ((e = cudaMemsetAsync(mem, 0, bytes, bt->stream)) != cudaSuccess ||
      (e = cgb::hydro_calc_dt(b, d_conserved, J.dti, bt->stream)) != cudaSuccess) {
    cudaFreeAsync(mem, bt->stream);
    return bcuda(e, "batch_add");
  }
  bt->jobs.push_back(J);
  cgb_batch::Slot sl{bt->next_id, mem, false, {}};
  for (int i = 0; i < 6; i++) sl.flags[i] = flags[i];
  bt->slots.push_back(sl);
  *job_id   = bt->next_id++;
  bt->dirty = true;
  return CGB_OK;
}

// Remove a job (its scratch is released on the batch stream; the caller's state is kept).
int cgb_batch_remove(cgb_batch *bt, int job_id)
{
  if (!bt) return bfail(CGB_ERR_ARGS, "null batch");
  std::lock_guard<std::mutex> lk(bt->mu);
  int pos = -1;
  for (size_t i = 0; i < bt->slots.size(); i++)
    if (bt->slots[i].id == job_id) pos = (int)i;
  if (pos < 0) return bfail(CGB_ERR_ARGS, "no such job");
  cudaFreeAsync(bt->slots[pos].mem, bt->stream);
  size_t const last = bt->jobs.size() - 1;
  if ((size_t)pos != last) {
    bt->jobs[pos]  = bt->jobs[last];
    bt->slots[pos] = bt->slots[last];
  }
  bt->jobs.pop_back();
  bt->slots.pop_back();
  bt->dirty = true;
  return CGB_OK;
}

int cgb_batch_n_jobs(const cgb_batch *bt) { return bt ? (int)bt->jobs.size() : -1; }

// Hold a job out of the steps (hold = 1) or release it (hold = 0).  A held job keeps its state,
// scratch, time and pending dt; it resumes where it stopped.  Takes effect at the next step.
int cgb_batch_hold(cgb_batch *bt, int job_id, int hold)
{
  if (!bt) return bfail(CGB_ERR_ARGS, "null batch");
  std::lock_guard<std::mutex> lk(bt->mu);
  for (auto &sl : bt->slots) {
    if (sl.id != job_id) continue;
    if (sl.held != (hold != 0)) bt->dirty = true;
    sl.held = hold != 0;
    return CGB_OK;
  }
  return bfail(CGB_ERR_ARGS, "no such job");
}

// Jobs of at least `cells` padded cells run solo: their own chain of the single-box kernels
// (the box engine's step), the others share the batched kernels.  Takes effect at the next step.
int cgb_batch_set_solo_cells(cgb_batch *bt, long long cells)
{
  if (!bt || cells < 0) return bfail(CGB_ERR_ARGS, "bad argument");
  std::lock_guard<std::mutex> lk(bt->mu);
  if (cells != bt->solo_cells) bt->dirty = true;
  bt->solo_cells = cells;
  return CGB_OK;
}

// Minimum number of parallel chains of launches the jobs are spread over (1 .. BATCH_MAX_JOBS;
// more are used when the jobs exceed BATCH_CHUNK per chain).  Takes effect at the next step.
int cgb_batch_set_chains(cgb_batch *bt, int chains)
{
  if (!bt || chains < 1 || chains > cgb::BATCH_MAX_JOBS) return bfail(CGB_ERR_ARGS, "bad argument");
  std::lock_guard<std::mutex> lk(bt->mu);
  if (chains != bt->chains) bt->dirty = true;
  bt->chains = chains;
  return CGB_OK;
}

// Sweep tile set of the shared-kernel chains: 0 or 1 (two compiled shapes; they agree to the
// rounding of the compiler's contractions).  Takes effect at the next step.
int cgb_batch_set_tiles(cgb_batch *bt, int set)
{
  if (!bt || set < 0 || set > 1) return bfail(CGB_ERR_ARGS, "tile set must be 0 or 1");
  std::lock_guard<std::mutex> lk(bt->mu);
  if (set != bt->tiles) bt->dirty = true;
  bt->tiles = set;
  return CGB_OK;
}

// Advance every job of the batch by n_steps on the batch stream, without host synchronisation.
int cgb_batch_step(cgb_batch *bt, int n_steps)
{
  if (!bt || n_steps < 0) return bfail(CGB_ERR_ARGS, "bad argument");
  std::lock_guard<std::mutex> lk(bt->mu);
  if (bt->jobs.empty() || n_steps == 0) return CGB_OK;
  cudaError_t e;
  if (bt->dirty) {
    if (bt->graph) cudaGraphExecDestroy(bt->graph);
    bt->graph = nullptr;
    if ((e = make_plan(*bt)) != cudaSuccess) return bcuda(e, "batch plan");
    bt->dirty  = false;
    bt->stable = 0;
  }
  if (bt->plan.chunks.empty() && bt->plan.solo.empty()) return CGB_OK;  // every job held
  for (int i = 0; i < n_steps; i++) {
    // A job set that changes every step or two (arrivals, departures, holds) is launched
    // directly: a capture and instantiation per change would cost more host time than the
    // launches.  Once it has held for two steps it is captured and replayed.
    if (!bt->graph && bt->stable >= 2) {
      cudaGraph_t g;
      if ((e = cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return bcuda(e, "batch capture");
      cudaError_t const ce = launch_plan(*bt);
      e                    = cudaStreamEndCapture(bt->stream, &g);
      if (ce != cudaSuccess || e != cudaSuccess) return bcuda(ce != cudaSuccess ? ce : e, "batch capture");
      e = cudaGraphInstantiate(&bt->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return bcuda(e, "batch graph");
    }
    e = bt->graph ? cudaGraphLaunch(bt->graph, bt->stream) : launch_plan(*bt);
    if (e != cudaSuccess) return bcuda(e, "batch step");
    bt->stable++;
  }
  bt->steps += n_steps;
  return CGB_OK;
}

namespace
{
const char *kBadJob =
    "the job holds a real cell with non-finite density or energy, or density <= 0 after the negative-density repair";
const char *kTimedOut = "a bounded device wait for a TMA copy ran out; a step of the job left a tile undone";
}

// Time and last dt of one job (synchronises the batch stream).  Returns CGB_ERR_NONFINITE (with t
// and dt filled in) while the job's status word records a bad cell.
int cgb_batch_job_time(cgb_batch *bt, int job_id, double *t, double *dt_last)
{
  if (!bt) return bfail(CGB_ERR_ARGS, "null batch");
  std::lock_guard<std::mutex> lk(bt->mu);
  for (size_t i = 0; i < bt->slots.size(); i++) {
    if (bt->slots[i].id != job_id) continue;
    double h[2];
    int st        = 0;
    cudaError_t e = cudaStreamSynchronize(bt->stream);
    if (e == cudaSuccess) e = cudaMemcpy(h, bt->jobs[i].dt_t, 16, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, bt->jobs[i].status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return bcuda(e, "batch_job_time");
    if (t) *t = h[1];
    if (dt_last) *dt_last = h[0];
    if (st & CGB_STATUS_TIMEOUT) return bfail(CGB_ERR_TIMEOUT, kTimedOut);
    if (st & CGB_STATUS_NONFINITE) return bfail(CGB_ERR_NONFINITE, kBadJob);
    return CGB_OK;
  }
  return bfail(CGB_ERR_ARGS, "no such job");
}

// Status bits (CGB_STATUS_*) of one job without clearing them (synchronises the batch stream).
int cgb_batch_job_status(cgb_batch *bt, int job_id, int *flags)
{
  if (!bt || !flags) return bfail(CGB_ERR_ARGS, "null argument");
  std::lock_guard<std::mutex> lk(bt->mu);
  for (size_t i = 0; i < bt->slots.size(); i++) {
    if (bt->slots[i].id != job_id) continue;
    cudaError_t e = cudaStreamSynchronize(bt->stream);
    if (e == cudaSuccess) e = cudaMemcpy(flags, bt->jobs[i].status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return bcuda(e, "batch_job_status");
    if (*flags & CGB_STATUS_TIMEOUT) return bfail(CGB_ERR_TIMEOUT, kTimedOut);
    if (*flags & CGB_STATUS_NONFINITE) return bfail(CGB_ERR_NONFINITE, kBadJob);
    return CGB_OK;
  }
  return bfail(CGB_ERR_ARGS, "no such job");
}

}  // extern "C"

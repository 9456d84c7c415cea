// sw_batch_graph.cu -- a batch as one CUDA graph of per-lattice step launches.
//
// The second way to advance many lattices together (the first is the
// persistent kernel of sw_batch.cuh).  Each lattice gets a chain of K
// launches of the single-lattice step (sw_step_checked: sw_step / sw_step_accum with the
// storage type's tuned launch configuration, its own __grid_constant__
// parameters and the hardware block scheduler), and the chains are captured
// on separate streams, so they are parallel branches of one graph between a
// fork and a join: lattices run concurrently and the GPU fills the tail of one
// lattice's step with blocks of another's.  A member on the in-place AA
// pattern (entry.ghost set) gets a chain of alternating odd and even
// sw_step_aa launches instead.  The graph is captured again for
// every call (the step index, force row and buffer parity of each launch are
// kernel parameters) and swapped into an executable graph with
// cudaGraphExecUpdate, which keeps the instantiation when the shape (lattices
// and launches per lattice) is unchanged.  Two executable graphs alternate,
// so the one being updated is never the one the GPU may still be running.
#include <new>
#include <vector>

#include "sw_aux.cuh"

struct sw_batch_graph {
  int device = -1;
  cudaStream_t origin = nullptr;                    // capture origin (fork and join)
  std::vector<cudaStream_t> branch;                 // one per lattice
  std::vector<cudaEvent_t> joined;
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  int slot = 0;
  long long launched = 0;                           // step kernels in graphs launched so far
};

namespace {

int status_of(cudaError_t e) { return e == cudaSuccess ? SW_OK : sw::note_cuda_error((int)e); }

cudaError_t ensure_branches(sw_batch_graph *g, int n) {
  while ((int)g->branch.size() < n) {
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      cudaStreamDestroy(s);
      return e;
    }
    g->branch.push_back(s);
    g->joined.push_back(ev);
  }
  return cudaSuccess;
}

bool accumulates(const sw_batch_entry &e, long long t) {
  return e.acc != nullptr && t >= e.n_spin && (t - e.n_spin) % e.acc_every == 0;
}

}  // namespace

extern "C" {

int sw_batch_graph_create(sw_batch_graph **out) {
  if (!out) return SW_ERR_BAD_ARG;
  *out = nullptr;
  sw_batch_graph *g = new (std::nothrow) sw_batch_graph();
  if (!g) return SW_ERR_OOM;
  cudaError_t e = cudaGetDevice(&g->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->origin, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&g->done[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    sw_batch_graph_destroy(g);
    return status_of(e);
  }
  *out = g;
  return SW_OK;
}

int sw_batch_graph_destroy(sw_batch_graph *g) {
  if (!g) return SW_OK;
  for (int i = 0; i < 2; ++i) {
    if (g->done[i]) cudaEventSynchronize(g->done[i]);
    if (g->exec[i]) cudaGraphExecDestroy(g->exec[i]);
    if (g->done[i]) cudaEventDestroy(g->done[i]);
  }
  for (cudaStream_t s : g->branch) cudaStreamDestroy(s);
  for (cudaEvent_t ev : g->joined) cudaEventDestroy(ev);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->origin) cudaStreamDestroy(g->origin);
  delete g;
  return SW_OK;
}

int64_t sw_batch_graph_launches(const sw_batch_graph *g) { return g ? g->launched : -1; }

int sw_batch_graph_run(sw_batch_graph *g, const sw_batch_entry *entries, int32_t n, int dtype, int32_t k_steps,
                       sw_stream s) {
  if (!g || !entries || n <= 0 || n > SW_BATCH_MAX_ENTRIES || k_steps <= 0) return SW_ERR_BAD_ARG;
  if (sw_dtype_size(dtype) == 0) return SW_ERR_BAD_ARG;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return status_of(e);
  if (dev != g->device) return SW_ERR_BAD_ARG;
  for (int i = 0; i < n; ++i) {
    const sw_batch_entry &b = entries[i];
    if (!b.f[0] || !b.f[1] || b.cur0 < 0 || b.cur0 > 1 || b.t0 < 0 || b.steps_left < 0) return SW_ERR_BAD_ARG;
    if ((b.ghost != nullptr) != (b.f[0] == b.f[1])) return SW_ERR_BAD_ARG;    // in place exactly for AA members
    if (b.acc && b.acc_every <= 0) return SW_ERR_BAD_ARG;
  }
  e = ensure_branches(g, n);
  if (e != cudaSuccess) return status_of(e);

  // capture: fork -> one chain per lattice -> join
  e = cudaStreamBeginCapture(g->origin, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return status_of(e);
  int rc = SW_OK;
  e = cudaEventRecord(g->fork, g->origin);
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(g->branch[i], g->fork, 0);
  long long launches = 0;
  for (int k = 0; k < k_steps && e == cudaSuccess && rc == SW_OK; ++k) {
    for (int i = 0; i < n && rc == SW_OK; ++i) {
      const sw_batch_entry &b = entries[i];
      if (k >= b.steps_left) continue;
      const long long t = b.t0 + k;
      const int cur = (b.cur0 + k) & 1;
      sw_stream bs = reinterpret_cast<sw_stream>(g->branch[i]);
      if (b.ghost)                                    // in place: odd and even AA steps alternate
        rc = sw_step_aa(&b.geom, dtype, b.f[0], cur == 0, b.flag, b.tiles, b.uin, b.nu0, b.cs, b.x_sponge,
                        b.nu_sponge, b.force, t, accumulates(b, t) ? b.acc : nullptr, b.ghost, b.status, bs);
      else                                            // the storage type's installed configuration
        rc = sw_step_checked(&b.geom, dtype, b.f[cur], b.f[cur ^ 1], b.flag, b.tiles, b.uin, b.nu0, b.cs,
                             b.x_sponge, b.nu_sponge, b.force, t, accumulates(b, t) ? b.acc : nullptr, -1, b.status,
                             bs);
      ++launches;
    }
  }
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    e = cudaEventRecord(g->joined[i], g->branch[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(g->origin, g->joined[i], 0);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t e_end = cudaStreamEndCapture(g->origin, &graph);
  if (rc != SW_OK || e != cudaSuccess || e_end != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return rc != SW_OK ? rc : status_of(e != cudaSuccess ? e : e_end);
  }

  // swap into the executable graph of this slot (the other one may still run)
  const int slot = g->slot;
  e = cudaEventSynchronize(g->done[slot]);
  if (e == cudaSuccess && g->exec[slot]) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(g->exec[slot], graph, &info) != cudaSuccess) {
      cudaGetLastError();                                   // clear the update failure; instantiate anew
      cudaGraphExecDestroy(g->exec[slot]);
      g->exec[slot] = nullptr;
    }
  }
  if (e == cudaSuccess && !g->exec[slot]) e = cudaGraphInstantiate(&g->exec[slot], graph, 0);
  cudaGraphDestroy(graph);
  if (e == cudaSuccess) e = cudaGraphLaunch(g->exec[slot], reinterpret_cast<cudaStream_t>(s));
  if (e == cudaSuccess) e = cudaEventRecord(g->done[slot], reinterpret_cast<cudaStream_t>(s));
  if (e != cudaSuccess) return status_of(e);
  g->slot ^= 1;
  g->launched += launches;
  return SW_OK;
}

}  // extern "C"

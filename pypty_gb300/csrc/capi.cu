// C ABI of the GB300 ptychography path: host-side validation, workspace planning and
// dispatch to the per-window-size launch paths. See include/pypty_gb300.h for the contract.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "plan.h"

namespace {

using namespace pty;

__global__ void iota_kernel(int* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}

int upload_geometry(const pty_problem_t* p, const Plan& q, void* ws, const int32_t* pos,
                    const float* corr, const int32_t* seq, cudaStream_t st) {
  if (cudaMemcpyAsync(at<int>(ws, q.o_pos), pos, (size_t)q.N * 2 * sizeof(int), cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return PTY_ERR_CUDA;
  if (corr) {
    // host or device memory: the optimizer passes device-resident trial corrections
    if (cudaMemcpyAsync(at<float>(ws, q.o_corr), corr, (size_t)q.N * 2 * sizeof(float), cudaMemcpyDefault,
                        st) != cudaSuccess)
      return PTY_ERR_CUDA;
  } else if (cudaMemsetAsync(at<float>(ws, q.o_corr), 0, (size_t)q.N * 2 * sizeof(float), st) != cudaSuccess) {
    return PTY_ERR_CUDA;
  }
  if (cudaMemcpyAsync(at<int>(ws, q.o_seq), seq, (size_t)q.nseq * sizeof(int), cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return PTY_ERR_CUDA;
  return PTY_OK;
}

int launch_path(const pty_problem_t* p, const Plan& q, const void* obj, const void* probe, const int32_t* pos,
                const float* corr, const int32_t* seq, const float* measured, double* loss_sse,
                void* object_grad, void* probe_grad, float* pos_grad, float* patterns, void* ws,
                cudaStream_t st);

// ------------------------------------------------------------------ launch-graph cache
// A call of pty_loss_and_direction is 15-40 launches plus three small copies. Repeated calls
// with the same problem and the same buffers (an optimizer's line search, a benchmark loop)
// replay one CUDA graph instead: the second call with a given key captures the launch sequence
// on the caller's stream, later ones launch the instantiated graph. The geometry copies in the
// graph read the caller's host buffers when the graph runs, so their current contents are used;
// the host-side checks (validation, positions in range) still run on every call. Calls are not
// cached while the launch profiler records, when the caller's stream is itself being captured,
// for 256-px windows, or when a host buffer is pageable (its copy cannot be captured).
struct GraphKey {
  int device;
  pty_problem_t prob;
  uint64_t dist_hash;
  const void* ptr[10];
  size_t ws_bytes;
  cudaStream_t st;
  bool operator==(const GraphKey& o) const { return std::memcmp(this, &o, sizeof(GraphKey)) == 0; }
};

struct GraphEntry {
  GraphKey key;
  bool used = false;
  bool uncapturable = false;
  int calls = 0;
  uint64_t last = 0;
  cudaGraphExec_t exec = nullptr;
};

constexpr int kGraphSlots = 16;
std::mutex g_graph_mu;
GraphEntry g_graphs[kGraphSlots];
uint64_t g_graph_clock = 0;

GraphKey make_key(const pty_problem_t* p, const void* const (&ptrs)[10], size_t ws_bytes, cudaStream_t st) {
  GraphKey k;
  std::memset(&k, 0, sizeof(k));   // padding bytes take part in the comparison
  cudaGetDevice(&k.device);
  k.prob = *p;
  k.prob.slice_distances = nullptr;
  uint64_t h = 1469598103934665603ull;   // FNV-1a over the per-step distances (baked into the launches)
  if (p->slice_distances) {
    const unsigned char* b = reinterpret_cast<const unsigned char*>(p->slice_distances);
    for (size_t i = 0; i < (size_t)(p->n_slices > 1 ? p->n_slices - 1 : 0) * sizeof(float); ++i) h = (h ^ b[i]) * 1099511628211ull;
    h ^= 1;
  }
  k.dist_hash = h;
  for (int i = 0; i < 10; ++i) k.ptr[i] = ptrs[i];
  k.ws_bytes = ws_bytes;
  k.st = st;
  return k;
}

// host pointers must be page-locked (or device memory) for their copies to be captured
bool capturable_host(const void* ptr) {
  if (!ptr) return true;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Stream to capture on: a private non-blocking stream per device (capture is not permitted on
// the legacy default stream that callers often use; a capture executes nothing, so the stream
// it is recorded on does not matter for the graph).
cudaStream_t capture_stream(int device) {
  static cudaStream_t streams[64] = {};
  if (device < 0 || device >= 64) return nullptr;
  if (!streams[device] && cudaStreamCreateWithFlags(&streams[device], cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    streams[device] = nullptr;
  }
  return streams[device];
}

// Runs the call through the cache; returns false when the caller should launch directly.
bool run_cached(const pty_problem_t* p, const Plan& q, const void* obj, const void* probe, const int32_t* pos,
                const float* corr, const int32_t* seq, const float* measured, double* loss_sse, void* object_grad,
                void* probe_grad, float* pos_grad, void* ws, size_t ws_bytes, cudaStream_t st, int* rc) {
  if (q.W > 128 || prof_active()) return false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return false;
  }
  const void* ptrs[10] = {obj, probe, pos, corr, seq, measured, loss_sse, object_grad, probe_grad, pos_grad};
  const GraphKey key = make_key(p, ptrs, ws_bytes, st);
  std::lock_guard<std::mutex> lock(g_graph_mu);
  GraphEntry* e = nullptr;
  GraphEntry* victim = &g_graphs[0];
  for (GraphEntry& g : g_graphs) {
    if (g.used && g.key == key) {
      e = &g;
      break;
    }
    if (!g.used || (victim->used && g.last < victim->last)) victim = &g;
  }
  if (!e) {   // first call with this key: record it and launch directly
    if (victim->exec) {
      cudaStreamSynchronize(victim->key.st);   // its last replay may still run
      cudaGraphExecDestroy(victim->exec);
    }
    *victim = GraphEntry{};
    victim->key = key;
    victim->used = true;
    victim->calls = 1;
    victim->last = ++g_graph_clock;
    return false;
  }
  e->last = ++g_graph_clock;
  e->calls += 1;
  if (e->uncapturable) return false;
  if (!e->exec) {
    if (!capturable_host(pos) || !capturable_host(seq) || !capturable_host(corr)) {
      e->uncapturable = true;
      return false;
    }
    cudaStream_t cap = capture_stream(key.device);
    if (!cap || cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      e->uncapturable = true;
      return false;
    }
    const int r = launch_path(p, q, obj, probe, pos, corr, seq, measured, loss_sse, object_grad, probe_grad,
                              pos_grad, nullptr, ws, cap);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(cap, &graph);
    cudaGraphExec_t exec = nullptr;
    const bool ok = r == PTY_OK && ec == cudaSuccess && graph &&
                    cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
      cudaGetLastError();
      e->uncapturable = true;
      return false;   // nothing ran: the caller launches directly
    }
    e->exec = exec;
  }
  *rc = cudaGraphLaunch(e->exec, st) == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
  return true;
}

int run_common(const pty_problem_t* p, const void* obj, const void* probe, const int32_t* pos,
               const float* corr, const int32_t* seq, const float* measured, double* loss_sse,
               void* object_grad, void* probe_grad, float* pos_grad, float* patterns, void* ws,
               size_t ws_bytes, void* stream) {
  int rc = validate(p);
  if (rc) return rc;
  if (!obj || !probe || !pos || !seq || !ws) return PTY_ERR_INVALID;
  if (!patterns && (!measured || !loss_sse)) return PTY_ERR_INVALID;
  if ((rc = check_geometry(p, pos, seq))) return rc;
  const Plan q = make_plan(p);
  if (ws_bytes < q.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!patterns && run_cached(p, q, obj, probe, pos, corr, seq, measured, loss_sse, object_grad, probe_grad,
                              pos_grad, ws, ws_bytes, st, &rc))
    return rc;
  return launch_path(p, q, obj, probe, pos, corr, seq, measured, loss_sse, object_grad, probe_grad, pos_grad,
                     patterns, ws, st);
}

int launch_path(const pty_problem_t* p, const Plan& q, const void* obj, const void* probe, const int32_t* pos,
                const float* corr, const int32_t* seq, const float* measured, double* loss_sse,
                void* object_grad, void* probe_grad, float* pos_grad, float* patterns, void* ws,
                cudaStream_t st) {
  int rc;
  if ((rc = upload_geometry(p, q, ws, pos, corr, seq, st))) return rc;
  if (q.W == 64)
    return run_path<64>(p, q, static_cast<const float2*>(obj), static_cast<const float2*>(probe), measured,
                        loss_sse, static_cast<float2*>(object_grad), static_cast<float2*>(probe_grad), pos_grad,
                        patterns, ws, st);
  if (q.W == 256)
    return run_path<256>(p, q, static_cast<const float2*>(obj), static_cast<const float2*>(probe), measured,
                         loss_sse, static_cast<float2*>(object_grad), static_cast<float2*>(probe_grad), pos_grad,
                         patterns, ws, st);
  return run_path<128>(p, q, static_cast<const float2*>(obj), static_cast<const float2*>(probe), measured,
                       loss_sse, static_cast<float2*>(object_grad), static_cast<float2*>(probe_grad), pos_grad,
                       patterns, ws, st);
}

// Launch profiler: one CUDA event per marked launch, read back in pty_profile_end.
// Single-threaded use only (profiling / benchmarking).
// A mark's interval ends at the next mark recorded on the same stream, so launches that run
// on two streams at once are each timed on their own stream.
struct Profiler {
  bool on = false;
  int cap = 0, n = 0;
  cudaEvent_t* ev = nullptr;
  int* ids = nullptr;
  cudaStream_t* sts = nullptr;
  bool overflow = false;
};
Profiler g_prof;

const char* kKernelNames[KID_COUNT] = {
    "build_twiddles", "tables", "probe_fft", "obj_to_slices", "object_windows", "fused_multislice",
    "grad_windows", "tile_lists", "scatter_tiles", "probe_partial", "slices_to_obj", "probe_final",
    "finalize_scalars", "fft2_batch", "layout", "clean_tables", "clean_pass_x", "clean_pass_y",
    "clean_pass_x_inverse", "opt_vector", "opt_scalar", "opt_accept", "orthogonalize_modes", "dft_tables",
    "dft_gemm_bf16x3", "layered_elementwise", "warm_start_net", "probe_spectrum", "shifted_probes"};

}  // namespace

namespace pty {
void prof_mark(cudaStream_t st, int id) {
  Profiler& P = g_prof;
  if (!P.on) return;
  if (P.n >= P.cap) {
    P.overflow = true;
    return;
  }
  cudaEventRecord(P.ev[P.n], st);
  P.sts[P.n] = st;
  P.ids[P.n++] = id;
}

bool prof_active() { return g_prof.on; }

constexpr int kMaxSideDevices = 64;
struct SideStreams {
  SideStream dev[kMaxSideDevices];
  ~SideStreams() {
    for (SideStream& d : dev) {
      for (cudaEvent_t e : d.ev)
        if (e) cudaEventDestroy(e);
      if (d.s) cudaStreamDestroy(d.s);
      if (d.s2) cudaStreamDestroy(d.s2);
    }
  }
};
static thread_local SideStreams t_side;

int side_stream(SideStream** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PTY_ERR_CUDA;
  if (dev < 0 || dev >= kMaxSideDevices) return PTY_ERR_UNSUPPORTED;
  SideStream& d = t_side.dev[dev];
  if (!d.s) {
    SideStream n;
    bool ok = cudaStreamCreateWithFlags(&n.s, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&n.s2, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t& e : n.ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      for (cudaEvent_t e : n.ev)
        if (e) cudaEventDestroy(e);
      if (n.s) cudaStreamDestroy(n.s);
      if (n.s2) cudaStreamDestroy(n.s2);
      return PTY_ERR_CUDA;
    }
    d = n;
  }
  *out = &d;
  return PTY_OK;
}
}  // namespace pty

extern "C" {

int pty_profile_begin(int32_t max_launches) {
  Profiler& P = g_prof;
  if (max_launches <= 0) return PTY_ERR_INVALID;
  if (2 * max_launches > P.cap) {
    for (int i = 0; i < P.cap; ++i) cudaEventDestroy(P.ev[i]);
    delete[] P.ev;
    delete[] P.ids;
    delete[] P.sts;
    P.cap = 0;
    P.ev = new cudaEvent_t[2 * max_launches];
    P.ids = new int[2 * max_launches];
    P.sts = new cudaStream_t[2 * max_launches];
    for (int i = 0; i < 2 * max_launches; ++i) {
      if (cudaEventCreate(&P.ev[i]) != cudaSuccess) return PTY_ERR_CUDA;
      P.cap = i + 1;
    }
  }
  P.n = 0;
  P.overflow = false;
  P.on = true;
  return PTY_OK;
}

int pty_profile_end(double* ms_by_kernel, int32_t* launches_by_kernel, int32_t n_kinds) {
  Profiler& P = g_prof;
  if (!P.on) return PTY_ERR_INVALID;
  P.on = false;
  for (int k = 0; k < n_kinds; ++k) {
    if (ms_by_kernel) ms_by_kernel[k] = 0.0;
    if (launches_by_kernel) launches_by_kernel[k] = 0;
  }
  if (P.n == 0) return PTY_OK;
  for (int i = 0; i < P.n; ++i)
    if (cudaEventSynchronize(P.ev[i]) != cudaSuccess) return PTY_ERR_CUDA;
  for (int i = 0; i + 1 < P.n; ++i) {
    const int id = P.ids[i];
    if (id < 0 || id >= n_kinds) continue;
    int j = i + 1;
    while (j < P.n && P.sts[j] != P.sts[i]) ++j;
    if (j == P.n) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, P.ev[i], P.ev[j]) != cudaSuccess) return PTY_ERR_CUDA;
    if (ms_by_kernel) ms_by_kernel[id] += ms;
    if (launches_by_kernel) launches_by_kernel[id] += 1;
  }
  return P.overflow ? PTY_ERR_WORKSPACE : PTY_OK;
}

const char* pty_kernel_name(int32_t id) { return (id >= 0 && id < KID_COUNT) ? kKernelNames[id] : "unknown"; }

int pty_kernel_count(void) { return KID_COUNT; }


int pty_graph_cache_info(int32_t* keys, int32_t* graphs, int32_t* uncapturable, int64_t* replays) {
  std::lock_guard<std::mutex> lock(g_graph_mu);
  int32_t k = 0, g = 0, u = 0;
  int64_t r = 0;
  for (const GraphEntry& e : g_graphs) {
    if (!e.used) continue;
    ++k;
    if (e.exec) {
      ++g;
      r += e.calls - 2;   // the first call launched directly, the second captured and launched
    }
    if (e.uncapturable) ++u;
  }
  if (keys) *keys = k;
  if (graphs) *graphs = g;
  if (uncapturable) *uncapturable = u;
  if (replays) *replays = r;
  return PTY_OK;
}

int pty_version(void) { return 100; }

const char* pty_status_string(int status) {
  switch (status) {
    case PTY_OK: return "ok";
    case PTY_ERR_INVALID: return "invalid argument";
    case PTY_ERR_UNSUPPORTED:
      return "unsupported problem (window 64, 128 or 256; Mp*Mo <= 8 for 64/128, <= 64 for 256)";
    case PTY_ERR_POSITION: return "scan position or sequence entry out of range";
    case PTY_ERR_WORKSPACE: return "workspace too small";
    case PTY_ERR_CUDA: return "CUDA launch or copy failed";
    default: return "unknown status";
  }
}

int pty_workspace_bytes(const pty_problem_t* problem, size_t* bytes) {
  if (problem && problem->n_sequence == 0) {   // an empty sequence needs no workspace
    pty_problem_t one = *problem;
    one.n_sequence = 1;
    const int rc = validate(&one);
    if (rc) return rc;
    if (!bytes) return PTY_ERR_INVALID;
    *bytes = 0;
    return PTY_OK;
  }
  int rc = validate(problem);
  if (rc) return rc;
  if (!bytes) return PTY_ERR_INVALID;
  *bytes = make_plan(problem).total;
  return PTY_OK;
}

int pty_loss_and_direction(const pty_problem_t* problem, const void* obj, const void* probe,
                           const int32_t* positions_host, const float* pos_correction_host,
                           const int32_t* sequence_host, const float* measured, double* loss_sse,
                           void* object_grad, void* probe_grad, float* pos_grad, void* workspace,
                           size_t workspace_bytes, void* stream) {
  if (problem && problem->n_sequence == 0) {
    // no positions: the reference's batch loop does not run, so the loss, sse and every
    // gradient are zero (pypty/objective.py:372-382, 741-742)
    pty_problem_t one = *problem;
    one.n_sequence = 1;
    const int rc = validate(&one);
    if (rc) return rc;
    if (!loss_sse || (problem->step_obj && !object_grad) || (problem->step_probe && !probe_grad) ||
        (problem->step_pos && !pos_grad))
      return PTY_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t W = (size_t)problem->window;
    bool ok = cudaMemsetAsync(loss_sse, 0, 2 * sizeof(double), st) == cudaSuccess;
    if (object_grad)
      ok = ok && cudaMemsetAsync(object_grad, 0,
                                 (size_t)problem->obj_ny * problem->obj_nx * problem->n_slices *
                                     problem->n_obj_modes * sizeof(float2),
                                 st) == cudaSuccess;
    if (probe_grad)
      ok = ok && cudaMemsetAsync(probe_grad, 0, W * W * problem->n_probe_modes * sizeof(float2), st) == cudaSuccess;
    if (pos_grad)
      ok = ok && cudaMemsetAsync(pos_grad, 0, (size_t)problem->n_positions * 2 * sizeof(float), st) == cudaSuccess;
    return ok ? PTY_OK : PTY_ERR_CUDA;
  }
  return run_common(problem, obj, probe, positions_host, pos_correction_host, sequence_host, measured, loss_sse,
                    object_grad, probe_grad, pos_grad, nullptr, workspace, workspace_bytes, stream);
}

int pty_simulate_patterns(const pty_problem_t* problem, const void* obj, const void* probe,
                          const int32_t* positions_host, const float* pos_correction_host,
                          const int32_t* sequence_host, float* patterns, void* workspace,
                          size_t workspace_bytes, void* stream) {
  if (!patterns) return PTY_ERR_INVALID;
  return run_common(problem, obj, probe, positions_host, pos_correction_host, sequence_host, nullptr, nullptr,
                    nullptr, nullptr, nullptr, patterns, workspace, workspace_bytes, stream);
}

int pty_split_workspace_bytes(const pty_problem_t* problem, size_t* bytes) {
  int rc = validate(problem);
  if (rc) return rc;
  if (!bytes) return PTY_ERR_INVALID;
  *bytes = make_plan(problem, true).total;
  return PTY_OK;
}

int pty_forward(const pty_problem_t* problem, const void* obj, const void* probe, const int32_t* positions_host,
                const float* pos_correction_host, const int32_t* sequence_host, const float* measured,
                double* loss_sse, void* workspace, size_t workspace_bytes, void* stream) {
  int rc = validate(problem);
  if (rc) return rc;
  if (!obj || !probe || !positions_host || !sequence_host || !measured || !loss_sse || !workspace)
    return PTY_ERR_INVALID;
  if ((rc = check_geometry(problem, positions_host, sequence_host))) return rc;
  const Plan q = make_plan(problem, true);
  if (workspace_bytes < q.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if ((rc = upload_geometry(problem, q, workspace, positions_host, pos_correction_host, sequence_host, st)))
    return rc;
  const float2* o = static_cast<const float2*>(obj);
  const float2* pr = static_cast<const float2*>(probe);
  if (q.W == 64) return run_forward<64>(problem, q, o, pr, measured, loss_sse, workspace, st);
  if (q.W == 256) return run_forward<256>(problem, q, o, pr, measured, loss_sse, workspace, st);
  return run_forward<128>(problem, q, o, pr, measured, loss_sse, workspace, st);
}

int pty_backward(const pty_problem_t* problem, double* loss_sse, void* object_grad, void* probe_grad,
                 float* pos_grad, void* workspace, size_t workspace_bytes, void* stream) {
  int rc = validate(problem);
  if (rc) return rc;
  if (!loss_sse || !workspace) return PTY_ERR_INVALID;
  if ((problem->step_obj && !object_grad) || (problem->step_probe && !probe_grad) ||
      (problem->step_pos && !pos_grad))
    return PTY_ERR_INVALID;
  const Plan q = make_plan(problem, true);
  if (workspace_bytes < q.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float2* og = static_cast<float2*>(object_grad);
  float2* pg = static_cast<float2*>(probe_grad);
  if (q.W == 64) return run_backward<64>(problem, q, loss_sse, og, pg, pos_grad, workspace, st);
  if (q.W == 256) return run_backward<256>(problem, q, loss_sse, og, pg, pos_grad, workspace, st);
  return run_backward<128>(problem, q, loss_sse, og, pg, pos_grad, workspace, st);
}

// ------------------------------------------------------------------ multislice_core seams
static int ms_validate(int32_t B, int32_t W, int32_t Z, int32_t Mp, int32_t Mo, int32_t Ny, int32_t Nx) {
  if (W != 64 && W != 128) return PTY_ERR_UNSUPPORTED;
  if (B <= 0 || Z <= 0 || Mp <= 0 || Mo <= 0 || Ny < 0 || Nx < 0) return PTY_ERR_INVALID;
  if (Mp * Mo > 8) return PTY_ERR_UNSUPPORTED;
  return PTY_OK;
}

static int ms_upload_positions(const MsPlan& q, const int32_t* pos, void* ws, cudaStream_t st) {
  for (int b = 0; b < q.B; ++b) {
    const int y = pos[2 * b], x = pos[2 * b + 1];
    if (y < 0 || x < 0 || y + q.W > q.Ny || x + q.W > q.Nx) return PTY_ERR_POSITION;
  }
  if (cudaMemcpyAsync(at<int>(ws, q.o_pos), pos, (size_t)q.B * 2 * sizeof(int), cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return PTY_ERR_CUDA;
  iota_kernel<<<(q.B + 255) / 256, 256, 0, st>>>(at<int>(ws, q.o_seq), q.B);
  return cuda_status();
}

int pty_multislice_workspace_bytes(int32_t batch, int32_t window, int32_t n_slices, int32_t n_probe_modes,
                                   int32_t n_obj_modes, int32_t obj_ny, int32_t obj_nx, size_t* bytes) {
  int rc = ms_validate(batch, window, n_slices, n_probe_modes, n_obj_modes, obj_ny, obj_nx);
  if (rc) return rc;
  if (!bytes) return PTY_ERR_INVALID;
  *bytes = make_ms_plan(window, batch, n_slices, n_probe_modes, n_obj_modes, obj_ny, obj_nx).total;
  return PTY_OK;
}

int pty_multislice(const void* probe_b, const void* obj_b, const void* propagator, float edge_mult, int32_t batch,
                   int32_t window, int32_t n_slices, int32_t n_probe_modes, int32_t n_obj_modes, void* waves,
                   void* exit_wave, void* workspace, size_t workspace_bytes, void* stream) {
  int rc = ms_validate(batch, window, n_slices, n_probe_modes, n_obj_modes, 0, 0);
  if (rc) return rc;
  if (!probe_b || !obj_b || !propagator || !waves || !exit_wave || !workspace) return PTY_ERR_INVALID;
  const MsPlan q = make_ms_plan(window, batch, n_slices, n_probe_modes, n_obj_modes, 0, 0);
  if (workspace_bytes < q.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  iota_kernel<<<(q.B + 255) / 256, 256, 0, st>>>(at<int>(workspace, q.o_seq), q.B);
  auto f = [](const void* x) { return static_cast<const float2*>(x); };
  auto g = [](void* x) { return static_cast<float2*>(x); };
  if (window == 64)
    return run_ms_forward<64>(q, f(probe_b), f(obj_b), f(propagator), edge_mult, g(waves), g(exit_wave), workspace, st);
  return run_ms_forward<128>(q, f(probe_b), f(obj_b), f(propagator), edge_mult, g(waves), g(exit_wave), workspace,
                             st);
}

int pty_multislice_grads(const void* d_exit, const void* waves, const void* obj_b, const void* propagator,
                         float edge_mult, const float* mask_clean, const int32_t* positions_host, int32_t batch,
                         int32_t window, int32_t n_slices, int32_t n_probe_modes, int32_t n_obj_modes,
                         int32_t obj_ny, int32_t obj_nx, int32_t step_obj, void* object_grad, void* probe_grad,
                         void* workspace, size_t workspace_bytes, void* stream) {
  int rc = ms_validate(batch, window, n_slices, n_probe_modes, n_obj_modes, obj_ny, obj_nx);
  if (rc) return rc;
  if (!d_exit || !obj_b || !propagator || !workspace) return PTY_ERR_INVALID;
  if (step_obj && (!waves || !mask_clean || !positions_host || !object_grad)) return PTY_ERR_INVALID;
  const MsPlan q = make_ms_plan(window, batch, n_slices, n_probe_modes, n_obj_modes, obj_ny, obj_nx);
  if (workspace_bytes < q.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (step_obj) {
    if ((rc = ms_upload_positions(q, positions_host, workspace, st))) return rc;
  } else {
    iota_kernel<<<(q.B + 255) / 256, 256, 0, st>>>(at<int>(workspace, q.o_seq), q.B);
  }
  auto f = [](const void* x) { return static_cast<const float2*>(x); };
  auto g = [](void* x) { return static_cast<float2*>(x); };
  if (window == 64)
    return run_ms_grads<64>(q, f(d_exit), f(waves), f(obj_b), f(propagator), edge_mult, mask_clean, step_obj ? 1 : 0,
                            g(object_grad), g(probe_grad), workspace, st);
  return run_ms_grads<128>(q, f(d_exit), f(waves), f(obj_b), f(propagator), edge_mult, mask_clean, step_obj ? 1 : 0,
                           g(object_grad), g(probe_grad), workspace, st);
}

int pty_scatteradd_workspace_bytes(int32_t batch, int32_t window, int32_t n_planes, int32_t obj_ny,
                                   int32_t obj_nx, size_t* bytes) {
  return pty_multislice_workspace_bytes(batch, window, n_planes, 1, 1, obj_ny, obj_nx, bytes);
}

int pty_scatteradd(void* full, int32_t obj_ny, int32_t obj_nx, int32_t n_planes, const int32_t* positions_host,
                   int32_t batch, int32_t window, const void* chop, void* workspace, size_t workspace_bytes,
                   void* stream) {
  int rc = ms_validate(batch, window, n_planes, 1, 1, obj_ny, obj_nx);
  if (rc) return rc;
  if (!full || !positions_host || !chop || !workspace) return PTY_ERR_INVALID;
  const MsPlan q = make_ms_plan(window, batch, n_planes, 1, 1, obj_ny, obj_nx);
  if (workspace_bytes < q.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if ((rc = ms_upload_positions(q, positions_host, workspace, st))) return rc;
  if (window == 64)
    return run_scatteradd<64>(q, static_cast<float2*>(full), static_cast<const float2*>(chop), workspace, st);
  return run_scatteradd<128>(q, static_cast<float2*>(full), static_cast<const float2*>(chop), workspace, st);
}

int pty_fft2_workspace_bytes(int32_t window, size_t* bytes) {
  if (window != 64 && window != 128 && window != 256) return PTY_ERR_UNSUPPORTED;
  if (!bytes) return PTY_ERR_INVALID;
  *bytes = align_up(tw_count(window) * sizeof(float2));
  return PTY_OK;
}

int pty_fft2(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse, int32_t shift,
             void* workspace, size_t workspace_bytes, void* stream) {
  if (window != 64 && window != 128 && window != 256) return PTY_ERR_UNSUPPORTED;
  if (!in || !out || !workspace || batch <= 0) return PTY_ERR_INVALID;
  size_t need = 0;
  pty_fft2_workspace_bytes(window, &need);
  if (workspace_bytes < need) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float2* tw = static_cast<float2*>(workspace);
  const float2* src = static_cast<const float2*>(in);
  float2* dst = static_cast<float2*>(out);
  if (window == 64) return run_fft2<64>(src, dst, batch, inverse, shift, tw, st);
  if (window == 256) return run_fft2<256>(src, dst, batch, inverse, shift, tw, st);
  return run_fft2<128>(src, dst, batch, inverse, shift, tw, st);
}

}  // extern "C"

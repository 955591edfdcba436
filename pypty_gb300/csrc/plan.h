// Workspace plan shared by the C ABI and the per-window-size launch paths.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/pypty_gb300.h"
#include "window_fft.cuh"

namespace pty {

constexpr int kTileSize = 32;   // object tile edge of the deterministic scatter

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Byte offsets of every buffer inside the caller's workspace.
struct Plan {
  int W, Ny, Nx, Z, Mo, Mp, N, nseq, Bb, nbatch, zm, ntx, nty, ntiles, nchunk, chunk;
  size_t o_tw, o_mask, o_mask_sc, o_prop, o_prop_edge, o_pyx, o_sx, o_sy, o_probe_f;
  size_t o_pos, o_corr, o_seq, o_obj, o_grad, o_obl, o_stack, o_gsum, o_fprobe, o_partial;
  size_t o_lists, o_counts, o_loss_part, o_pos_part, o_sim, o_err, o_gbuf, o_psi, o_dldi, o_pgr, o_seg, o_gpark;
  size_t total;
  int ckpt;   // kept slices every ckpt (256 windows)
  bool split;   // one batch with every position: pty_forward / pty_backward
  // W <= 128 with several batches: object windows, wave stacks, gradient windows and shifted
  // probes are double-buffered (nbuf = 2): consecutive batches' fused kernels run on two
  // streams (one's tail overlaps the next one's start) and a third stream extracts batch
  // ib + 1's windows and scatters batch ib's gradients meanwhile; s_* are the buffer strides
  // in bytes
  int nbuf;
  size_t s_obl, s_gsum, s_fprobe, s_stack;
  int per_step;   // one propagator table per slice step (slice_distances given, Z > 1)
  size_t o_steps;
  // scatter runs per tile (scatter_tiles_kernel groups): > 1 when tiles x slices give too few
  // blocks to fill the GPU; o_scpart holds their partial tiles
  int sgroups;
  size_t o_scpart;
  size_t o_done;   // per (slice, tile) count of finished run blocks (sgroups > 1)
};

// blocks the scatter aims for: two per SM of a 152-SM GB300
constexpr int kScatterBlocks = 304;

// twiddle tables in global memory: W = 256 windows use the 128 tables of their sub-transforms
inline int tw_count(int W) { return W == 64 ? Geo<64>::TW1 + Geo<64>::TW2 : Geo<128>::TW1 + Geo<128>::TW2; }

inline int validate(const pty_problem_t* p) {
  if (!p) return PTY_ERR_INVALID;
  if (p->window != 64 && p->window != 128 && p->window != 256) return PTY_ERR_UNSUPPORTED;
  if (p->obj_ny <= 0 || p->obj_nx <= 0 || p->n_slices <= 0 || p->n_obj_modes <= 0 ||
      p->n_probe_modes <= 0 || p->n_positions <= 0 || p->n_sequence <= 0 || p->compute_batch <= 0)
    return PTY_ERR_INVALID;
  // W <= 128: the modes of a position form one cluster (<= 8 blocks); W = 256: the modes run
  // one after another inside the position's 4-block cluster
  if (p->n_obj_modes * p->n_probe_modes > (p->window == 256 ? 64 : 8)) return PTY_ERR_UNSUPPORTED;
  if (p->algorithm < PTY_LSQ_SQRT || p->algorithm > PTY_LSQ_SQRT_2) return PTY_ERR_UNSUPPORTED;
  if (p->step_pos && !p->probe_shift) return PTY_ERR_INVALID;
  if ((int64_t)p->obj_ny * p->obj_nx >= (int64_t)1 << 31) return PTY_ERR_UNSUPPORTED;
  if (p->checkpoint_every > 1 && p->window != 256) return PTY_ERR_UNSUPPORTED;
  if (p->slice_distances)
    for (int z = 0; z + 1 < p->n_slices; ++z)
      if (!(p->slice_distances[z] == p->slice_distances[z])) return PTY_ERR_INVALID;   // NaN
  return PTY_OK;
}

// split = true plans one batch holding every position of the sequence, kept in the
// workspace between pty_forward and pty_backward.
inline Plan make_plan(const pty_problem_t* p, bool split = false) {
  Plan q{};
  q.split = split;
  q.W = p->window;
  q.Ny = p->obj_ny;
  q.Nx = p->obj_nx;
  q.Z = p->n_slices;
  q.Mo = p->n_obj_modes;
  q.Mp = p->n_probe_modes;
  q.N = p->n_positions;
  q.nseq = p->n_sequence;
  q.Bb = split ? p->n_sequence : std::min(p->compute_batch, p->n_sequence);
  q.nbatch = (q.nseq + q.Bb - 1) / q.Bb;
  q.zm = q.Z * q.Mo;
  q.ntx = (q.Nx + kTileSize - 1) / kTileSize;
  q.nty = (q.Ny + kTileSize - 1) / kTileSize;
  q.ntiles = q.ntx * q.nty;
  q.chunk = 8;
  q.nchunk = (q.Bb + q.chunk - 1) / q.chunk;
  const size_t WW = (size_t)q.W * q.W, c8 = sizeof(float2), f4 = sizeof(float);
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align_up(bytes); return r; };
  q.o_tw = take(tw_count(q.W) * c8);
  q.o_mask = take(WW * f4);
  q.o_mask_sc = take(WW * f4);
  q.o_prop = take(WW * c8);
  q.o_prop_edge = take(WW * c8);
  q.o_pyx = take(2 * (size_t)q.W * c8);
  q.o_sx = take(q.W * f4);
  q.o_sy = take(q.W * f4);
  q.o_probe_f = take(q.Mp * WW * c8);
  q.o_pos = take((size_t)q.N * 2 * sizeof(int));
  q.o_corr = take((size_t)q.N * 2 * f4);
  q.o_seq = take((size_t)q.nseq * sizeof(int));
  q.o_obj = take((size_t)q.zm * q.Ny * q.Nx * c8);
  q.o_grad = take((size_t)q.zm * q.Ny * q.Nx * c8);
  q.nbuf = (!split && q.W <= 128 && q.nbatch > 1) ? 2 : 1;
  q.s_obl = align_up((size_t)q.Bb * q.zm * WW * c8);
  // W <= 128: one contribution window per probe mode (the fused kernel's adjoint writes each
  // mode's own; grad_windows_kernel sums them); 256 windows: one probe-mode-summed window
  q.s_gsum = q.W <= 128 ? align_up((size_t)q.Bb * q.zm * q.Mp * WW * c8) : q.s_obl;
  q.s_fprobe = align_up((size_t)q.Bb * q.Mp * WW * c8);
  q.o_obl = take(q.nbuf * q.s_obl);
  q.ckpt = (p->window == 256 && p->checkpoint_every > 1) ? std::min(p->checkpoint_every, q.Z) : 1;
  const int n_kept = (q.Z + q.ckpt - 1) / q.ckpt;
  q.s_stack = align_up((size_t)q.Bb * n_kept * q.Mp * q.Mo * WW * c8);
  q.o_stack = take(q.nbuf * q.s_stack);
  q.o_gsum = take(q.nbuf * q.s_gsum);
  q.o_fprobe = take(q.nbuf * q.s_fprobe);
  q.o_partial = take((size_t)q.nchunk * q.Mp * WW * c8);
  q.o_lists = take((size_t)q.ntiles * q.Bb * sizeof(int));
  q.o_counts = take((size_t)q.ntiles * sizeof(int));
  q.o_loss_part = take((size_t)q.nseq * 2 * sizeof(double));
  q.o_pos_part = take((size_t)q.nseq * q.Mp * 2 * sizeof(double));
  q.o_sim = take((size_t)q.Bb * WW * f4);
  q.o_err = take(sizeof(int));
  const bool w256 = q.W == 256;
  q.o_gbuf = take(split && !w256 ? (size_t)q.Bb * q.Mp * q.Mo * WW * c8 : 0);
  q.o_psi = take(w256 ? (size_t)q.Bb * q.Mp * q.Mo * WW * c8 : 0);
  q.o_dldi = take(w256 ? (size_t)q.Bb * WW * f4 : 0);
  q.o_pgr = take(w256 && q.Mo > 1 ? (size_t)q.Bb * q.Mp * WW * c8 : 0);
  q.o_seg = take(q.ckpt > 1 ? (size_t)q.Bb * q.ckpt * WW * c8 : 0);
  q.o_gpark = take(q.ckpt > 1 ? (size_t)q.Bb * WW * c8 : 0);
  q.per_step = p->slice_distances && q.Z > 1;
  q.o_steps = take(q.per_step ? (size_t)(q.Z - 1) * WW * c8 : 0);
  {
    const int cells = q.ntiles * q.zm;
    int g = (kScatterBlocks + cells - 1) / cells;
    g = std::min(g, std::max(1, q.Bb / 8));   // runs of at least ~8 windows
    q.sgroups = std::max(1, std::min(g, 32));
  }
  q.o_scpart = take(q.sgroups > 1 ? (size_t)q.sgroups * q.ntiles * q.zm * kTileSize * kTileSize * c8 : 0);
  q.o_done = take(q.sgroups > 1 ? (size_t)q.ntiles * q.zm * sizeof(int) : 0);
  q.total = o;
  return q;
}

inline int check_geometry(const pty_problem_t* p, const int32_t* pos, const int32_t* seq) {
  for (int i = 0; i < p->n_sequence; ++i) {
    const int s = seq[i];
    if (s < 0 || s >= p->n_positions) return PTY_ERR_POSITION;
    const int y = pos[2 * s], x = pos[2 * s + 1];
    if (y < 0 || x < 0 || y + p->window > p->obj_ny || x + p->window > p->obj_nx) return PTY_ERR_POSITION;
  }
  return PTY_OK;
}

template <typename T>
T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

inline int cuda_status() { return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA; }

template <typename K>
int set_smem(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess
             ? PTY_OK
             : PTY_ERR_CUDA;
}


// Workspace of the multislice_core-style entry points (pty_multislice,
// pty_multislice_grads, pty_scatteradd): caller-given windows in the reference layout.
struct MsPlan {
  int W, B, Z, Mp, Mo, Ny, Nx, zm, ntx, nty, ntiles;
  size_t o_tw, o_prop, o_prop_edge, o_mask, o_mask_sc, o_pyx, o_probe_b, o_obl, o_stack, o_gbuf, o_gsum;
  size_t o_fprobe, o_grad, o_lists, o_counts, o_pos, o_seq, o_corr, o_err, o_parts, total;
};

inline MsPlan make_ms_plan(int W, int B, int Z, int Mp, int Mo, int Ny, int Nx) {
  MsPlan q{};
  q.W = W;
  q.B = B;
  q.Z = Z;
  q.Mp = Mp;
  q.Mo = Mo;
  q.Ny = Ny;
  q.Nx = Nx;
  q.zm = Z * Mo;
  q.ntx = (Nx + kTileSize - 1) / kTileSize;
  q.nty = (Ny + kTileSize - 1) / kTileSize;
  q.ntiles = q.ntx * q.nty;
  const size_t WW = (size_t)W * W, c8 = sizeof(float2);
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align_up(bytes); return r; };
  q.o_tw = take(tw_count(W) * c8);
  q.o_prop = take(WW * c8);
  q.o_prop_edge = take(WW * c8);
  q.o_mask = take(WW * sizeof(float));
  q.o_mask_sc = take(WW * sizeof(float));
  q.o_pyx = take(2 * (size_t)W * c8);
  q.o_probe_b = take((size_t)B * Mp * WW * c8);
  q.o_obl = take((size_t)B * q.zm * WW * c8);
  q.o_stack = take((size_t)B * Z * Mp * Mo * WW * c8);
  q.o_gbuf = take((size_t)B * Mp * Mo * WW * c8);
  q.o_gsum = take((size_t)B * q.zm * Mp * WW * c8);   // one contribution window per probe mode
  q.o_fprobe = take((size_t)B * Mp * WW * c8);
  q.o_grad = take((size_t)q.zm * Ny * Nx * c8);
  q.o_lists = take((size_t)q.ntiles * B * sizeof(int));
  q.o_counts = take((size_t)q.ntiles * sizeof(int));
  q.o_pos = take((size_t)B * 2 * sizeof(int));
  q.o_seq = take((size_t)B * sizeof(int));
  q.o_corr = take((size_t)B * 2 * sizeof(float));
  q.o_err = take(sizeof(int));
  q.o_parts = take((size_t)B * (2 + 2 * Mp) * sizeof(double));
  q.total = o;
  return q;
}

// Kernel classes reported by the launch profiler (pty_profile_begin / pty_profile_end).
enum KernelId : int {
  KID_TWIDDLES = 0, KID_TABLES, KID_PROBE_FFT, KID_OBJ_TO_SLICES, KID_OBJECT_WINDOWS, KID_FUSED,
  KID_GRAD_WINDOWS, KID_TILE_LISTS, KID_SCATTER, KID_PROBE_PARTIAL, KID_SLICES_TO_OBJ, KID_PROBE_FINAL,
  KID_FINALIZE, KID_FFT2, KID_LAYOUT, KID_CLEAN_TABLES, KID_CLEAN_X, KID_CLEAN_Y, KID_CLEAN_XI,
  KID_VEC, KID_SCALAR, KID_ACCEPT, KID_ORTHO, KID_DFT_TABLES, KID_DFT_GEMM, KID_ELEMENTWISE, KID_NN, KID_PROBE_SPECTRUM, KID_PROBE_SHIFT, KID_COUNT
};

// Records an event on `st` before a launch of kernel class `id` while profiling is on
// (id < 0 closes the last interval on that stream). No-op otherwise.
void prof_mark(cudaStream_t st, int id);
// True while the launch profiler records. The batch loops then issue every launch on the
// caller's stream, one after another, so that each profiled interval is one kernel running
// alone (the durations the roofline is computed from).
bool prof_active();
// Two more streams and four events for the caller's device, created on first use by each
// host thread and kept until the thread exits.
struct SideStream {
  cudaStream_t s = nullptr, s2 = nullptr;
  cudaEvent_t ev[4] = {};
};
int side_stream(SideStream** out);

// Launch paths, instantiated in path_w64.cu / path_w128.cu and specialised for W = 256 in
// path_w256.cu.
template <int W>
int run_path(const pty_problem_t* p, const Plan& q, const float2* obj, const float2* probe,
             const float* measured, double* loss_sse, float2* object_grad, float2* probe_grad,
             float* pos_grad, float* patterns, void* ws, cudaStream_t st);

template <int W>
int run_forward(const pty_problem_t* p, const Plan& q, const float2* obj, const float2* probe,
                const float* measured, double* loss_sse, void* ws, cudaStream_t st);

template <int W>
int run_backward(const pty_problem_t* p, const Plan& q, double* loss_sse, float2* object_grad,
                 float2* probe_grad, float* pos_grad, void* ws, cudaStream_t st);

template <>
int run_path<256>(const pty_problem_t*, const Plan&, const float2*, const float2*, const float*, double*, float2*,
                  float2*, float*, float*, void*, cudaStream_t);
template <>
int run_forward<256>(const pty_problem_t*, const Plan&, const float2*, const float2*, const float*, double*, void*,
                     cudaStream_t);
template <>
int run_backward<256>(const pty_problem_t*, const Plan&, double*, float2*, float2*, float*, void*, cudaStream_t);

// multislice_core-style entry points (reference layouts, caller-given windows)
template <int W>
int run_ms_forward(const MsPlan& q, const float2* probe_b, const float2* obj_b, const float2* propagator,
                   float edge_mult, float2* waves, float2* exit_wave, void* ws, cudaStream_t st);

template <int W>
int run_ms_grads(const MsPlan& q, const float2* d_exit, const float2* waves, const float2* obj_b,
                 const float2* propagator, float edge_mult, const float* mask_clean, int step_obj,
                 float2* object_grad, float2* probe_grad, void* ws, cudaStream_t st);

template <int W>
int run_scatteradd(const MsPlan& q, float2* full, const float2* chop, void* ws, cudaStream_t st);

// one-pass propagation step (tab, tab_stride apart per group of nper windows, conj, scale) or
// band limit (rtab: real mask, unscaled; scale folds the inverse's 1/W^2) of nwin natural 256-px
// windows in place; tw holds the 128-point twiddle tables
int layered_step256(float2* x, long long nwin, const float2* tab, size_t tab_stride, int nper, int conj, float scale,
                    const float* rtab, const float2* tw, cudaStream_t st);
// one-pass forward step (slice, stack, propagation) of Bn positions' 256-px windows
int layered_fwd256(const float2* pin, size_t pin_stride, float2* psi, float2* stack, const float2* ob, int z, int Z,
                   int Mp, int Mo, int Bn, const float2* tab, size_t tab_stride, float scale, const float2* tw,
                   cudaStream_t st);

template <int W>
int run_fft2(const float2* in, float2* out, int batch, int inverse, int shift, float2* tw, cudaStream_t st,
             int build_tw = 1);   // build_tw = 0: tw already holds this window's twiddles
template <>
int run_fft2<256>(const float2*, float2*, int, int, int, float2*, cudaStream_t, int);

}  // namespace pty

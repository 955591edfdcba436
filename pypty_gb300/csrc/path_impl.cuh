// Launch sequence of the loss-and-gradient path for window size W, as composable stages:
//   prepare   twiddles, tables, probe spectrum, slice-major object, error word
//   windows   band-limited object windows of one batch
//   fused     the fused multislice kernel of one batch (whole pass, forward half or adjoint half)
//   gradients band limit of the gradient windows, deterministic scatter, probe partial sums
//   finalize  object-gradient transpose, probe gradient, loss / sse / position gradient
// pty_loss_and_direction runs them batch by batch; pty_forward / pty_backward split one batch
// holding every position between the two calls. Instantiated once per W in path_w64.cu /
// path_w128.cu so the two compile in parallel.
#pragma once
#include "plan.h"
#include "ptycho_kernels.cuh"

namespace pty {

static_assert(TS == kTileSize, "scatter tile size of the kernels and the plan");

template <int W>
struct Path {
  using G = Geo<W>;
  static constexpr int T = G::T;
  static constexpr size_t WW = (size_t)W * W;
  const pty_problem_t* p;
  const Plan& q;
  void* ws;
  cudaStream_t st;
  cudaStream_t side;   // stream of windows() and gradients(): st, or a second stream when overlapping
  cudaStream_t fst;    // stream of fused(): st, or alternately st and a third stream when overlapping
  float2* tw;
  TableArgs ta{};
  // One slice and one object mode: the reference's (Ny, Nx, Z, Mo) layout is the slice layout,
  // so the windows read the caller's object and the scatter writes the caller's gradient
  // directly (no transposes).
  const float2* obj_src = nullptr;
  float2* grad_out = nullptr;
  bool lists_done = false;         // batch 0's tile lists were built by prepare()
  cudaStream_t pbranch = nullptr;  // one batch: the probe-gradient sum runs here, beside the
                                   // object-gradient band limit and scatter
  cudaStream_t sbranch = nullptr;  // one batch: the FP64 scalars and position gradient

  Path(const pty_problem_t* p_, const Plan& q_, void* ws_, cudaStream_t st_)
      : p(p_), q(q_), ws(ws_), st(st_), side(st_), fst(st_) {
    tw = at<float2>(ws, q.o_tw);
    ta.pyx = at<float2>(ws, q.o_pyx);
    ta.mask = at<float>(ws, q.o_mask);
    ta.mask_sc = at<float>(ws, q.o_mask_sc);
    ta.prop = at<float2>(ws, q.o_prop);
    ta.prop_edge = at<float2>(ws, q.o_prop_edge);
    ta.sx = at<float>(ws, q.o_sx);
    ta.sy = at<float>(ws, q.o_sy);
    ta.px = p->pixel_size_x;
    ta.py = p->pixel_size_y;
    ta.cutoff = p->damping_cutoff;
    ta.rolloff = p->smooth_rolloff;
    ta.distance = p->slice_distance;
    ta.wavelength = p->wavelength;
    ta.edge_mult = p->edge_mult;
    ta.use_edge = (p->edge_mult > 1.0f && q.Z > 1) ? 1 : 0;
    ta.tw = tw;   // tables_kernel writes the twiddle tables too
  }

  static int attributes() {
    const size_t smem = Smem<W>::bytes;
    int rc;
    if ((rc = set_smem(probe_fft_kernel<W>, smem)) || (rc = set_smem(object_windows_kernel<W>, smem)) ||
        (rc = set_smem(fused_multislice_kernel<W, 0>, FusedSmem<W>::bytes)) ||
        (rc = set_smem(fused_multislice_kernel<W, 1>, FusedSmem<W>::bytes)) ||
        (rc = set_smem(grad_windows_kernel<W>, smem)) || (rc = set_smem(probe_final_kernel<W>, smem)))
      return rc;
    return PTY_OK;
  }

  // Independent launches of a call's ends (the probe spectrum beside the tile lists and the
  // object transpose; the probe-gradient transform beside the object-gradient transpose and the
  // scalars) run on side streams: fork() makes the side stream wait for st, join() makes st wait
  // for it. While the launch profiler records, everything stays on st.
  cudaStream_t fork() {
    SideStream* sd = nullptr;
    if (prof_active() || side_stream(&sd) != PTY_OK) return st;
    if (cudaEventRecord(sd->ev[0], st) != cudaSuccess || cudaStreamWaitEvent(sd->s, sd->ev[0], 0) != cudaSuccess)
      return st;
    return sd->s;
  }
  // a second branch (the stream of the second fused kernel when batches overlap, free otherwise)
  cudaStream_t fork2() {
    SideStream* sd = nullptr;
    if (prof_active() || side_stream(&sd) != PTY_OK) return st;
    if (cudaEventRecord(sd->ev[2], st) != cudaSuccess || cudaStreamWaitEvent(sd->s2, sd->ev[2], 0) != cudaSuccess)
      return st;
    return sd->s2;
  }
  int join(cudaStream_t other) {
    if (other == st) return PTY_OK;
    SideStream* sd = nullptr;
    if (side_stream(&sd) != PTY_OK) return PTY_ERR_CUDA;
    prof_mark(other, -1);
    if (cudaEventRecord(sd->ev[1], other) != cudaSuccess || cudaStreamWaitEvent(st, sd->ev[1], 0) != cudaSuccess)
      return PTY_ERR_CUDA;
    return PTY_OK;
  }

  // The tables (with the twiddles) first; then the probe spectrum on a branch beside the tile
  // lists (early_lists: the call has one batch and object gradients, so batch 0's lists, which
  // depend only on the geometry, are built here) and the object transpose.
  int prepare(const float2* obj, const float2* probe, bool early_lists = false) {
    int rc = attributes();
    if (rc) return rc;
    prof_mark(st, KID_TABLES);
    tables_kernel<W><<<(unsigned)((WW + 255) / 256), 256, 0, st>>>(ta);   // with the twiddles
    if (q.per_step)
      launch_step_props<W>(ta.mask, p->slice_distances, q.Z - 1, ta.px, ta.py, ta.wavelength, ta.edge_mult,
                           ta.use_edge, 0.0f, 0.0f, at<float2>(ws, q.o_steps), st);
    cudaStream_t fs = fork();
    if (p->probe_shift) {
      prof_mark(fs, KID_PROBE_FFT);
      probe_fft_kernel<W><<<q.Mp, T, Smem<W>::bytes, fs>>>(probe, q.Mp, tw, at<float2>(ws, q.o_probe_f));
    }
    if (q.sgroups > 1 &&
        cudaMemsetAsync(at<int>(ws, q.o_done), 0, (size_t)q.ntiles * q.zm * sizeof(int), st) != cudaSuccess)
      return PTY_ERR_CUDA;
    if (early_lists && q.nbatch == 1 && p->step_obj) {
      prof_mark(st, KID_TILE_LISTS);
      tile_lists_kernel<<<q.ntiles, 256, 0, st>>>(at<int>(ws, q.o_pos), seq_of(0), batch_count(0), W, q.ntx,
                                                  at<int>(ws, q.o_lists), at<int>(ws, q.o_counts));
      lists_done = true;
    }
    const int nyx = q.Ny * q.Nx;
    if (q.zm == 1) {
      obj_src = obj;
    } else {
      prof_mark(st, KID_OBJ_TO_SLICES);
      obj_to_slices_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(obj, at<float2>(ws, q.o_obj), nyx, q.zm);
      obj_src = at<float2>(ws, q.o_obj);
    }
    if (cudaMemsetAsync(at<int>(ws, q.o_err), 0, sizeof(int), st) != cudaSuccess) return PTY_ERR_CUDA;
    if ((rc = join(fs))) return rc;
    return cuda_status();
  }

  int batch_count(int ib) const { return std::min(q.Bb, q.nseq - ib * q.Bb); }
  float2* obl(int ib) const { return at<float2>(ws, q.o_obl + (size_t)(ib % q.nbuf) * q.s_obl); }
  float2* gsum(int ib) const { return at<float2>(ws, q.o_gsum + (size_t)(ib % q.nbuf) * q.s_gsum); }
  float2* fprobe(int ib) const { return at<float2>(ws, q.o_fprobe + (size_t)(ib % q.nbuf) * q.s_fprobe); }
  float2* stack(int ib) const { return at<float2>(ws, q.o_stack + (size_t)(ib % q.nbuf) * q.s_stack); }
  const int* seq_of(int ib) const { return at<int>(ws, q.o_seq) + ib * q.Bb; }

  int windows(int ib) {
    WindowArgs wa{};
    wa.obj = obj_src;
    wa.pos = at<int>(ws, q.o_pos);
    wa.seq = seq_of(ib);
    wa.mask_sc = ta.mask_sc;
    wa.tw = tw;
    wa.out = obl(ib);
    wa.Ny = q.Ny;
    wa.Nx = q.Nx;
    wa.zm = q.zm;
    prof_mark(side, KID_OBJECT_WINDOWS);
    object_windows_kernel<W><<<(unsigned)(batch_count(ib) * q.zm), T, Smem<W>::bytes, side>>>(wa);
    return cuda_status();
  }

  // phase 0: the whole pass; 1: forward half (keeps the wave stack and dL/d(exit wave));
  // 2: adjoint half
  int fused(int ib, int phase, const float2* probe, const float* measured, float* patterns) {
    const int Bn = batch_count(ib);
    const int s0 = ib * q.Bb;
    const bool simulate = patterns != nullptr;
    FusedArgs fa{};
    fa.Z = q.Z;
    fa.Mp = q.Mp;
    fa.Mo = q.Mo;
    fa.algorithm = p->algorithm;
    fa.step_obj = p->step_obj && !simulate;
    fa.step_probe = p->step_probe && !simulate;
    fa.step_pos = p->step_pos && !simulate;
    fa.probe_shift = p->probe_shift ? 1 : 0;
    fa.simulate = simulate ? 1 : 0;
    fa.use_edge = ta.use_edge;
    fa.phase = phase;
    fa.loss_weight = p->loss_weight;
    fa.probe = probe;
    fa.probe_f = at<float2>(ws, q.o_probe_f);
    fa.obl = obl(ib);
    fa.prop = ta.prop;
    fa.prop_edge = ta.prop_edge;
    fa.pyx = ta.pyx;
    fa.use_sep = (p->smooth_rolloff == 0.0f && !q.per_step) ? 1 : 0;
    fa.mask_bin = p->smooth_rolloff == 0.0f ? 1 : 0;   // tables_kernel's mask is then 0/1
    fa.prop_steps = q.per_step ? at<float2>(ws, q.o_steps) : nullptr;
    fa.mask = ta.mask;
    fa.sx = ta.sx;
    fa.sy = ta.sy;
    fa.corr = at<float>(ws, q.o_corr);
    fa.seq = seq_of(ib);
    fa.measured = measured;
    fa.tw = tw;
    fa.stack = stack(ib);
    fa.gsum = gsum(ib);
    fa.fprobe = fprobe(ib);
    fa.gbuf = at<float2>(ws, q.o_gbuf);
    fa.loss_part = at<double>(ws, q.o_loss_part) + 2 * (size_t)s0;
    fa.pos_part = at<double>(ws, q.o_pos_part) + 2 * (size_t)s0 * q.Mp;
    fa.sim_out = simulate ? patterns + (size_t)s0 * WW : nullptr;
    fa.err = at<int>(ws, q.o_err);
    const int nmodes = q.Mp * q.Mo;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(Bn * nmodes));
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = FusedSmem<W>::bytes;
    cfg.stream = fst;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)nmodes;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    prof_mark(fst, KID_FUSED);
    const cudaError_t e = fa.phase == 0 ? cudaLaunchKernelEx(&cfg, fused_multislice_kernel<W, 0>, fa)
                                        : cudaLaunchKernelEx(&cfg, fused_multislice_kernel<W, 1>, fa);
    if (e != cudaSuccess) return PTY_ERR_CUDA;
    return cuda_status();
  }

  int gradients(int ib) {
    const int Bn = batch_count(ib);
    const int* seq_b = seq_of(ib);
    const int* d_pos = at<int>(ws, q.o_pos);
    if (p->step_obj) {
      float2* gs = gsum(ib);
      float2* gdst = grad_out ? grad_out : at<float2>(ws, q.o_grad);
      prof_mark(side, KID_GRAD_WINDOWS);
      grad_windows_kernel<W><<<(unsigned)(Bn * q.zm), T, Smem<W>::bytes, side>>>(gs, ta.mask_sc, tw, q.Mp);
      int* lists = at<int>(ws, q.o_lists);
      int* counts = at<int>(ws, q.o_counts);
      if (!lists_done) {
        prof_mark(side, KID_TILE_LISTS);
        tile_lists_kernel<<<q.ntiles, 256, 0, side>>>(d_pos, seq_b, Bn, W, q.ntx, lists, counts);
      }
      prof_mark(side, KID_SCATTER);
      // sgroups > 1: the last run block of each tile adds the runs in order (counters in o_done,
      // zeroed by prepare() and by each merging block)
      float2* scpart = q.sgroups > 1 ? at<float2>(ws, q.o_scpart) : nullptr;
      int* done = q.sgroups > 1 ? at<int>(ws, q.o_done) : nullptr;
      scatter_tiles_kernel<<<dim3(q.ntiles, q.zm, q.sgroups), dim3(32, 8), 0, side>>>(
          gs, d_pos, seq_b, lists, counts, gdst, Bn, W, q.Ny, q.Nx, q.ntx, q.zm, ib > 0 ? 1 : 0, q.sgroups, scpart,
          q.Mp, done);
    }
    if (p->step_probe) {
      const int nch = (Bn + q.chunk - 1) / q.chunk;
      cudaStream_t ps = pbranch ? pbranch : side;
      // chunks beyond this batch's count keep their previous value: the first batch has the
      // largest count, so every chunk read later was written
      prof_mark(ps, KID_PROBE_PARTIAL);
      probe_partial_kernel<<<dim3((unsigned)((WW + 255) / 256), q.Mp, nch), 256, 0, ps>>>(
          fprobe(ib), at<float2>(ws, q.o_partial), Bn, q.Mp, (int)WW, q.chunk, ib > 0 ? 1 : 0);
    }
    return cuda_status();
  }

  // with_grads = false: only loss and sse
  int finalize(double* loss_sse, float2* object_grad, float2* probe_grad, float* pos_grad, bool with_grads) {
    const int nyx = q.Ny * q.Nx;
    const bool do_pos = with_grads && p->step_pos;
    cudaStream_t fs = pbranch ? pbranch : st;
    if (with_grads) {
      if (p->step_probe) {
        if (!pbranch) fs = fork();
        prof_mark(fs, KID_PROBE_FINAL);
        // the chunk sum over the GPU first (into chunk 0), then one block per mode transforms
        probe_chunks_kernel<<<dim3((unsigned)((WW + 255) / 256), q.Mp), 256, 0, fs>>>(at<float2>(ws, q.o_partial),
                                                                                     q.nchunk, q.Mp, (int)WW);
        probe_final_kernel<W><<<q.Mp, T, Smem<W>::bytes, fs>>>(at<float2>(ws, q.o_partial), 1, q.Mp,
                                                               ta.mask_sc, tw, probe_grad);
      } else if (probe_grad) {
        cudaMemsetAsync(probe_grad, 0, WW * q.Mp * sizeof(float2), st);
      }
      if (p->step_obj) {
        if (!grad_out) {
          prof_mark(st, KID_SLICES_TO_OBJ);
          slices_to_obj_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(at<float2>(ws, q.o_grad), object_grad, nyx,
                                                                  q.zm);
        }
      } else if (object_grad) {
        cudaMemsetAsync(object_grad, 0, (size_t)nyx * q.zm * sizeof(float2), st);
      }
    }
    // the scalars depend on the fused kernels alone: beside the scatter when there is a branch
    cudaStream_t ss = sbranch ? sbranch : st;
    if (with_grads && pos_grad) cudaMemsetAsync(pos_grad, 0, (size_t)q.N * 2 * sizeof(float), ss);
    prof_mark(ss, KID_FINALIZE);
    finalize_scalars_kernel<<<1, 256, 0, ss>>>(at<double>(ws, q.o_loss_part), at<double>(ws, q.o_pos_part),
                                                at<int>(ws, q.o_seq), q.nseq, q.Mp, W, (double)p->loss_weight,
                                                do_pos ? 1 : 0, at<int>(ws, q.o_err), loss_sse, pos_grad);
    int rc = join(fs);
    if (!rc && sbranch) rc = join(sbranch);
    if (rc) return rc;
    prof_mark(st, -1);
    return cuda_status();
  }
};

// The batch loop on three streams (double-buffered windows, wave stacks, gradient windows
// and shifted probes, nbuf = 2). Batch ib's fused kernel runs on F(ib % 2) -- the caller's
// stream st for even batches, a second stream for odd ones -- so that one launch's last,
// partly filled wave overlaps the next launch's first; a third stream S extracts windows and
// scatters gradients:
//   S:    windows(0) | windows(1) gradients(0) | windows(2) gradients(1) | ...
//   F(0): fused(0)                             | fused(2)                | ...
//   F(1):              fused(1)                           | fused(3)     | ...
// Events (each wait is issued after the record it refers to and before that event's next
// record): ev[0] start, then fused(ib) done; ev[1] windows(ib) done; ev[2 + ib % 2]
// gradients(ib) done, which fused(ib + 2) waits for before it rewrites gradient buffer ib % 2.
// fused(ib + 2) follows fused(ib) on its stream, so its wave stack is free. windows(ib + 1)
// rewrites obl((ib + 1) % 2), last read by fused(ib - 1): S waited for that fused kernel before
// gradients(ib - 1). The scatter into the object gradient and the probe partial sums accumulate
// in batch order on S, so the results are those of the one-stream loop bit for bit. Each
// stage closes its launch-profiler interval on its own stream, so profiled durations exclude
// the waits between the streams.
template <int W>
int run_batches_overlapped(Path<W>& P, const float2* probe, const float* measured, float* patterns) {
  SideStream* sd = nullptr;
  int rc = side_stream(&sd);
  if (rc) return rc;
  cudaStream_t st = P.st, ss = sd->s;
  const cudaStream_t fs[2] = {st, sd->s2};
  cudaEvent_t ev_f = sd->ev[0], ev_w = sd->ev[1];
  auto ok = [](cudaError_t e) { return e == cudaSuccess; };
  prof_mark(st, -1);
  if (!ok(cudaEventRecord(ev_f, st)) || !ok(cudaStreamWaitEvent(ss, ev_f, 0)) ||
      !ok(cudaStreamWaitEvent(fs[1], ev_f, 0)))
    return PTY_ERR_CUDA;
  P.side = ss;
  const int n = P.q.nbatch;
  rc = P.windows(0);
  prof_mark(ss, -1);
  if (!rc && !ok(cudaEventRecord(ev_w, ss))) rc = PTY_ERR_CUDA;
  for (int ib = 0; ib < n && !rc; ++ib) {
    cudaStream_t f = fs[ib % 2];
    P.fst = f;
    if (!ok(cudaStreamWaitEvent(f, ev_w, 0))) { rc = PTY_ERR_CUDA; break; }
    if (!patterns && ib >= 2 && !ok(cudaStreamWaitEvent(f, sd->ev[2 + ib % 2], 0))) { rc = PTY_ERR_CUDA; break; }
    if ((rc = P.fused(ib, 0, probe, measured, patterns))) break;
    prof_mark(f, -1);
    if (!ok(cudaEventRecord(ev_f, f))) { rc = PTY_ERR_CUDA; break; }
    if (ib + 1 < n) {
      if ((rc = P.windows(ib + 1))) break;
      prof_mark(ss, -1);
      if (!ok(cudaEventRecord(ev_w, ss))) { rc = PTY_ERR_CUDA; break; }
    }
    if (!ok(cudaStreamWaitEvent(ss, ev_f, 0))) { rc = PTY_ERR_CUDA; break; }
    if (!patterns) {
      if ((rc = P.gradients(ib))) break;
      prof_mark(ss, -1);
      if (!ok(cudaEventRecord(sd->ev[2 + ib % 2], ss))) { rc = PTY_ERR_CUDA; break; }
    }
  }
  // join: S waited for every fused kernel it followed; everything queued on S and on the
  // second fused stream completes before st's next launch
  P.side = st;
  P.fst = st;
  cudaEvent_t ev_join = sd->ev[1];
  if (!ok(cudaEventRecord(ev_join, fs[1])) || !ok(cudaStreamWaitEvent(st, ev_join, 0))) return PTY_ERR_CUDA;
  if (!ok(cudaEventRecord(ev_join, ss)) || !ok(cudaStreamWaitEvent(st, ev_join, 0))) return PTY_ERR_CUDA;
  return rc;
}

template <int W>
int run_path(const pty_problem_t* p, const Plan& q, const float2* obj, const float2* probe,
             const float* measured, double* loss_sse, float2* object_grad, float2* probe_grad,
             float* pos_grad, float* patterns, void* ws, cudaStream_t st) {
  Path<W> P(p, q, ws, st);
  int rc = P.prepare(obj, probe, !patterns);
  if (rc) return rc;
  if (!patterns && q.zm == 1 && p->step_obj && object_grad) P.grad_out = object_grad;
  if (q.nbuf == 2 && !prof_active()) {
    if ((rc = run_batches_overlapped(P, probe, measured, patterns))) return rc;
  } else {
    for (int ib = 0; ib < q.nbatch; ++ib) {
      if ((rc = P.windows(ib)) || (rc = P.fused(ib, 0, probe, measured, patterns))) return rc;
      if (!patterns && q.nbatch == 1) {   // branches after the fused kernel
        P.pbranch = P.fork();
        P.sbranch = P.fork2();
      }
      if (!patterns && (rc = P.gradients(ib))) return rc;
    }
  }
  if (patterns) {
    prof_mark(st, -1);
    return cuda_status();
  }
  return P.finalize(loss_sse, object_grad, probe_grad, pos_grad, true);
}

template <int W>
int run_forward(const pty_problem_t* p, const Plan& q, const float2* obj, const float2* probe,
                const float* measured, double* loss_sse, void* ws, cudaStream_t st) {
  Path<W> P(p, q, ws, st);
  int rc = P.prepare(obj, probe);
  if (rc) return rc;
  if ((rc = P.windows(0)) || (rc = P.fused(0, 1, probe, measured, nullptr))) return rc;
  return P.finalize(loss_sse, nullptr, nullptr, nullptr, false);
}

template <int W>
int run_backward(const pty_problem_t* p, const Plan& q, double* loss_sse, float2* object_grad,
                 float2* probe_grad, float* pos_grad, void* ws, cudaStream_t st) {
  Path<W> P(p, q, ws, st);
  int rc = Path<W>::attributes();
  if (rc) return rc;
  if (q.zm == 1 && p->step_obj && object_grad) P.grad_out = object_grad;
  if ((rc = P.fused(0, 2, nullptr, nullptr, nullptr)) || (rc = P.gradients(0))) return rc;
  return P.finalize(loss_sse, object_grad, probe_grad, pos_grad, true);
}

// ------------------------------------------------------------------ multislice_core seams
// Shared launch of the fused kernel on caller-given windows (phase 3 or 4).
template <int W>
int ms_fused(const MsPlan& q, int phase, int step_obj, int step_probe, int use_edge, void* ws, cudaStream_t st) {
  const size_t WW = (size_t)W * W;
  if (set_smem(fused_multislice_kernel<W, 1>, FusedSmem<W>::bytes)) return PTY_ERR_CUDA;
  FusedArgs fa{};
  fa.Z = q.Z;
  fa.Mp = q.Mp;
  fa.Mo = q.Mo;
  fa.algorithm = 0;
  fa.step_obj = step_obj;
  fa.step_probe = step_probe;
  fa.step_pos = 0;
  fa.probe_shift = 0;
  fa.simulate = 0;
  fa.use_edge = use_edge;
  fa.phase = phase;
  fa.loss_weight = 1.0f;
  fa.probe_b = phase == 3 ? at<float2>(ws, q.o_probe_b) : nullptr;
  fa.exit_out = at<float2>(ws, q.o_gbuf);
  fa.obl = at<float2>(ws, q.o_obl);
  fa.prop = at<float2>(ws, q.o_prop);
  fa.prop_edge = at<float2>(ws, q.o_prop_edge);
  fa.pyx = at<float2>(ws, q.o_pyx);
  fa.use_sep = 0;
  fa.mask = at<float>(ws, q.o_mask);
  fa.sx = at<float>(ws, q.o_corr);     // not read without a probe shift
  fa.sy = at<float>(ws, q.o_corr);
  fa.corr = at<float>(ws, q.o_corr);
  fa.seq = at<int>(ws, q.o_seq);
  fa.tw = at<float2>(ws, q.o_tw);
  fa.stack = at<float2>(ws, q.o_stack);
  fa.gsum = at<float2>(ws, q.o_gsum);
  fa.fprobe = at<float2>(ws, q.o_fprobe);
  fa.gbuf = at<float2>(ws, q.o_gbuf);
  fa.loss_part = at<double>(ws, q.o_parts);
  fa.pos_part = at<double>(ws, q.o_parts) + 2 * (size_t)q.B;
  fa.err = at<int>(ws, q.o_err);
  const int nmodes = q.Mp * q.Mo;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)(q.B * nmodes));
  cfg.blockDim = dim3(Geo<W>::T);
  cfg.dynamicSmemBytes = FusedSmem<W>::bytes;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)nmodes;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  prof_mark(st, KID_FUSED);
  if (cudaLaunchKernelEx(&cfg, fused_multislice_kernel<W, 1>, fa) != cudaSuccess) return PTY_ERR_CUDA;
  return cuda_status();
}

template <int W>
int ms_tables(const MsPlan& q, const float2* propagator, float edge_mult, const float* mask_clean, void* ws,
              cudaStream_t st) {
  const size_t WW = (size_t)W * W;
  int rc = Path<W>::attributes();
  if (rc) return rc;
  prof_mark(st, KID_TWIDDLES);
  build_twiddles_kernel<W><<<1, 256, 0, st>>>(at<float2>(ws, q.o_tw));
  prof_mark(st, KID_TABLES);
  external_tables_kernel<W><<<(unsigned)((WW + 255) / 256), 256, 0, st>>>(
      propagator, mask_clean, edge_mult, (edge_mult > 1.0f && q.Z > 1) ? 1 : 0, at<float2>(ws, q.o_prop),
      at<float2>(ws, q.o_prop_edge), at<float>(ws, q.o_mask), at<float>(ws, q.o_mask_sc), at<float2>(ws, q.o_pyx));
  if (cudaMemsetAsync(at<float>(ws, q.o_corr), 0, (size_t)q.B * 2 * sizeof(float), st) != cudaSuccess ||
      cudaMemsetAsync(at<int>(ws, q.o_err), 0, sizeof(int), st) != cudaSuccess)
    return PTY_ERR_CUDA;
  return cuda_status();
}

template <int W>
int run_ms_forward(const MsPlan& q, const float2* probe_b, const float2* obj_b, const float2* propagator,
                   float edge_mult, float2* waves, float2* exit_wave, void* ws, cudaStream_t st) {
  constexpr int T = Geo<W>::T;
  int rc = ms_tables<W>(q, propagator, edge_mult, nullptr, ws, st);
  if (rc) return rc;
  prof_mark(st, KID_LAYOUT);
  ref_to_native_kernel<W><<<q.B * q.Mp, T, 0, st>>>(probe_b, at<float2>(ws, q.o_probe_b), q.Mp);
  ref_to_native_kernel<W><<<q.B * q.zm, T, 0, st>>>(obj_b, at<float2>(ws, q.o_obl), q.zm);
  if ((rc = ms_fused<W>(q, 3, 1, 0, (edge_mult > 1.0f && q.Z > 1) ? 1 : 0, ws, st))) return rc;
  prof_mark(st, KID_LAYOUT);
  native_to_ref_kernel<W><<<q.B * q.Z * q.Mp * q.Mo, T, 0, st>>>(at<float2>(ws, q.o_stack), waves,
                                                                q.Z * q.Mp * q.Mo);
  native_to_ref_kernel<W><<<q.B * q.Mp * q.Mo, T, 0, st>>>(at<float2>(ws, q.o_gbuf), exit_wave, q.Mp * q.Mo);
  prof_mark(st, -1);
  return cuda_status();
}

template <int W>
int run_ms_grads(const MsPlan& q, const float2* d_exit, const float2* waves, const float2* obj_b,
                 const float2* propagator, float edge_mult, const float* mask_clean, int step_obj,
                 float2* object_grad, float2* probe_grad, void* ws, cudaStream_t st) {
  constexpr int T = Geo<W>::T;
  const size_t WW = (size_t)W * W;
  int rc = ms_tables<W>(q, propagator, edge_mult, mask_clean, ws, st);
  if (rc) return rc;
  prof_mark(st, KID_LAYOUT);
  ref_to_native_kernel<W><<<q.B * q.Mp * q.Mo, T, 0, st>>>(d_exit, at<float2>(ws, q.o_gbuf), q.Mp * q.Mo);
  ref_to_native_kernel<W><<<q.B * q.zm, T, 0, st>>>(obj_b, at<float2>(ws, q.o_obl), q.zm);
  if (step_obj)
    ref_to_native_kernel<W><<<q.B * q.Z * q.Mp * q.Mo, T, 0, st>>>(waves, at<float2>(ws, q.o_stack),
                                                                  q.Z * q.Mp * q.Mo);
  if ((rc = ms_fused<W>(q, 4, step_obj, probe_grad != nullptr, (edge_mult > 1.0f && q.Z > 1) ? 1 : 0, ws, st)))
    return rc;
  if (step_obj) {
    float2* gs = at<float2>(ws, q.o_gsum);
    float2* grad = at<float2>(ws, q.o_grad);
    const int nyx = q.Ny * q.Nx;
    prof_mark(st, KID_GRAD_WINDOWS);
    grad_windows_kernel<W><<<(unsigned)(q.B * q.zm), T, Smem<W>::bytes, st>>>(gs, at<float>(ws, q.o_mask_sc),
                                                                            at<float2>(ws, q.o_tw), q.Mp);
    prof_mark(st, KID_OBJ_TO_SLICES);
    obj_to_slices_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(object_grad, grad, nyx, q.zm);
    prof_mark(st, KID_TILE_LISTS);
    tile_lists_kernel<<<q.ntiles, 256, 0, st>>>(at<int>(ws, q.o_pos), at<int>(ws, q.o_seq), q.B, W, q.ntx,
                                                 at<int>(ws, q.o_lists), at<int>(ws, q.o_counts));
    prof_mark(st, KID_SCATTER);
    scatter_tiles_kernel<<<dim3(q.ntiles, q.zm), dim3(32, 8), 0, st>>>(
        gs, at<int>(ws, q.o_pos), at<int>(ws, q.o_seq), at<int>(ws, q.o_lists), at<int>(ws, q.o_counts), grad, q.B,
        W, q.Ny, q.Nx, q.ntx, q.zm, 1, 1, nullptr, q.Mp);
    prof_mark(st, KID_SLICES_TO_OBJ);
    slices_to_obj_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(grad, object_grad, nyx, q.zm);
  }
  if (probe_grad) {
    prof_mark(st, KID_LAYOUT);
    native_to_ref_kernel<W><<<q.B * q.Mp, T, 0, st>>>(at<float2>(ws, q.o_fprobe), probe_grad, q.Mp);
  }
  (void)WW;
  prof_mark(st, -1);
  return cuda_status();
}

template <int W>
int run_scatteradd(const MsPlan& q, float2* full, const float2* chop, void* ws, cudaStream_t st) {
  const int WW = W * W;
  const int nyx = q.Ny * q.Nx;
  float2* planes = at<float2>(ws, q.o_gsum);
  float2* grad = at<float2>(ws, q.o_grad);
  prof_mark(st, KID_LAYOUT);
  ref_to_planes_kernel<<<(unsigned)(((size_t)q.B * WW + 255) / 256), 256, 0, st>>>(chop, planes, q.B, WW, q.zm);
  prof_mark(st, KID_OBJ_TO_SLICES);
  obj_to_slices_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(full, grad, nyx, q.zm);
  prof_mark(st, KID_TILE_LISTS);
  tile_lists_kernel<<<q.ntiles, 256, 0, st>>>(at<int>(ws, q.o_pos), at<int>(ws, q.o_seq), q.B, W, q.ntx,
                                               at<int>(ws, q.o_lists), at<int>(ws, q.o_counts));
  prof_mark(st, KID_SCATTER);
  scatter_tiles_kernel<<<dim3(q.ntiles, q.zm), dim3(32, 8), 0, st>>>(
      planes, at<int>(ws, q.o_pos), at<int>(ws, q.o_seq), at<int>(ws, q.o_lists), at<int>(ws, q.o_counts), grad, q.B,
      W, q.Ny, q.Nx, q.ntx, q.zm, 1);
  prof_mark(st, KID_SLICES_TO_OBJ);
  slices_to_obj_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(grad, full, nyx, q.zm);
  prof_mark(st, -1);
  return cuda_status();
}

template <int W>
int run_fft2(const float2* in, float2* out, int batch, int inverse, int shift, float2* tw, cudaStream_t st,
             int build_tw) {
  if (set_smem(fft2_batch_kernel<W>, Smem<W>::bytes)) return PTY_ERR_CUDA;
  if (build_tw) {
    prof_mark(st, KID_TWIDDLES);
    build_twiddles_kernel<W><<<1, 256, 0, st>>>(tw);
  }
  prof_mark(st, KID_FFT2);
  fft2_batch_kernel<W><<<batch, Geo<W>::T, Smem<W>::bytes, st>>>(in, out, inverse, shift, tw);
  prof_mark(st, -1);
  return cuda_status();
}

}  // namespace pty

// Launch paths for 256 x 256 windows: every window kernel runs as clusters of 4 blocks.
#include "plan.h"
#include "kernels256.cuh"

namespace pty {

namespace {

int set_attrs256() {
  int rc;
  if ((rc = set_smem(probe_fft256_kernel, Smem256::small)) || (rc = set_smem(object_windows256_kernel, Smem256::small)) ||
      (rc = set_smem(grad_windows256_kernel, Smem256::small)) || (rc = set_smem(probe_final256_kernel, Smem256::small)) ||
      (rc = set_smem(fused256_kernel<1>, Smem256::fused)) ||
      (rc = set_smem(fused256_kernel<2>, Smem256::fused)) ||
      (rc = set_smem(probe_spectrum256_kernel, Smem256::small)) ||
      (rc = set_smem(shifted_probes256_kernel, Smem256::small)) || (rc = set_smem(fft2_batch256_kernel, Smem256::small)))
    return rc;
  return PTY_OK;
}

template <typename K, typename... Args>
int launch4(K kernel, unsigned nclusters, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(nclusters * 4);
  cfg.blockDim = dim3(Geo256::T);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 4;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...) == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

struct Path256 {
  static constexpr size_t WW = 65536;
  const pty_problem_t* p;
  const Plan& q;
  void* ws;
  cudaStream_t st;
  float2* tw;
  TableArgs ta{};

  Path256(const pty_problem_t* p_, const Plan& q_, void* ws_, cudaStream_t st_) : p(p_), q(q_), ws(ws_), st(st_) {
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
  }

  int prepare(const float2* obj, const float2* probe) {
    int rc = set_attrs256();
    if (rc) return rc;
    prof_mark(st, KID_TWIDDLES);
    build_twiddles_kernel<128><<<1, 256, 0, st>>>(tw);
    prof_mark(st, KID_TABLES);
    tables_kernel<256><<<(unsigned)((WW + 255) / 256), 256, 0, st>>>(ta);
    if (q.per_step)
      launch_step_props<256>(ta.mask, p->slice_distances, q.Z - 1, ta.px, ta.py, ta.wavelength, ta.edge_mult,
                             ta.use_edge, 0.0f, 0.0f, at<float2>(ws, q.o_steps), st);
    if (p->probe_shift) {
      prof_mark(st, KID_PROBE_FFT);
      if ((rc = launch4(probe_fft256_kernel, q.Mp, Smem256::small, st, probe, q.Mp, (const float2*)tw,
                        at<float2>(ws, q.o_probe_f))))
        return rc;
    }
    const int nyx = q.Ny * q.Nx;
    prof_mark(st, KID_OBJ_TO_SLICES);
    obj_to_slices_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(obj, at<float2>(ws, q.o_obj), nyx, q.zm);
    if (cudaMemsetAsync(at<int>(ws, q.o_err), 0, sizeof(int), st) != cudaSuccess) return PTY_ERR_CUDA;
    return cuda_status();
  }

  int batch_count(int ib) const { return std::min(q.Bb, q.nseq - ib * q.Bb); }
  const int* seq_of(int ib) const { return at<int>(ws, q.o_seq) + ib * q.Bb; }

  int windows(int ib) {
    WindowArgs wa{};
    wa.obj = at<float2>(ws, q.o_obj);
    wa.pos = at<int>(ws, q.o_pos);
    wa.seq = seq_of(ib);
    wa.mask_sc = ta.mask_sc;
    wa.tw = tw;
    wa.out = at<float2>(ws, q.o_obl);
    wa.Ny = q.Ny;
    wa.Nx = q.Nx;
    wa.zm = q.zm;
    prof_mark(st, KID_OBJECT_WINDOWS);
    int rc = launch4(object_windows256_kernel, (unsigned)(batch_count(ib) * q.zm), Smem256::small, st, wa);
    return rc ? rc : cuda_status();
  }

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
    fa.obl = at<float2>(ws, q.o_obl);
    fa.prop = ta.prop;
    fa.prop_edge = ta.prop_edge;
    fa.pyx = ta.pyx;
    fa.use_sep = (p->smooth_rolloff == 0.0f && !q.per_step) ? 1 : 0;
    fa.prop_steps = q.per_step ? at<float2>(ws, q.o_steps) : nullptr;
    fa.mask = ta.mask;
    fa.sx = ta.sx;
    fa.sy = ta.sy;
    fa.corr = at<float>(ws, q.o_corr);
    fa.seq = seq_of(ib);
    fa.measured = measured;
    fa.tw = tw;
    fa.stack = at<float2>(ws, q.o_stack);
    fa.gsum = at<float2>(ws, q.o_gsum);
    fa.fprobe = at<float2>(ws, q.o_fprobe);
    fa.psi = at<float2>(ws, q.o_psi);
    fa.dldi = at<float>(ws, q.o_dldi);
    fa.pgr = at<float2>(ws, q.o_pgr);
    fa.ckpt = q.ckpt;
    fa.seg = at<float2>(ws, q.o_seg);
    fa.gpark = at<float2>(ws, q.o_gpark);
    fa.loss_part = at<double>(ws, q.o_loss_part) + 2 * (size_t)s0;
    fa.pos_part = at<double>(ws, q.o_pos_part) + 2 * (size_t)s0 * q.Mp;
    fa.sim_out = simulate ? patterns + (size_t)s0 * WW : nullptr;
    fa.err = at<int>(ws, q.o_err);
    // phase 0 = forward + loss (phase 1) then the adjoint (phase 2), through dldi
    int rc = PTY_OK;
    if (phase != 2) {
      prof_mark(st, KID_PROBE_SHIFT);
      rc = launch4(shifted_probes256_kernel, (unsigned)(Bn * q.Mp), Smem256::small, st, fa);
      prof_mark(st, KID_FUSED);
      if (!rc) rc = launch4(fused256_kernel<1>, (unsigned)Bn, Smem256::fused, st, fa);
    }
    prof_mark(st, KID_FUSED);
    if (!rc && phase != 1 && !simulate) {
      rc = launch4(fused256_kernel<2>, (unsigned)Bn, Smem256::fused, st, fa);
      if (!rc && (fa.step_probe || fa.step_pos)) {
        prof_mark(st, KID_PROBE_SPECTRUM);
        rc = launch4(probe_spectrum256_kernel, (unsigned)(Bn * q.Mp), Smem256::small, st, fa);
      }
    }
    return rc ? rc : cuda_status();
  }

  int gradients(int ib) {
    const int Bn = batch_count(ib);
    const int* seq_b = seq_of(ib);
    const int* d_pos = at<int>(ws, q.o_pos);
    int rc;
    if (p->step_obj) {
      float2* gs = at<float2>(ws, q.o_gsum);
      prof_mark(st, KID_GRAD_WINDOWS);
      if ((rc = launch4(grad_windows256_kernel, (unsigned)(Bn * q.zm), Smem256::small, st, gs,
                        (const float*)ta.mask_sc, (const float2*)tw)))
        return rc;
      int* lists = at<int>(ws, q.o_lists);
      int* counts = at<int>(ws, q.o_counts);
      prof_mark(st, KID_TILE_LISTS);
      tile_lists_kernel<<<q.ntiles, 256, 0, st>>>(d_pos, seq_b, Bn, 256, q.ntx, lists, counts);
      prof_mark(st, KID_SCATTER);
      scatter_tiles_kernel<<<dim3(q.ntiles, q.zm), dim3(32, 8), 0, st>>>(
          gs, d_pos, seq_b, lists, counts, at<float2>(ws, q.o_grad), Bn, 256, q.Ny, q.Nx, q.ntx, q.zm, ib > 0 ? 1 : 0);
    }
    if (p->step_probe) {
      const int nch = (Bn + q.chunk - 1) / q.chunk;
      prof_mark(st, KID_PROBE_PARTIAL);
      probe_partial_kernel<<<dim3((unsigned)((WW + 255) / 256), q.Mp, nch), 256, 0, st>>>(
          at<float2>(ws, q.o_fprobe), at<float2>(ws, q.o_partial), Bn, q.Mp, (int)WW, q.chunk, ib > 0 ? 1 : 0);
    }
    return cuda_status();
  }

  int finalize(double* loss_sse, float2* object_grad, float2* probe_grad, float* pos_grad, bool with_grads) {
    const int nyx = q.Ny * q.Nx;
    const bool do_pos = with_grads && p->step_pos;
    int rc;
    if (with_grads) {
      if (p->step_obj) {
        prof_mark(st, KID_SLICES_TO_OBJ);
        slices_to_obj_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(at<float2>(ws, q.o_grad), object_grad, nyx, q.zm);
      } else if (object_grad) {
        cudaMemsetAsync(object_grad, 0, (size_t)nyx * q.zm * sizeof(float2), st);
      }
      if (p->step_probe) {
        prof_mark(st, KID_PROBE_FINAL);
        if ((rc = launch4(probe_final256_kernel, (unsigned)q.Mp, Smem256::small, st,
                          (const float2*)at<float2>(ws, q.o_partial), q.nchunk, q.Mp, (const float*)ta.mask_sc,
                          (const float2*)tw, probe_grad)))
          return rc;
      } else if (probe_grad) {
        cudaMemsetAsync(probe_grad, 0, WW * q.Mp * sizeof(float2), st);
      }
      if (pos_grad) cudaMemsetAsync(pos_grad, 0, (size_t)q.N * 2 * sizeof(float), st);
    }
    prof_mark(st, KID_FINALIZE);
    finalize_scalars_kernel<<<1, 256, 0, st>>>(at<double>(ws, q.o_loss_part), at<double>(ws, q.o_pos_part),
                                                at<int>(ws, q.o_seq), q.nseq, q.Mp, 256, (double)p->loss_weight,
                                                do_pos ? 1 : 0, at<int>(ws, q.o_err), loss_sse, pos_grad);
    prof_mark(st, -1);
    return cuda_status();
  }
};

}  // namespace

template <>
int run_path<256>(const pty_problem_t* p, const Plan& q, const float2* obj, const float2* probe,
                  const float* measured, double* loss_sse, float2* object_grad, float2* probe_grad,
                  float* pos_grad, float* patterns, void* ws, cudaStream_t st) {
  Path256 P(p, q, ws, st);
  int rc = P.prepare(obj, probe);
  if (rc) return rc;
  for (int ib = 0; ib < q.nbatch; ++ib) {
    if ((rc = P.windows(ib)) || (rc = P.fused(ib, 0, probe, measured, patterns))) return rc;
    if (!patterns && (rc = P.gradients(ib))) return rc;
  }
  if (patterns) {
    prof_mark(st, -1);
    return cuda_status();
  }
  return P.finalize(loss_sse, object_grad, probe_grad, pos_grad, true);
}

template <>
int run_forward<256>(const pty_problem_t* p, const Plan& q, const float2* obj, const float2* probe,
                     const float* measured, double* loss_sse, void* ws, cudaStream_t st) {
  Path256 P(p, q, ws, st);
  int rc = P.prepare(obj, probe);
  if (rc) return rc;
  if ((rc = P.windows(0)) || (rc = P.fused(0, 1, probe, measured, nullptr))) return rc;
  return P.finalize(loss_sse, nullptr, nullptr, nullptr, false);
}

template <>
int run_backward<256>(const pty_problem_t* p, const Plan& q, double* loss_sse, float2* object_grad,
                      float2* probe_grad, float* pos_grad, void* ws, cudaStream_t st) {
  Path256 P(p, q, ws, st);
  int rc = set_attrs256();
  if (rc) return rc;
  if ((rc = P.fused(0, 2, nullptr, nullptr, nullptr)) || (rc = P.gradients(0))) return rc;
  return P.finalize(loss_sse, object_grad, probe_grad, pos_grad, true);
}

// one-pass propagation step / band limit of the layered path's 256-px windows (in place)
int layered_step256(float2* x, long long nwin, const float2* tab, size_t tab_stride, int nper, int conj, float scale,
                    const float* rtab, const float2* tw, cudaStream_t st) {
  if (set_smem(layered_step256_kernel, Smem256::small)) return PTY_ERR_CUDA;
  prof_mark(st, KID_FFT2);
  const int rc = launch4(layered_step256_kernel, (unsigned)nwin, Smem256::small, st, x, tab, tab_stride, nper, conj,
                         scale, rtab, tw);
  return rc ? rc : cuda_status();
}

// one-pass forward step of the layered path's 256-px windows
int layered_fwd256(const float2* pin, size_t pin_stride, float2* psi, float2* stack, const float2* ob, int z, int Z,
                   int Mp, int Mo, int Bn, const float2* tab, size_t tab_stride, float scale, const float2* tw,
                   cudaStream_t st) {
  if (set_smem(layered_fwd256_kernel, Smem256::small)) return PTY_ERR_CUDA;
  prof_mark(st, KID_FUSED);
  const int rc = launch4(layered_fwd256_kernel, (unsigned)(Bn * Mp * Mo), Smem256::small, st, pin, pin_stride, psi,
                         stack, ob, z, Z, Mp, Mo, tab, tab_stride, scale, tw);
  return rc ? rc : cuda_status();
}

template <>
int run_fft2<256>(const float2* in, float2* out, int batch, int inverse, int shift, float2* tw, cudaStream_t st,
                  int build_tw) {
  int rc = set_attrs256();
  if (rc) return rc;
  if (build_tw) {
    prof_mark(st, KID_TWIDDLES);
    build_twiddles_kernel<128><<<1, 256, 0, st>>>(tw);
  }
  prof_mark(st, KID_FFT2);
  if ((rc = launch4(fft2_batch256_kernel, (unsigned)batch, Smem256::small, st, in, out, inverse, shift,
                    (const float2*)tw)))
    return rc;
  prof_mark(st, -1);
  return cuda_status();
}

}  // namespace pty

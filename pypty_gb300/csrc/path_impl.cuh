// Launch sequence of one loss-and-gradient (or simulation) call for window size W.
// Instantiated once per W in path_w64.cu / path_w128.cu so the two compile in parallel.
#pragma once
#include "plan.h"
#include "ptycho_kernels.cuh"

namespace pty {

static_assert(TS == kTileSize, "scatter tile size of the kernels and the plan");

template <int W>
int run_path(const pty_problem_t* p, const Plan& q, const float2* obj, const float2* probe,
             const float* measured, double* loss_sse, float2* object_grad, float2* probe_grad,
             float* pos_grad, float* patterns, void* ws, cudaStream_t st) {
  using G = Geo<W>;
  constexpr int T = G::T;
  const size_t smem = Smem<W>::bytes;
  const size_t WW = (size_t)W * W;
  const bool simulate = patterns != nullptr;
  int rc;
  if ((rc = set_smem(probe_fft_kernel<W>, smem)) || (rc = set_smem(object_windows_kernel<W>, smem)) ||
      (rc = set_smem(fused_multislice_kernel<W>, FusedSmem<W>::bytes)) ||
      (rc = set_smem(grad_windows_kernel<W>, smem)) ||
      (rc = set_smem(probe_final_kernel<W>, smem)))
    return rc;

  float2* tw = at<float2>(ws, q.o_tw);
  prof_mark(st, KID_TWIDDLES);
  build_twiddles_kernel<W><<<1, 256, 0, st>>>(tw);
  TableArgs ta{};
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
  prof_mark(st, KID_TABLES);
  tables_kernel<W><<<(unsigned)((WW + 255) / 256), 256, 0, st>>>(ta);
  if (p->probe_shift) {
    prof_mark(st, KID_PROBE_FFT);
    probe_fft_kernel<W><<<q.Mp, T, smem, st>>>(probe, q.Mp, tw, at<float2>(ws, q.o_probe_f));
  }
  const int nyx = q.Ny * q.Nx;
  prof_mark(st, KID_OBJ_TO_SLICES);
  obj_to_slices_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(obj, at<float2>(ws, q.o_obj), nyx, q.zm);
  if (cudaMemsetAsync(at<int>(ws, q.o_err), 0, sizeof(int), st) != cudaSuccess) return PTY_ERR_CUDA;
  if ((rc = cuda_status())) return rc;

  const bool do_obj = p->step_obj && !simulate;
  const bool do_probe = p->step_probe && !simulate;
  const bool do_pos = p->step_pos && !simulate;
  const int* d_pos = at<int>(ws, q.o_pos);
  const int* d_seq = at<int>(ws, q.o_seq);
  const int nmodes = q.Mp * q.Mo;

  for (int ib = 0; ib < q.nbatch; ++ib) {
    const int s0 = ib * q.Bb;
    const int Bn = std::min(q.Bb, q.nseq - s0);
    const int* seq_b = d_seq + s0;
    WindowArgs wa{};
    wa.obj = at<float2>(ws, q.o_obj);
    wa.pos = d_pos;
    wa.seq = seq_b;
    wa.mask_sc = ta.mask_sc;
    wa.tw = tw;
    wa.out = at<float2>(ws, q.o_obl);
    wa.Ny = q.Ny;
    wa.Nx = q.Nx;
    wa.zm = q.zm;
    prof_mark(st, KID_OBJECT_WINDOWS);
    object_windows_kernel<W><<<(unsigned)(Bn * q.zm), T, smem, st>>>(wa);

    FusedArgs fa{};
    fa.Z = q.Z;
    fa.Mp = q.Mp;
    fa.Mo = q.Mo;
    fa.algorithm = p->algorithm;
    fa.step_obj = do_obj;
    fa.step_probe = do_probe;
    fa.step_pos = do_pos;
    fa.probe_shift = p->probe_shift ? 1 : 0;
    fa.simulate = simulate ? 1 : 0;
    fa.use_edge = ta.use_edge;
    fa.loss_weight = p->loss_weight;
    fa.probe = probe;
    fa.probe_f = at<float2>(ws, q.o_probe_f);
    fa.obl = wa.out;
    fa.prop = ta.prop;
    fa.prop_edge = ta.prop_edge;
    fa.pyx = ta.pyx;
    fa.use_sep = p->smooth_rolloff == 0.0f ? 1 : 0;
    fa.mask = ta.mask;
    fa.sx = ta.sx;
    fa.sy = ta.sy;
    fa.corr = at<float>(ws, q.o_corr);
    fa.seq = seq_b;
    fa.measured = measured;
    fa.tw = tw;
    fa.stack = at<float2>(ws, q.o_stack);
    fa.gsum = at<float2>(ws, q.o_gsum);
    fa.fprobe = at<float2>(ws, q.o_fprobe);
    fa.loss_part = at<double>(ws, q.o_loss_part) + 2 * (size_t)s0;
    fa.pos_part = at<double>(ws, q.o_pos_part) + 2 * (size_t)s0 * q.Mp;
    fa.sim_out = simulate ? patterns + (size_t)s0 * WW : nullptr;
    fa.err = at<int>(ws, q.o_err);

    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(Bn * nmodes));
    cfg.blockDim = dim3(T);
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
    if (cudaLaunchKernelEx(&cfg, fused_multislice_kernel<W>, fa) != cudaSuccess) return PTY_ERR_CUDA;

    if (do_obj) {
      prof_mark(st, KID_GRAD_WINDOWS);
      grad_windows_kernel<W><<<(unsigned)(Bn * q.zm), T, smem, st>>>(fa.gsum, ta.mask_sc, tw);
      int* lists = at<int>(ws, q.o_lists);
      int* counts = at<int>(ws, q.o_counts);
      prof_mark(st, KID_TILE_LISTS);
      tile_lists_kernel<<<q.ntiles, 256, 0, st>>>(d_pos, seq_b, Bn, W, q.ntx, lists, counts);
      prof_mark(st, KID_SCATTER);
      scatter_tiles_kernel<<<dim3(q.ntiles, q.zm), dim3(32, 8), 0, st>>>(
          fa.gsum, d_pos, seq_b, lists, counts, at<float2>(ws, q.o_grad), Bn, W, q.Ny, q.Nx, q.ntx, q.zm,
          ib > 0 ? 1 : 0);
    }
    if (do_probe) {
      const int nch = (Bn + q.chunk - 1) / q.chunk;
      // chunks beyond this batch's count keep their previous (or, in batch 0, no) value:
      // the first batch has the largest count, so every chunk read later was written
      prof_mark(st, KID_PROBE_PARTIAL);
      probe_partial_kernel<<<dim3((unsigned)((WW + 255) / 256), q.Mp, nch), 256, 0, st>>>(
          fa.fprobe, at<float2>(ws, q.o_partial), Bn, q.Mp, (int)WW, q.chunk, ib > 0 ? 1 : 0);
    }
    if ((rc = cuda_status())) return rc;
  }
  if (simulate) {
    prof_mark(st, -1);
    return cuda_status();
  }

  if (do_obj) {
    prof_mark(st, KID_SLICES_TO_OBJ);
    slices_to_obj_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(at<float2>(ws, q.o_grad), object_grad, nyx, q.zm);
  } else if (object_grad) {
    cudaMemsetAsync(object_grad, 0, (size_t)nyx * q.zm * sizeof(float2), st);
  }
  if (do_probe) {
    prof_mark(st, KID_PROBE_FINAL);
    probe_final_kernel<W><<<q.Mp, T, smem, st>>>(at<float2>(ws, q.o_partial), q.nchunk, q.Mp, ta.mask_sc, tw,
                                                 probe_grad);
  } else if (probe_grad) {
    cudaMemsetAsync(probe_grad, 0, WW * q.Mp * sizeof(float2), st);
  }
  if (pos_grad) cudaMemsetAsync(pos_grad, 0, (size_t)q.N * 2 * sizeof(float), st);
  prof_mark(st, KID_FINALIZE);
  finalize_scalars_kernel<<<1, 256, 0, st>>>(at<double>(ws, q.o_loss_part), at<double>(ws, q.o_pos_part), d_seq,
                                              q.nseq, q.Mp, W, (double)p->loss_weight, do_pos ? 1 : 0,
                                              at<int>(ws, q.o_err), loss_sse, pos_grad);
  prof_mark(st, -1);
  return cuda_status();
}

template <int W>
int run_fft2(const float2* in, float2* out, int batch, int inverse, int shift, float2* tw, cudaStream_t st) {
  if (set_smem(fft2_batch_kernel<W>, Smem<W>::bytes)) return PTY_ERR_CUDA;
  prof_mark(st, KID_TWIDDLES);
  build_twiddles_kernel<W><<<1, 256, 0, st>>>(tw);
  prof_mark(st, KID_FFT2);
  fft2_batch_kernel<W><<<batch, Geo<W>::T, Smem<W>::bytes, st>>>(in, out, inverse, shift, tw);
  prof_mark(st, -1);
  return cuda_status();
}

}  // namespace pty

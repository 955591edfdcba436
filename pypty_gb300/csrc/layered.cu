// loss_and_direction with a selectable window-DFT engine: the precision sweep of the path.
//
// The fused path (path_impl.cuh) keeps every window in registers between FFTs. This path
// runs the same algorithm (pypty/objective.py:283-742, pypty/multislice_core.py:9-200) as a
// sequence of batched passes over windows in natural row-major layout, so that every window
// DFT goes through one interchangeable engine:
//   PTY_DFT_FP32_FFT  the FP32 register FFT (pty_fft2),
//   PTY_DFT_BF16X3    dense GEMMs on the tensor cores in BF16x3 split precision
//                     (pty_fft2_bf16x3, dft_gemm.cu),
//   PTY_DFT_BF16X6    the same with three BF16 terms per operand (pty_fft2_bf16x6).
// Both inverses are normalised by 1/W^2 (numpy.fft.ifft2). Between the DFTs, small
// elementwise kernels apply the band-limit mask, propagator, probe-shift ramps, slice
// transmission, loss and their adjoints; the scatter-add of object-gradient windows, the
// probe-gradient chunk sums and the FP64 loss / position-gradient reductions are the fused
// path's deterministic kernels. Per batch of positions (pypty/objective.py:425-705):
//   gather + band-limit object windows; probe spectrum x ramp -> probe per position;
//   Z slices: stack conj(psi), psi *= O_z, psi = IDFT(DFT(psi) P);  far field, loss, dL/dPsi;
//   Z slices back: dO_z = sum_p stack * g, g *= conj(O_z), g = IDFT(DFT(g) conj P);
//   band-limit and scatter dO; probe-gradient spectra (shift adjoint, position gradient).
#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"
#include "ptycho_kernels.cuh"

extern "C" int pty_fft2(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse, int32_t shift,
                        void* workspace, size_t workspace_bytes, void* stream);
extern "C" int pty_fft2_workspace_bytes(int32_t window, size_t* bytes);
extern "C" int pty_fft2_bf16x3(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse,
                               void* workspace, size_t workspace_bytes, void* stream);
extern "C" int pty_fft2_bf16x3_workspace_bytes(int32_t batch, int32_t window, size_t* bytes);
extern "C" int pty_fft2_bf16x6(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse,
                               void* workspace, size_t workspace_bytes, void* stream);
extern "C" int pty_fft2_bf16x6_workspace_bytes(int32_t batch, int32_t window, size_t* bytes);

namespace pty {
namespace lay {

constexpr int EB = 256;   // threads per block of the elementwise kernels

// ------------------------------------------------------------------ elementwise kernels
// dst[b][k] = slices[k][y_b + .][x_b + .]   grid (WW / EB, zm, Bn)
__global__ void gather_kernel(const float2* __restrict__ slices, float2* __restrict__ dst, const int* __restrict__ pos,
                              const int* __restrict__ seq, int W, int Ny, int Nx, int zm) {
  const int u = blockIdx.x * EB + threadIdx.x, k = blockIdx.y, b = blockIdx.z;
  const int gi = seq[b];
  const int y = u / W, x = u % W;
  dst[((size_t)b * zm + k) * W * W + u] =
      slices[(size_t)k * Ny * Nx + (size_t)(pos[2 * gi] + y) * Nx + pos[2 * gi + 1] + x];
}

// x[w][u] *= mask[u]   grid (WW / EB, nwin)
__global__ void mask_kernel(float2* __restrict__ x, const float* __restrict__ mask, int WW) {
  const int u = blockIdx.x * EB + threadIdx.x;
  float2* p = x + (size_t)blockIdx.y * WW + u;
  *p = cscale(*p, mask[u]);
}

// x[w][u] *= scale * tab[u] (conj(tab) when conj)   grid (WW / EB, nwin)
__global__ void prop_kernel(float2* __restrict__ x, const float2* __restrict__ tab, int WW, int conj, float scale) {
  const int u = blockIdx.x * EB + threadIdx.x;
  float2* p = x + (size_t)blockIdx.y * WW + u;
  const float2 t = cscale(tab[u], scale);
  *p = conj ? cmulc(*p, t) : cmul(*p, t);
}

// exp(smx dx + smy dy) * mask (pypty/objective.py:308-313, 473), as the fused kernel
__device__ __forceinline__ float2 ramp(const float* sx, const float* sy, int ky, int kx, float mk, float dy, float dx) {
  const float th = __fadd_rn(__fmul_rn(__fmul_rn(sx[kx], mk), dx), __fmul_rn(__fmul_rn(sy[ky], mk), dy));
  float s, c;
  sincosf(th, &s, &c);
  return make_float2(c * mk, s * mk);
}

// spec[b][p][u] = probe_f[p][u] * ramp_b[u]   grid (WW / EB, Mp, Bn)
__global__ void probe_spec_kernel(float2* __restrict__ spec, const float2* __restrict__ pf, const float* __restrict__ sx,
                                  const float* __restrict__ sy, const float* __restrict__ mask,
                                  const float* __restrict__ corr, const int* __restrict__ seq, int W, int Mp) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y, b = blockIdx.z;
  const int gi = seq[b];
  const int ky = u / W, kx = u % W;
  const size_t WW = (size_t)W * W;
  spec[((size_t)b * Mp + p) * WW + u] =
      cmul(pf[(size_t)p * WW + u], ramp(sx, sy, ky, kx, mask[u], corr[2 * gi], corr[2 * gi + 1]));
}

// one forward slice (multislice_core.py:61-66): in = z == 0 ? probe_b[p] : psi[b][p][m];
// stack[b][z][p][m] = conj(in); psi[b][p][m] = in * O[b][z][m]   grid (WW / EB, Mp * Mo, Bn)
__global__ void fwd_slice_kernel(const float2* __restrict__ pb, size_t pb_stride, float2* __restrict__ psi,
                                 float2* __restrict__ stack, const float2* __restrict__ ob, int z, int Z, int Mp,
                                 int Mo, int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, pm = blockIdx.y, b = blockIdx.z;
  const int p = pm / Mo, m = pm % Mo;
  const size_t wi = ((size_t)b * Mp * Mo + pm) * WW + u;
  const float2 in = z == 0 ? pb[(size_t)b * pb_stride + (size_t)p * WW + u] : psi[wi];
  stack[(((size_t)b * Z + z) * Mp * Mo + pm) * WW + u] = cconj(in);
  psi[wi] = cmul(in, ob[(((size_t)b * Z + z) * Mo + m) * WW + u]);
}

// far field, loss and dL/dPsi (pypty/objective.py:501-597), one block per position: F is the
// unshifted spectrum of the exit waves; the detector pixel of u is the fftshifted index.
// On exit F holds dL/dPsi * W^2 * loss_weight (the W^2 cancels the normalised inverse).
__global__ void __launch_bounds__(1024) loss_kernel(float2* __restrict__ F, const float* __restrict__ mask,
                                                    const float* __restrict__ measured, const int* __restrict__ seq,
                                                    int W, int Mp, int Mo, int alg, float scale,
                                                    double* __restrict__ loss_part) {
  __shared__ double red[64];
  const int b = blockIdx.x, gi = seq[b];
  const int WW = W * W, nm = Mp * Mo;
  const float* meas = measured + (size_t)gi * WW;
  float2* f = F + (size_t)b * nm * WW;
  double lsum = 0.0, ssum = 0.0;
  for (int u = threadIdx.x; u < WW; u += blockDim.x) {
    const int ky = u / W, kx = u % W;
    const float mk = mask[u];
    float acc = 0.0f;
    for (int k = 0; k < nm; ++k) acc += cabs2(cscale(f[(size_t)k * WW + u], mk));
    const float I = nm == 1 ? acc : acc * (1.0f / (float)nm);
    const int didx = ((ky + W / 2) & (W - 1)) * W + ((kx + W / 2) & (W - 1));
    float d = loss_pixel(alg, I, meas[didx], lsum, ssum);
    if (nm > 1) d = d / (float)nm;
    for (int k = 0; k < nm; ++k) {
      float2* q = f + (size_t)k * WW + u;
      *q = cscale(cscale(cscale(*q, mk), d), scale);
    }
  }
  block_sum2(lsum, ssum, red);
  if (threadIdx.x == 0) {
    loss_part[2 * b] = lsum;
    loss_part[2 * b + 1] = ssum;
  }
}

// one adjoint slice (multislice_core.py:176-186): dO[b][z][m] = sum_p stack[b][z][p][m] g[b][p][m]
// (probes in ascending order), then g[b][p][m] *= conj(O[b][z][m])   grid (WW / EB, Mo, Bn)
__global__ void adj_slice_kernel(float2* __restrict__ g, const float2* __restrict__ stack,
                                 const float2* __restrict__ ob, float2* __restrict__ dob, int z, int Z, int Mp, int Mo,
                                 int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, m = blockIdx.y, b = blockIdx.z;
  const float2 o = ob[(((size_t)b * Z + z) * Mo + m) * WW + u];
  float2 acc = make_float2(0.f, 0.f);
  for (int p = 0; p < Mp; ++p) {
    const size_t wi = ((size_t)b * Mp * Mo + p * Mo + m) * WW + u;
    const float2 gv = g[wi];
    acc = cadd(acc, cmul(stack[(((size_t)b * Z + z) * Mp * Mo + p * Mo + m) * WW + u], gv));
    g[wi] = cmulc(gv, o);
  }
  dob[(((size_t)b * Z + z) * Mo + m) * WW + u] = acc;
}

// dL/d(probe_b)[b][p] = sum_m g[b][p][m]   grid (WW / EB, Mp, Bn)
__global__ void probe_sum_kernel(const float2* __restrict__ g, float2* __restrict__ out, int Mp, int Mo, int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y, b = blockIdx.z;
  float2 s = make_float2(0.f, 0.f);
  for (int m = 0; m < Mo; ++m) s = cadd(s, g[(((size_t)b * Mp + p) * Mo + m) * WW + u]);
  out[((size_t)b * Mp + p) * WW + u] = s;
}

// shift adjoint and position gradient (pypty/objective.py:641-658), one block per (p, b):
// F = spectrum of the probe gradient of position b, mode p; F *= conj(ramp_b); partial sums of
// -(s_y mask) Im(F conj(Pf)) and -(s_x mask) Im(F conj(Pf)) as the fused kernel's pos_part.
__global__ void __launch_bounds__(1024) probe_adj_kernel(float2* __restrict__ F, const float2* __restrict__ pf,
                                                         const float* __restrict__ sx, const float* __restrict__ sy,
                                                         const float* __restrict__ mask, const float* __restrict__ corr,
                                                         const int* __restrict__ seq, int W, int Mp, int step_pos,
                                                         double* __restrict__ pos_part) {
  __shared__ double red[64];
  const int p = blockIdx.x, b = blockIdx.y, gi = seq[b];
  const int WW = W * W;
  const float dy = corr[2 * gi], dx = corr[2 * gi + 1];
  float2* f = F + ((size_t)b * Mp + p) * WW;
  double gy = 0.0, gx = 0.0;
  for (int u = threadIdx.x; u < WW; u += blockDim.x) {
    const int ky = u / W, kx = u % W;
    const float mk = mask[u];
    const float2 v = cmulc(f[u], ramp(sx, sy, ky, kx, mk, dy, dx));
    f[u] = v;
    if (step_pos) {
      const float im = cmulc(v, pf[(size_t)p * WW + u]).y;
      gy += (double)(-(sy[ky] * mk) * im);
      gx += (double)(-(sx[kx] * mk) * im);
    }
  }
  if (!step_pos) return;
  block_sum2(gy, gx, red);
  if (threadIdx.x == 0) {
    pos_part[(b * Mp + p) * 2] = gy;
    pos_part[(b * Mp + p) * 2 + 1] = gx;
  }
}

// out[p][u] = mask[u] * sum_c partial[c][p][u]   grid (WW / EB, Mp)
__global__ void probe_total_kernel(const float2* __restrict__ partial, int nchunk, int Mp, const float* __restrict__ mask,
                                   float2* __restrict__ out, int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y;
  float2 s = make_float2(0.f, 0.f);
  for (int c = 0; c < nchunk; ++c) s = cadd(s, partial[((size_t)c * Mp + p) * WW + u]);
  out[(size_t)p * WW + u] = cscale(s, mask[u]);
}

// (W, W, Mp) reference layout <-> Mp natural planes   grid (WW / EB, Mp)
__global__ void probe_to_planes_kernel(const float2* __restrict__ ref, float2* __restrict__ planes, int Mp, int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y;
  planes[(size_t)p * WW + u] = ref[(size_t)u * Mp + p];
}
__global__ void planes_to_probe_kernel(const float2* __restrict__ planes, float2* __restrict__ ref, int Mp, int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y;
  ref[(size_t)u * Mp + p] = planes[(size_t)p * WW + u];
}

// ------------------------------------------------------------------ plan
struct LPlan {
  int W, WW, Ny, Nx, Z, Mo, Mp, N, nseq, Bb, zm, ntx, nty, ntiles, chunk, nchunk, engine;
  size_t o_pos, o_corr, o_seq, o_tab_pyx, o_mask, o_mask_sc, o_prop, o_prop_edge, o_sx, o_sy, o_planes, o_pf;
  size_t o_obj, o_grad, o_ob, o_tmp, o_dob, o_stack, o_psi, o_psi2, o_pb, o_pbs, o_partial, o_lists, o_counts;
  size_t o_loss_part, o_pos_part, o_dft, dft_bytes, total;
};

inline LPlan make_lplan(const pty_problem_t* p, int engine) {
  LPlan q{};
  q.W = p->window;
  q.WW = q.W * q.W;
  q.Ny = p->obj_ny;
  q.Nx = p->obj_nx;
  q.Z = p->n_slices;
  q.Mo = p->n_obj_modes;
  q.Mp = p->n_probe_modes;
  q.N = p->n_positions;
  q.nseq = p->n_sequence;
  q.Bb = p->compute_batch < q.nseq ? p->compute_batch : q.nseq;
  q.zm = q.Z * q.Mo;
  q.ntx = (q.Nx + kTileSize - 1) / kTileSize;
  q.nty = (q.Ny + kTileSize - 1) / kTileSize;
  q.ntiles = q.ntx * q.nty;
  q.chunk = 8;
  q.nchunk = (q.Bb + q.chunk - 1) / q.chunk;
  q.engine = engine;
  const size_t c8 = sizeof(float2), WWs = (size_t)q.WW;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t r = o;
    o = align_up(o + bytes);
    return r;
  };
  q.o_pos = take((size_t)q.N * 2 * sizeof(int));
  q.o_corr = take((size_t)q.N * 2 * sizeof(float));
  q.o_seq = take((size_t)q.nseq * sizeof(int));
  q.o_tab_pyx = take(2 * (size_t)q.W * c8);
  q.o_mask = take(WWs * sizeof(float));
  q.o_mask_sc = take(WWs * sizeof(float));
  q.o_prop = take(WWs * c8);
  q.o_prop_edge = take(WWs * c8);
  q.o_sx = take((size_t)q.W * sizeof(float));
  q.o_sy = take((size_t)q.W * sizeof(float));
  q.o_planes = take((size_t)q.Mp * WWs * c8);
  q.o_pf = take((size_t)q.Mp * WWs * c8);
  q.o_obj = take((size_t)q.zm * q.Ny * q.Nx * c8);
  q.o_grad = take((size_t)q.zm * q.Ny * q.Nx * c8);
  const size_t nobw = (size_t)q.Bb * q.zm, nwave = (size_t)q.Bb * q.Mp * q.Mo;
  q.o_ob = take(nobw * WWs * c8);
  q.o_tmp = take(nobw * WWs * c8);
  q.o_dob = take(nobw * WWs * c8);
  q.o_stack = take((size_t)q.Z * nwave * WWs * c8);
  q.o_psi = take(nwave * WWs * c8);
  q.o_psi2 = take(nwave * WWs * c8);
  q.o_pb = take((size_t)q.Bb * q.Mp * WWs * c8);
  q.o_pbs = take((size_t)q.Bb * q.Mp * WWs * c8);
  q.o_partial = take((size_t)q.nchunk * q.Mp * WWs * c8);
  q.o_lists = take((size_t)q.ntiles * q.Bb * sizeof(int));
  q.o_counts = take((size_t)q.ntiles * sizeof(int));
  q.o_loss_part = take((size_t)q.nseq * 2 * sizeof(double));
  q.o_pos_part = take((size_t)q.nseq * q.Mp * 2 * sizeof(double));
  size_t db = 0;
  const size_t maxwin = nobw > nwave ? nobw : nwave;
  const int32_t nmax = (int32_t)(maxwin > (size_t)q.Mp ? maxwin : (size_t)q.Mp);
  if (engine == PTY_DFT_BF16X3)
    pty_fft2_bf16x3_workspace_bytes(nmax, q.W, &db);
  else if (engine == PTY_DFT_BF16X6)
    pty_fft2_bf16x6_workspace_bytes(nmax, q.W, &db);
  else
    pty_fft2_workspace_bytes(q.W, &db);
  q.dft_bytes = db;
  q.o_dft = take(db);
  q.total = o;
  return q;
}

struct Run {
  const pty_problem_t* p;
  LPlan q;
  void* ws;
  cudaStream_t st;
  TableArgs ta{};

  int dft(const float2* in, float2* out, long long nwin, int inverse) {
    if (nwin <= 0) return PTY_OK;
    if (q.engine == PTY_DFT_BF16X3)
      return pty_fft2_bf16x3(in, out, (int32_t)nwin, q.W, inverse, at<void>(ws, q.o_dft), q.dft_bytes, st);
    if (q.engine == PTY_DFT_BF16X6)
      return pty_fft2_bf16x6(in, out, (int32_t)nwin, q.W, inverse, at<void>(ws, q.o_dft), q.dft_bytes, st);
    return pty_fft2(in, out, (int32_t)nwin, q.W, inverse, 0, at<void>(ws, q.o_dft), q.dft_bytes, st);
  }

  dim3 grid(int y, int z) const { return dim3((unsigned)(q.WW / EB), (unsigned)y, (unsigned)z); }

  int run(const float2* obj, const float2* probe, const float* measured, double* loss_sse, float2* object_grad,
          float2* probe_grad, float* pos_grad) {
    int rc;
    const int W = q.W, WW = q.WW;
    const bool shift = p->probe_shift != 0;
    const size_t WWs = (size_t)WW;
    ta.pyx = at<float2>(ws, q.o_tab_pyx);
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
    const float unfold = (float)WW;   // the tables fold 1/W^2 for the unnormalised register FFT: exact
    prof_mark(st, KID_TABLES);
    if (W == 64) tables_kernel<64><<<(WW + 255) / 256, 256, 0, st>>>(ta);
    else if (W == 128) tables_kernel<128><<<(WW + 255) / 256, 256, 0, st>>>(ta);
    else tables_kernel<256><<<(WW + 255) / 256, 256, 0, st>>>(ta);
    float2* planes = at<float2>(ws, q.o_planes);
    float2* pf = at<float2>(ws, q.o_pf);
    prof_mark(st, KID_LAYOUT);
    probe_to_planes_kernel<<<grid(q.Mp, 1), EB, 0, st>>>(probe, planes, q.Mp, WW);
    if ((rc = dft(planes, pf, q.Mp, 0))) return rc;
    const int nyx = q.Ny * q.Nx;
    prof_mark(st, KID_OBJ_TO_SLICES);
    obj_to_slices_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(obj, at<float2>(ws, q.o_obj), nyx, q.zm);
    const int* d_pos = at<int>(ws, q.o_pos);
    const float* d_corr = at<float>(ws, q.o_corr);
    float2 *ob = at<float2>(ws, q.o_ob), *tmp = at<float2>(ws, q.o_tmp), *dob = at<float2>(ws, q.o_dob);
    float2 *stack = at<float2>(ws, q.o_stack), *psi = at<float2>(ws, q.o_psi), *psi2 = at<float2>(ws, q.o_psi2);
    float2 *pb = at<float2>(ws, q.o_pb), *pbs = at<float2>(ws, q.o_pbs);
    const int nm = q.Mp * q.Mo;
    for (int i0 = 0, ib = 0; i0 < q.nseq; i0 += q.Bb, ++ib) {
      const int Bn = q.nseq - i0 < q.Bb ? q.nseq - i0 : q.Bb;
      const int* seq_b = at<int>(ws, q.o_seq) + i0;
      // object windows, band-limited (objective.py:436-441)
      prof_mark(st, KID_OBJECT_WINDOWS);
      gather_kernel<<<grid(q.zm, Bn), EB, 0, st>>>(at<float2>(ws, q.o_obj), ob, d_pos, seq_b, W, q.Ny, q.Nx, q.zm);
      if ((rc = dft(ob, tmp, (long long)Bn * q.zm, 0))) return rc;
      prof_mark(st, KID_ELEMENTWISE);
      mask_kernel<<<grid(Bn * q.zm, 1), EB, 0, st>>>(tmp, ta.mask, WW);
      if ((rc = dft(tmp, ob, (long long)Bn * q.zm, 1))) return rc;
      // incoming probe per position (objective.py:469-476)
      const float2* pin = planes;
      size_t pin_stride = 0;
      if (shift) {
        prof_mark(st, KID_ELEMENTWISE);
        probe_spec_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(pbs, pf, ta.sx, ta.sy, ta.mask, d_corr, seq_b, W, q.Mp);
        if ((rc = dft(pbs, pb, (long long)Bn * q.Mp, 1))) return rc;
        pin = pb;
        pin_stride = (size_t)q.Mp * WWs;
      }
      // forward multislice (multislice_core.py:61-82)
      for (int z = 0; z < q.Z; ++z) {
        prof_mark(st, KID_FUSED);
        fwd_slice_kernel<<<grid(nm, Bn), EB, 0, st>>>(pin, pin_stride, psi, stack, ob, z, q.Z, q.Mp, q.Mo, WW);
        if (z < q.Z - 1) {
          if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
          prof_mark(st, KID_ELEMENTWISE);
          prop_kernel<<<grid(Bn * nm, 1), EB, 0, st>>>(psi2, (z == 0 && ta.use_edge) ? ta.prop_edge : ta.prop, WW,
                                                       0, unfold);
          if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
        }
      }
      // far field, loss, dL/dPsi (objective.py:501-597)
      if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
      prof_mark(st, KID_FINALIZE);
      loss_kernel<<<Bn, 1024, 0, st>>>(psi2, ta.mask, measured, seq_b, W, q.Mp, q.Mo, p->algorithm,
                                       p->loss_weight * (float)WW, at<double>(ws, q.o_loss_part) + 2 * i0);
      if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
      // adjoint multislice (multislice_core.py:158-200)
      for (int z = q.Z - 1; z >= 0; --z) {
        prof_mark(st, KID_FUSED);
        adj_slice_kernel<<<grid(q.Mo, Bn), EB, 0, st>>>(psi, stack, ob, dob, z, q.Z, q.Mp, q.Mo, WW);
        if (z > 0) {
          if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
          prof_mark(st, KID_ELEMENTWISE);
          prop_kernel<<<grid(Bn * nm, 1), EB, 0, st>>>(psi2, (z == 1 && ta.use_edge) ? ta.prop_edge : ta.prop, WW,
                                                       1, unfold);
          if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
        }
      }
      if (p->step_obj) {
        // band-limited gradient windows (multislice_core.py:189-191), deterministic scatter
        if ((rc = dft(dob, tmp, (long long)Bn * q.zm, 0))) return rc;
        prof_mark(st, KID_ELEMENTWISE);
        mask_kernel<<<grid(Bn * q.zm, 1), EB, 0, st>>>(tmp, ta.mask, WW);
        if ((rc = dft(tmp, dob, (long long)Bn * q.zm, 1))) return rc;
        int* lists = at<int>(ws, q.o_lists);
        int* counts = at<int>(ws, q.o_counts);
        prof_mark(st, KID_TILE_LISTS);
        tile_lists_kernel<<<q.ntiles, 256, 0, st>>>(d_pos, seq_b, Bn, W, q.ntx, lists, counts);
        prof_mark(st, KID_SCATTER);
        scatter_tiles_kernel<<<dim3(q.ntiles, q.zm), dim3(32, 8), 0, st>>>(
            dob, d_pos, seq_b, lists, counts, at<float2>(ws, q.o_grad), Bn, W, q.Ny, q.Nx, q.ntx, q.zm, ib > 0);
      }
      if (p->step_probe || p->step_pos) {
        // probe-gradient spectra with the shift adjoint and the position gradient (objective.py:641-703)
        prof_mark(st, KID_PROBE_PARTIAL);
        probe_sum_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(psi, pbs, q.Mp, q.Mo, WW);
        if ((rc = dft(pbs, pb, (long long)Bn * q.Mp, 0))) return rc;
        prof_mark(st, KID_ELEMENTWISE);
        if (shift)
          probe_adj_kernel<<<dim3(q.Mp, Bn), 1024, 0, st>>>(pb, pf, ta.sx, ta.sy, ta.mask, d_corr, seq_b, W, q.Mp,
                                                           p->step_pos, at<double>(ws, q.o_pos_part) + (size_t)i0 * q.Mp * 2);
        if (p->step_probe) {
          const int nch = (Bn + q.chunk - 1) / q.chunk;
          prof_mark(st, KID_PROBE_PARTIAL);
          probe_partial_kernel<<<dim3((unsigned)((WW + 255) / 256), q.Mp, nch), 256, 0, st>>>(
              pb, at<float2>(ws, q.o_partial), Bn, q.Mp, WW, q.chunk, ib > 0 ? 1 : 0);
        }
      }
    }
    // probe gradient: IFFT(mask * sum_b spectra) (objective.py:703, 927-933)
    if (p->step_probe) {
      prof_mark(st, KID_PROBE_FINAL);
      probe_total_kernel<<<grid(q.Mp, 1), EB, 0, st>>>(at<float2>(ws, q.o_partial), q.nchunk, q.Mp, ta.mask, pbs, WW);
      if ((rc = dft(pbs, pb, q.Mp, 1))) return rc;
      prof_mark(st, KID_LAYOUT);
      planes_to_probe_kernel<<<grid(q.Mp, 1), EB, 0, st>>>(pb, probe_grad, q.Mp, WW);
    }
    if (p->step_obj) {
      prof_mark(st, KID_SLICES_TO_OBJ);
      slices_to_obj_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(at<float2>(ws, q.o_grad), object_grad, nyx, q.zm);
    }
    if (p->step_pos && cudaMemsetAsync(pos_grad, 0, (size_t)q.N * 2 * sizeof(float), st) != cudaSuccess)
      return PTY_ERR_CUDA;
    prof_mark(st, KID_FINALIZE);
    finalize_scalars_kernel<<<1, 256, 0, st>>>(at<double>(ws, q.o_loss_part), at<double>(ws, q.o_pos_part),
                                               at<int>(ws, q.o_seq), q.nseq, q.Mp, W, (double)p->loss_weight,
                                               p->step_pos && shift, nullptr, loss_sse, pos_grad);
    prof_mark(st, -1);
    return cuda_status();
  }
};

}  // namespace lay
}  // namespace pty

using namespace pty;

extern "C" {

int pty_layered_workspace_bytes(const pty_problem_t* problem, int32_t engine, size_t* bytes) {
  int rc = validate(problem);
  if (rc) return rc;
  if (!bytes || engine < PTY_DFT_FP32_FFT || engine > PTY_DFT_BF16X6) return PTY_ERR_INVALID;
  *bytes = lay::make_lplan(problem, engine).total;
  return PTY_OK;
}

int pty_loss_and_direction_layered(const pty_problem_t* problem, int32_t engine, const void* obj, const void* probe,
                                   const int32_t* positions_host, const float* pos_correction,
                                   const int32_t* sequence_host, const float* measured, double* loss_sse,
                                   void* object_grad, void* probe_grad, float* pos_grad, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  int rc = validate(problem);
  if (rc) return rc;
  if (engine < PTY_DFT_FP32_FFT || engine > PTY_DFT_BF16X6) return PTY_ERR_INVALID;
  if (!obj || !probe || !positions_host || !sequence_host || !measured || !loss_sse || !workspace)
    return PTY_ERR_INVALID;
  if ((problem->step_obj && !object_grad) || (problem->step_probe && !probe_grad) || (problem->step_pos && !pos_grad))
    return PTY_ERR_INVALID;
  if ((rc = check_geometry(problem, positions_host, sequence_host))) return rc;
  const lay::LPlan q = lay::make_lplan(problem, engine);
  if ((long long)q.Bb * (q.zm > q.Mp * q.Mo ? q.zm : q.Mp * q.Mo) > 65535) return PTY_ERR_UNSUPPORTED;
  if (workspace_bytes < q.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(at<int>(workspace, q.o_pos), positions_host, (size_t)q.N * 2 * sizeof(int), cudaMemcpyDefault,
                      st) != cudaSuccess)
    return PTY_ERR_CUDA;
  if (pos_correction) {
    if (cudaMemcpyAsync(at<float>(workspace, q.o_corr), pos_correction, (size_t)q.N * 2 * sizeof(float),
                        cudaMemcpyDefault, st) != cudaSuccess)
      return PTY_ERR_CUDA;
  } else if (cudaMemsetAsync(at<float>(workspace, q.o_corr), 0, (size_t)q.N * 2 * sizeof(float), st) != cudaSuccess) {
    return PTY_ERR_CUDA;
  }
  if (cudaMemcpyAsync(at<int>(workspace, q.o_seq), sequence_host, (size_t)q.nseq * sizeof(int), cudaMemcpyDefault,
                      st) != cudaSuccess)
    return PTY_ERR_CUDA;
  lay::Run r{problem, q, workspace, st};
  return r.run(static_cast<const float2*>(obj), static_cast<const float2*>(probe), measured, loss_sse,
               static_cast<float2*>(object_grad), static_cast<float2*>(probe_grad), pos_grad);
}

}  // extern "C"

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
namespace pty {
// dft_gemm.cu: one tensor-core transform inside a call that clears the error word once, and
// the error word of a tensor-core DFT workspace
int tc_fft2(const float2* in, float2* out, long long batch, int window, int inverse, int terms, void* ws,
            size_t ws_bytes, cudaStream_t st);
int* tc_err_word(void* ws, int window, int terms);
}  // namespace pty

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

// (W, W, Mp, S) reference layout <-> S x Mp natural planes   grid (WW / EB, Mp, S)
__global__ void probe_to_planes_s_kernel(const float2* __restrict__ ref, float2* __restrict__ planes, int Mp, int S,
                                         int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y, s = blockIdx.z;
  planes[((size_t)s * Mp + p) * WW + u] = ref[((size_t)u * Mp + p) * S + s];
}
__global__ void planes_to_probe_s_kernel(const float2* __restrict__ planes, float2* __restrict__ ref, int Mp, int S,
                                         int WW) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y, s = blockIdx.z;
  ref[((size_t)u * Mp + p) * S + s] = planes[((size_t)s * Mp + p) * WW + u];
}

// per-scenario chunk sums of the batch's probe-gradient spectra: partial[c][s][p] (+)= the sum
// over positions b of chunk c whose scenario is s (objective.py:700-701), in position order
// grid (WW / 256, Mp * S, nchunk), block 256
__global__ void probe_partial_s_kernel(const float2* __restrict__ fprobe, float2* __restrict__ partial, int Bn, int Mp,
                                       int S, int WW, int chunk, int accumulate, const int* __restrict__ pmarker,
                                       const int* __restrict__ seq) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int sp = blockIdx.y, c = blockIdx.z, s = sp / Mp, p = sp % Mp;
  if (e >= WW) return;
  float2 acc = make_float2(0.f, 0.f);
  const int b1 = min(Bn, (c + 1) * chunk);
  for (int b = c * chunk; b < b1; ++b) {
    int m = pmarker[seq[b]];
    if (m < 0 || m >= S) m = 0;
    if (m == s) acc = cadd(acc, fprobe[((size_t)b * Mp + p) * WW + e]);
  }
  float2* dst = partial + ((size_t)c * S * Mp + sp) * WW + e;
  *dst = accumulate ? cadd(*dst, acc) : acc;
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

// ------------------------------------------------------------------ variants
// Tables of pty_loss_and_direction_variants (after tables_kernel wrote the mask):
// propagator with the inside tilt (pypty/objective.py:343) and its edge power, the
// near-field CTF (objective.py:505) and the aberration basis imag(poly_j) = -A_j
// (pypty/utils.py:1333-1368 get_ctf_matrix, objective.py:326-327).
struct VarTableArgs {
  float2* prop;
  float2* prop_edge;
  float2* ctf;
  float* tgrid;           // [2][W] real-space tilt ramps (x, y)
  float* abasis;          // [n_abs][WW]
  const float* mask;
  const int* abn;         // [n_abs] Krivanek n
  const int* abm;         // [n_abs] Krivanek m
  const int* abk;         // [n_abs] 0: m = 0, 1: cos (a), 2: sin (b)
  int W, use_edge, near, n_abs;
  float px, py, distance, wavelength, edge_mult, tan_x, tan_y, defocus, cs;
  const float* tilt_row;  // device tilt row [6] whose inside tilt (2, 3) replaces tan_y, tan_x, or nullptr
};

__global__ void var_tables_kernel(VarTableArgs a) {
  const int W = a.W, WW = W * W;
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= WW) return;
  if (u < W) {
    // x_real_grid_tilt / y_real_grid_tilt (objective.py:303-307): fftshift(fftfreq(W)) *
    // 6.2831855 i * W * pixel size / lambda in float64, rounded to complex64
    const double f = (double)(u - W / 2) / (double)W;
    a.tgrid[u] = (float)(f * 6.2831855 * (double)W * (double)a.px / (double)a.wavelength);
    a.tgrid[W + u] = (float)(f * 6.2831855 * (double)W * (double)a.py / (double)a.wavelength);
  }
  const int ky = u / W, kx = u % W;
  const float qx = fftfreq_f32(kx, W, a.px), qy = fftfreq_f32(ky, W, a.py);
  const float q2 = __fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy));
  const float mk = a.mask[u];
  const float tan_x = a.tilt_row ? a.tilt_row[3] : a.tan_x, tan_y = a.tilt_row ? a.tilt_row[2] : a.tan_y;
  // lambda q2 + 2 (qx tan_x + qy tan_y), float32 in the reference's order
  const float tilt = __fmul_rn(2.0f, __fadd_rn(__fmul_rn(qx, tan_x), __fmul_rn(qy, tan_y)));
  const float x = __fadd_rn(__fmul_rn(a.wavelength, q2), tilt);
  const float inv = 1.0f / (float)WW;
  {
    const float phase = __fmul_rn(__fmul_rn(-3.141592654f, a.distance), x);
    float s, c;
    sincosf(phase, &s, &c);
    const float2 p = make_float2(c * mk, s * mk);
    a.prop[u] = make_float2(p.x * inv, p.y * inv);
    if (a.use_edge) {
      const float r = sqrtf(p.x * p.x + p.y * p.y);
      float2 pe = make_float2(0.f, 0.f);
      if (r > 0.f) {
        const float ang = atan2f(p.y, p.x) * a.edge_mult;
        const float re = powf(r, a.edge_mult);
        float se, ce;
        sincosf(ang, &se, &ce);
        pe = make_float2(re * ce, re * se);
      }
      a.prop_edge[u] = make_float2(pe.x * inv, pe.y * inv);
    }
  }
  if (a.near) {
    // exp(-i pi (x defocus + 0.5 Cs lambda^3 q2^2)) * mask
    const float l3 = __fmul_rn(__fmul_rn(a.wavelength, a.wavelength), a.wavelength);
    const float sph = __fmul_rn(__fmul_rn(__fmul_rn(0.5f, a.cs), l3), __fmul_rn(q2, q2));
    const float phase = __fmul_rn(-3.141592654f, __fadd_rn(__fmul_rn(x, a.defocus), sph));
    float s, c;
    sincosf(phase, &s, &c);
    a.ctf[u] = make_float2(c * mk, s * mk);
  }
  if (a.n_abs > 0) {
    // k = lambda q (float32); k_r ** (n + 1) / (n + 1) and cos / sin (m phi) in float64 (the
    // reference's int64 orders promote), scaled by float32(2 pi / lambda)
    const float kxv = __fmul_rn(a.wavelength, qx), kyv = __fmul_rn(a.wavelength, qy);
    const double kr = (double)sqrtf(__fadd_rn(__fmul_rn(kxv, kxv), __fmul_rn(kyv, kyv)));
    const double phi = (double)atan2f(kyv, kxv);
    const double sc = (double)__fdiv_rn(6.2831855f, a.wavelength);
    for (int j = 0; j < a.n_abs; ++j) {
      const int n = a.abn[j], m = a.abm[j];
      double term = pow(kr, (double)(n + 1)) / (double)(n + 1);
      if (a.abk[j] == 1) term *= cos((double)m * phi);
      else if (a.abk[j] == 2) term *= sin((double)m * phi);
      a.abasis[(size_t)j * WW + u] = -(float)(term * sc);
    }
  }
}

// aberration plate of position b at pixel u: exp(i sum_j imag(poly_j) c_j) * mask
// (objective.py:328; the sum runs over j in order in float32)
__device__ __forceinline__ float2 plate_at(const float* __restrict__ abasis, const float* __restrict__ coef, int n_abs,
                                           int WW, int u, float mk) {
  float th = 0.0f;
  for (int j = 0; j < n_abs; ++j) th = __fadd_rn(th, __fmul_rn(abasis[(size_t)j * WW + u], coef[j]));
  float s, c;
  sincosf(th, &s, &c);
  return make_float2(c * mk, s * mk);
}

struct VarProbeArgs {
  const float2* pf;          // [Mp][WW] probe spectra
  const float2* planes;      // [Mp][WW] probe planes
  const float *sx, *sy, *mask, *corr;
  const int* seq;
  const float* bc;           // beam current [N] or null
  const float* abasis;       // [n_abs][WW]
  const float* coefs;        // aberrations [sets][n_abs] or null
  const int* marker;         // [N]
  const float2* pspec;       // [Bn][Mp][WW] per-position probe spectra the shift was applied to, or null (bc FFT(P))
  int W, Mp, shift, n_abs, n_sets;
  const int* pmarker;        // probe scenario per position [N] (pf / planes hold S scenarios), or null
  int S;
};

// offset of position gi's probe scenario in [S][Mp][WW] planes / spectra (objective.py:443-444);
// a marker outside [0, S) reads scenario 0
__device__ __forceinline__ size_t scenario_off(const VarProbeArgs& a, int gi) {
  if (!a.pmarker) return 0;
  const int m = a.pmarker[gi];
  return (m >= 0 && m < a.S) ? (size_t)m * a.Mp * a.W * a.W : 0;
}

// aberration coefficients of position gi, or null (no plates, or a marker out of range)
__device__ __forceinline__ const float* coefs_of(const VarProbeArgs& a, int gi) {
  if (!a.coefs) return nullptr;
  const int m = a.marker[gi];
  return (m >= 0 && m < a.n_sets) ? a.coefs + (size_t)m * a.n_abs : nullptr;
}

// incoming probe per position (objective.py:448-476): with a shift or aberration plates the
// spectrum bc * FFT(P) times the shift ramp (the shift takes the spectrum before the plates,
// objective.py:461, 471) or the plate; else the real-space probe times bc.
// spec_or_pb[b][p][u]   grid (WW / EB, Mp, Bn)
__global__ void var_probe_in_kernel(VarProbeArgs a, float2* __restrict__ out) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y, b = blockIdx.z;
  const int W = a.W, WW = W * W, gi = a.seq[b];
  const float bc = a.bc ? fabsf(a.bc[gi]) : 1.0f;
  float2 v;
  if (a.shift || a.coefs) {
    const float mk = a.mask[u];
    const float* coef = coefs_of(a, gi);
    const float2 w = a.shift ? ramp(a.sx, a.sy, u / W, u % W, mk, a.corr[2 * gi], a.corr[2 * gi + 1])
                     : coef  ? plate_at(a.abasis, coef, a.n_abs, WW, u, mk)
                             : make_float2(mk, 0.0f);
    const float2* pf = a.pf + scenario_off(a, gi);
    v = cmul(a.bc ? cscale(pf[(size_t)p * WW + u], bc) : pf[(size_t)p * WW + u], w);
  } else {
    v = cscale(a.planes[scenario_off(a, gi) + (size_t)p * WW + u], bc);
  }
  out[((size_t)b * a.Mp + p) * WW + u] = v;
}

// pattern of every position (objective.py:509-512): mean over modes of |field|^2; the far
// field is the unshifted spectrum, masked, stored at the detector (fftshifted) pixel; the
// near field is the real-space wave.   grid (WW / EB, Bn)
__global__ void var_intensity_kernel(const float2* __restrict__ field, const float* __restrict__ mask,
                                     float* __restrict__ ibuf, int W, int nm, int near) {
  const int u = blockIdx.x * EB + threadIdx.x, b = blockIdx.y;
  const int WW = W * W;
  const float2* f = field + (size_t)b * nm * WW;
  float acc = 0.0f;
  if (near) {
    for (int k = 0; k < nm; ++k) acc += cabs2(f[(size_t)k * WW + u]);
  } else {
    const float mk = mask[u];
    for (int k = 0; k < nm; ++k) acc += cabs2(cscale(f[(size_t)k * WW + u], mk));
  }
  const float I = nm == 1 ? acc : acc * (1.0f / (float)nm);
  const int ky = u / W, kx = u % W;
  const int pix = near ? u : ((ky + W / 2) & (W - 1)) * W + ((kx + W / 2) & (W - 1));
  ibuf[(size_t)b * WW + pix] = I;
}

// measured-data preprocessing applied on the fly (pypty/utils.py:626-652) and the detector
// upsampling of objective.py:523-524, 590-591. The model pattern is W x W; without padded it
// is cropped by pad (objective.py:516-517) to S = W - 2 pad, else S = W. It is summed over
// up x up blocks (utils.py:403-426) to Sd = S / up. The measured patterns are Wm x Wm
// (Wm = Sd - 2 po, po = pad / up when padded, else 0), rolled by (sy, sx) with the rows /
// columns the reference zeroes, scaled by mult and zero-padded by po.
struct MeasPrep {
  int W, pad, padded, sy, sx;
  float mult;
  int up;
};

__host__ __device__ __forceinline__ int meas_side(const MeasPrep& mp) {
  const int S = mp.padded ? mp.W : mp.W - 2 * mp.pad;
  return S / mp.up - 2 * (mp.padded ? mp.pad / mp.up : 0);
}

// source index along one axis of the rolled Wm-long measured axis, or -1 for a zeroed entry
// (np.roll then a[-s:] = 0 for s > 0, a[:-s] = 0 for s < 0)
__device__ __forceinline__ int rolled(int i, int s, int n) {
  if ((s > 0 && i >= n - s) || (s < 0 && i < -s)) return -1;
  int j = (i - s) % n;
  return j < 0 ? j + n : j;
}

// per-pixel losses (objective.py:527-559) on the (cropped, block-summed) pattern: every
// model pixel of a block gets that block's dL/dI / nm (utils.py:376-399 without scaling),
// pixels cropped away get zero; FP64 partial sums per position   grid Bn, block 1024
__global__ void __launch_bounds__(1024) var_pixel_loss_kernel(float* __restrict__ ibuf, const float* __restrict__ measured,
                                                              const int* __restrict__ seq, MeasPrep mp, int nm, int alg,
                                                              double* __restrict__ loss_part) {
  __shared__ double red[64];
  const int b = blockIdx.x;
  const int W = mp.W, WW = W * W, up = mp.up;
  const int S = mp.padded ? W : W - 2 * mp.pad, c0 = mp.padded ? 0 : mp.pad;
  const int Sd = S / up, po = mp.padded ? mp.pad / up : 0, Wm = meas_side(mp);
  const float* meas = measured + (size_t)seq[b] * Wm * Wm;
  float* I = ibuf + (size_t)b * WW;
  if (S < W) {   // cropped model pattern: no loss, dL/dI padded with zeros
    for (int u = threadIdx.x; u < WW; u += blockDim.x) {
      const int y = u / W - c0, x = u % W - c0;
      if (y < 0 || y >= S || x < 0 || x >= S) I[u] = 0.0f;
    }
  }
  double lsum = 0.0, ssum = 0.0;
  for (int d = threadIdx.x; d < Sd * Sd; d += blockDim.x) {
    const int yd = d / Sd, xd = d % Sd;
    float* blk = I + (size_t)(c0 + yd * up) * W + c0 + xd * up;
    float P = 0.0f;
    for (int i = 0; i < up; ++i)
      for (int j = 0; j < up; ++j) P += blk[i * W + j];
    const int ym = yd - po, xm = xd - po;
    float Mv = 0.0f;
    if (ym >= 0 && ym < Wm && xm >= 0 && xm < Wm) {
      const int ry = rolled(ym, mp.sy, Wm), rx = rolled(xm, mp.sx, Wm);
      if (ry >= 0 && rx >= 0) Mv = meas[ry * Wm + rx];
      if (mp.mult != 1.0f) Mv = Mv * mp.mult;
    }
    float g = loss_pixel(alg, P, Mv, lsum, ssum);
    if (nm > 1) g = g / (float)nm;
    for (int i = 0; i < up; ++i)
      for (int j = 0; j < up; ++j) blk[i * W + j] = g;
  }
  block_sum2(lsum, ssum, red);
  if (threadIdx.x == 0) {
    loss_part[2 * b] = lsum;
    loss_part[2 * b + 1] = ssum;
  }
}

// static background (objective.py:359-361, 525-526): pattern += bg^2 * exclude_mask, the
// band-limit mask in detector (fftshifted) order; mask is in FFT order   grid (WW / EB, Bn)
__global__ void var_add_static_kernel(float* __restrict__ ibuf, const float* __restrict__ bg,
                                      const float* __restrict__ mask, int W) {
  const int u = blockIdx.x * EB + threadIdx.x, b = blockIdx.y;
  const int ky = u / W, kx = u % W;
  const float mk = mask[((ky + W / 2) & (W - 1)) * W + ((kx + W / 2) & (W - 1))];
  const float s = bg[u];
  ibuf[(size_t)b * W * W + u] += (s * s) * mk;
}

// static-background gradient (objective.py:588-589): acc[u] += sum_b dL/dI[b][u] * 2 bg[u] lw,
// positions summed in order in FP64   grid WW / 256, block 256
__global__ void var_static_grad_kernel(const float* __restrict__ ibuf, const float* __restrict__ bg, int Bn, int WW,
                                       float lw, double* __restrict__ acc) {
  const int u = blockIdx.x * 256 + threadIdx.x;
  if (u >= WW) return;
  double sum = 0.0;
  for (int b = 0; b < Bn; ++b) sum += (double)ibuf[(size_t)b * WW + u];
  acc[u] += sum * (2.0 * (double)bg[u] * (double)lw);
}

__global__ void var_static_final_kernel(const double* __restrict__ acc, int WW, float* __restrict__ grad) {
  const int u = blockIdx.x * 256 + threadIdx.x;
  if (u < WW) grad[u] = (float)acc[u];
}

// detector coefficients coef[b][j] = sum_u I[b][u] masks[j][u] (objective.py:561)
// grid (n_masks, Bn), block 256
__global__ void var_coef_kernel(const float* __restrict__ ibuf, const float* __restrict__ masks, int WW, int nmask,
                                float* __restrict__ coef) {
  __shared__ double red[64];
  const int j = blockIdx.x, b = blockIdx.y;
  const float* I = ibuf + (size_t)b * WW;
  const float* m = masks + (size_t)j * WW;
  double acc = 0.0, unused = 0.0;
  for (int u = threadIdx.x; u < WW; u += blockDim.x) acc += (double)(I[u] * m[u]);
  block_sum2(acc, unused, red);
  if (threadIdx.x == 0) coef[(size_t)b * nmask + j] = (float)acc;
}

// compressed losses on the coefficients (objective.py:560-585): dco[b][j] = dL/dcoef,
// FP64 loss / sse partial sums per position   grid Bn, block 32
__global__ void var_closs_kernel(const float* __restrict__ coef, const float* __restrict__ measured,
                                 const int* __restrict__ seq, int nmask, int alg, float* __restrict__ dco,
                                 double* __restrict__ loss_part) {
  const int b = blockIdx.x;
  const float* ms = measured + (size_t)seq[b] * nmask;
  double lsum = 0.0, ssum = 0.0;
  for (int j = threadIdx.x; j < nmask; j += blockDim.x) {
    const float c = coef[(size_t)b * nmask + j], mv = ms[j];
    float d;
    if (alg == PTY_LSQ_COMPRESSED) {
      const float df = c - mv;
      const float t = df * df;
      lsum += (double)t;
      ssum += (double)t;
      d = 2.0f * df;
    } else if (alg == PTY_GAUSS_COMPRESSED) {
      float cs = sqrtf(c);
      const float dd = cs - sqrtf(mv);
      const float e = c - mv;
      ssum += (double)(e * e);
      lsum += (double)(dd * dd);
      if (cs == 0.0f) cs = 1.0f;
      d = dd / cs;
    } else {   // PTY_POISSON_COMPRESSED
      const float dd = c - mv;
      ssum += (double)(dd * dd);
      const float cz = c == 0.0f ? 1.0f : c;
      lsum += (double)(cz - mv * logf(cz));
      d = dd / cz;
    }
    dco[(size_t)b * nmask + j] = d;
  }
  for (int o = 16; o > 0; o >>= 1) {
    lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    ssum += __shfl_down_sync(0xffffffffu, ssum, o);
  }
  if (threadIdx.x == 0) {
    loss_part[2 * b] = lsum;
    loss_part[2 * b + 1] = ssum;
  }
}

// dL/dI = sum_j masks[j] dco[b][j] (j in order), / nm   grid (WW / EB, Bn)
__global__ void var_cdldi_kernel(float* __restrict__ ibuf, const float* __restrict__ masks,
                                 const float* __restrict__ dco, int WW, int nmask, int nm) {
  const int u = blockIdx.x * EB + threadIdx.x, b = blockIdx.y;
  float acc = 0.0f;
  for (int j = 0; j < nmask; ++j) acc += masks[(size_t)j * WW + u] * dco[(size_t)b * nmask + j];
  if (nm > 1) acc = acc / (float)nm;
  ibuf[(size_t)b * WW + u] = acc;
}

// dL/dwave: far field F_k *= mask * dL/dI[detector pixel] * scale (objective.py:595-596);
// near field wave_k *= dL/dI (objective.py:602)   grid (WW / EB, nm, Bn)
__global__ void var_apply_kernel(float2* __restrict__ field, const float* __restrict__ ibuf,
                                 const float* __restrict__ mask, int W, int nm, int near, float scale) {
  const int u = blockIdx.x * EB + threadIdx.x, k = blockIdx.y, b = blockIdx.z;
  const int WW = W * W;
  float2* q = field + ((size_t)b * nm + k) * WW + u;
  if (near) {
    *q = cscale(*q, ibuf[(size_t)b * WW + u]);
  } else {
    const int ky = u / W, kx = u % W;
    const int pix = ((ky + W / 2) & (W - 1)) * W + ((kx + W / 2) & (W - 1));
    *q = cscale(cscale(cscale(*q, mask[u]), ibuf[(size_t)b * WW + pix]), scale);
  }
}

// probe-gradient spectrum chain of one (probe mode p, position b) (objective.py:641-697):
// F = FFT(probe gradient); shift adjoint and position gradient partials; plate adjoint and
// aberration gradient partials against bc * FFT(P); beam-current gradient partial
// sum Re(F conj(FFT(P))) (Parseval: W^2 times the real-space sum); F *= bc for the probe
// gradient. Partials: pos_part[s][p][2], bc_part[s][p], ab_part[s][p][n_abs].
// grid (Mp, Bn), block 1024
// do_shift / do_rest split the chain around the adjoint of a tilt before the specimen, which
// the caller applies in real space between the two parts (objective.py:660-673).
__global__ void __launch_bounds__(1024) var_probe_adj_kernel(float2* __restrict__ F, VarProbeArgs a, int step_pos,
                                                             int step_bc, int step_ab, int step_probe, int do_shift,
                                                             int do_rest, double* __restrict__ pos_part,
                                                             double* __restrict__ bc_part,
                                                             double* __restrict__ ab_part) {
  __shared__ double red[64];
  const int p = blockIdx.x, b = blockIdx.y, gi = a.seq[b];
  const int W = a.W, WW = W * W;
  const float bc = a.bc ? fabsf(a.bc[gi]) : 1.0f;
  const float* coef = do_rest ? coefs_of(a, gi) : nullptr;
  const bool sh = a.shift && do_shift, bcr = a.bc && do_rest;
  const float dy = a.corr[2 * gi], dx = a.corr[2 * gi + 1];
  float2* f = F + ((size_t)b * a.Mp + p) * WW;
  const float2* pf = a.pf + scenario_off(a, gi) + (size_t)p * WW;
  double gy = 0.0, gx = 0.0, gb = 0.0;
  for (int u = threadIdx.x; u < WW; u += blockDim.x) {
    const int ky = u / W, kx = u % W;
    const float mk = a.mask[u];
    const float2 before = a.pspec ? a.pspec[((size_t)b * a.Mp + p) * WW + u] : (a.bc ? cscale(pf[u], bc) : pf[u]);
    float2 v = f[u];
    if (sh) {
      v = cmulc(v, ramp(a.sx, a.sy, ky, kx, mk, dy, dx));
      if (step_pos) {
        const float im = cmulc(v, before).y;
        gy += (double)(-(a.sy[ky] * mk) * im);
        gx += (double)(-(a.sx[kx] * mk) * im);
      }
    }
    if (coef) v = cmulc(v, plate_at(a.abasis, coef, a.n_abs, WW, u, mk));
    if (bcr && step_bc) gb += (double)cmulc(v, pf[u]).x;
    f[u] = v;
  }
  if (step_pos && sh) {
    double gyy = gy, gxx = gx;
    block_sum2(gyy, gxx, red);
    if (threadIdx.x == 0) {
      pos_part[((size_t)b * a.Mp + p) * 2] = gyy;
      pos_part[((size_t)b * a.Mp + p) * 2 + 1] = gxx;
    }
  }
  if (bcr && step_bc) {
    double unused = 0.0;
    block_sum2(gb, unused, red);
    if (threadIdx.x == 0) bc_part[(size_t)b * a.Mp + p] = gb;
  }
  if (coef && step_ab) {
    // sum_u -A_j Im(F conj(bc FFT(P))) for every aberration coefficient j; the plate adjoint
    // has been applied to f (objective.py:677-681)
    for (int j = 0; j < a.n_abs; ++j) {
      __syncthreads();
      double acc = 0.0, unused = 0.0;
      for (int u = threadIdx.x; u < WW; u += blockDim.x) {
        const float2 before = a.bc ? cscale(pf[u], bc) : pf[u];
        acc += (double)(a.abasis[(size_t)j * WW + u] * cmulc(f[u], before).y);
      }
      block_sum2(acc, unused, red);
      if (threadIdx.x == 0) ab_part[((size_t)b * a.Mp + p) * a.n_abs + j] = acc;
    }
  }
  // probe gradient times the beam current (objective.py:698-699); every thread rescales the
  // pixels it wrote itself
  if (bcr && step_probe)
    for (int u = threadIdx.x; u < WW; u += blockDim.x) f[u] = cscale(f[u], bc);
}

// beam-current and aberration gradients from the partials, in sequence order
// (objective.py:681-682, 693-697)   one block of 256
__global__ void var_finalize_kernel(const double* __restrict__ bc_part, const double* __restrict__ ab_part,
                                    const int* __restrict__ seq, int nseq, int Mp, int W, int N,
                                    const float* __restrict__ bc, float* __restrict__ bc_grad, int n_sets, int n_abs,
                                    const int* __restrict__ marker, float* __restrict__ ab_grad) {
  const double sh = 2.0 / ((double)W * (double)W);
  if (bc_grad) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) bc_grad[i] = 0.0f;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int s = 0; s < nseq; ++s) {
        double g = 0.0;
        for (int p = 0; p < Mp; ++p) g += bc_part[(size_t)s * Mp + p];
        const float sgn = bc[seq[s]] != 0.0f ? 1.0f : 0.0f;   // sign(|bc|)
        bc_grad[seq[s]] = (float)(sh * g) * sgn;
      }
    }
  }
  if (ab_grad) {
    for (int t = threadIdx.x; t < n_sets * n_abs; t += blockDim.x) {
      const int set = t / n_abs, j = t % n_abs;
      double g = 0.0;
      for (int s = 0; s < nseq; ++s) {
        if (marker[seq[s]] != set) continue;
        double gs = 0.0;
        for (int p = 0; p < Mp; ++p) gs += ab_part[((size_t)s * Mp + p) * n_abs + j];
        g += (double)(float)(sh * gs);
      }
      ab_grad[t] = (float)g;
    }
  }
}

// ------------------------------------------------------------------ beam tilts
// Tilt rows [tan_y, tan_x] before (0, 1), inside (2, 3) and after (4, 5) the specimen; row 0
// for every position with one row, else the row of the position (objective.py:420-435).
struct TiltArgs {
  const float* rows;     // [n_tilts][6]
  const float* grid;     // [2][W]: x ramp, y ramp (imaginary parts of objective.py:303-307)
  const int* seq;
  int single, W;
};

__device__ __forceinline__ const float* tilt_row(const TiltArgs& t, int b) {
  return t.rows + (t.single ? 0 : (size_t)t.seq[b] * 6);
}

// real-space tilt mask exp(x_grid tan_x + y_grid tan_y) at pixel u, columns c, c + 1 of the
// row (objective.py:465, 491): the purely imaginary complex64 grids times float32 tangents,
// summed in float32
__device__ __forceinline__ float2 tilt_mask_at(const TiltArgs& t, const float* row, int col, int u) {
  const int y = u / t.W, x = u % t.W;
  const float th = __fadd_rn(__fmul_rn(t.grid[x], row[col + 1]), __fmul_rn(t.grid[t.W + y], row[col]));
  float s, c;
  sincosf(th, &s, &c);
  return make_float2(c, s);
}

// x[b][k] *= mask (conj(mask)) with the tilt columns col (0 before, 4 after)
// grid (WW / EB, nper, Bn)
__global__ void var_tilt_mul_kernel(float2* __restrict__ x, TiltArgs t, int nper, int col, int conj) {
  const int u = blockIdx.x * EB + threadIdx.x, k = blockIdx.y, b = blockIdx.z;
  const int WW = t.W * t.W;
  const float2 m = tilt_mask_at(t, tilt_row(t, b), col, u);
  float2* q = x + ((size_t)b * nper + k) * WW + u;
  *q = conj ? cmulc(*q, m) : cmul(*q, m);
}

struct PropArgs {
  const float* mask;
  float distance, wavelength, px, py, edge_mult, defocus, cs;
  int W;
  const float* defoci;   // per-position near-field defocus [N] (device), or nullptr: defocus
};

// propagator of the position's inside tilt (objective.py:482-484), or its edge power
// (multislice_core.py:72-73), computed as tables_kernel / var_tables_kernel do
__device__ __forceinline__ float2 tilted_prop(const PropArgs& a, const float* row, int u, bool edge) {
  const int W = a.W, ky = u / W, kx = u % W;
  const float qx = fftfreq_f32(kx, W, a.px), qy = fftfreq_f32(ky, W, a.py);
  const float q2 = __fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy));
  const float tilt = __fmul_rn(2.0f, __fadd_rn(__fmul_rn(qx, row[3]), __fmul_rn(qy, row[2])));
  const float x = __fadd_rn(__fmul_rn(a.wavelength, q2), tilt);
  const float phase = __fmul_rn(__fmul_rn(-3.141592654f, a.distance), x);
  const float mk = a.mask[u];
  float s, c;
  sincosf(phase, &s, &c);
  float2 p = make_float2(c * mk, s * mk);
  if (edge) {
    const float r = sqrtf(p.x * p.x + p.y * p.y);
    float2 pe = make_float2(0.f, 0.f);
    if (r > 0.f) {
      const float ang = atan2f(p.y, p.x) * a.edge_mult;
      const float re = powf(r, a.edge_mult);
      float se, ce;
      sincosf(ang, &se, &ce);
      pe = make_float2(re * ce, re * se);
    }
    p = pe;
  }
  return p;
}

// near-field CTF of the position's inside tilt (objective.py:505)
__device__ __forceinline__ float2 tilted_ctf(const PropArgs& a, const float* row, int u, float defocus) {
  const int W = a.W, ky = u / W, kx = u % W;
  const float qx = fftfreq_f32(kx, W, a.px), qy = fftfreq_f32(ky, W, a.py);
  const float q2 = __fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy));
  const float tilt = __fmul_rn(2.0f, __fadd_rn(__fmul_rn(qx, row[3]), __fmul_rn(qy, row[2])));
  const float x = __fadd_rn(__fmul_rn(a.wavelength, q2), tilt);
  const float l3 = __fmul_rn(__fmul_rn(a.wavelength, a.wavelength), a.wavelength);
  const float sph = __fmul_rn(__fmul_rn(__fmul_rn(0.5f, a.cs), l3), __fmul_rn(q2, q2));
  const float phase = __fmul_rn(-3.141592654f, __fadd_rn(__fmul_rn(x, defocus), sph));
  const float mk = a.mask[u];
  float s, c;
  sincosf(phase, &s, &c);
  return make_float2(c * mk, s * mk);
}

// x[b][k] *= P_b (conj: conj(P_b)) * scale; ctf selects the near-field CTF instead of the
// propagator   grid (WW / EB, nper, Bn)
__global__ void var_tilted_mul_kernel(float2* __restrict__ x, TiltArgs t, PropArgs a, int nper, int edge, int ctf,
                                      int conj, float scale) {
  const int u = blockIdx.x * EB + threadIdx.x, k = blockIdx.y, b = blockIdx.z;
  const int WW = a.W * a.W;
  const float* row = tilt_row(t, b);
  const float df = a.defoci ? a.defoci[t.seq[b]] : a.defocus;
  const float2 P = cscale(ctf ? tilted_ctf(a, row, u, df) : tilted_prop(a, row, u, edge != 0), scale);
  float2* q = x + ((size_t)b * nper + k) * WW + u;
  *q = conj ? cmulc(*q, P) : cmul(*q, P);
}

// per-position propagators (and their edge powers) of one batch, tabulated once and used by
// every propagation step of the batch   grid (WW / EB, Bn)
__global__ void var_pos_prop_table_kernel(TiltArgs t, PropArgs a, float2* __restrict__ tab,
                                          float2* __restrict__ tab_edge) {
  const int u = blockIdx.x * EB + threadIdx.x, b = blockIdx.y;
  const size_t WW = (size_t)a.W * a.W;
  const float* row = tilt_row(t, b);
  tab[b * WW + u] = tilted_prop(a, row, u, false);
  if (tab_edge) tab_edge[b * WW + u] = tilted_prop(a, row, u, true);
}

// x[b][k] *= tab[b] (conj: conj(tab[b]))   grid (WW / EB, nper, Bn)
__global__ void var_pos_table_mul_kernel(float2* __restrict__ x, const float2* __restrict__ tab, int nper, int WW,
                                         int conj) {
  const int u = blockIdx.x * EB + threadIdx.x, k = blockIdx.y, b = blockIdx.z;
  const float2 P = tab[(size_t)b * WW + u];
  float2* q = x + ((size_t)b * nper + k) * WW + u;
  *q = conj ? cmulc(*q, P) : cmul(*q, P);
}

// spec[b][p][u] *= the position's shift ramp   grid (WW / EB, Mp, Bn)
__global__ void var_ramp_mul_kernel(float2* __restrict__ spec, const float* __restrict__ sx, const float* __restrict__ sy,
                                    const float* __restrict__ mask, const float* __restrict__ corr,
                                    const int* __restrict__ seq, int W, int Mp) {
  const int u = blockIdx.x * EB + threadIdx.x, p = blockIdx.y, b = blockIdx.z;
  const int gi = seq[b];
  float2* q = spec + ((size_t)b * Mp + p) * W * W + u;
  *q = cmul(*q, ramp(sx, sy, u / W, u % W, mask[u], corr[2 * gi], corr[2 * gi + 1]));
}

// inside-tilt gradient terms of one propagation step (multislice_core.py:178-182):
// part[b] += sh * sum_u (qy, qx) Im(sum_k conj(F_k) G_k), F = FFT(psi O) of the forward step,
// G = the adjoint wave's spectrum times conj(P)   grid Bn, block 1024
__global__ void __launch_bounds__(1024) var_inside_tilt_kernel(const float2* __restrict__ G, const float2* __restrict__ F,
                                                               int nm, int W, float px, float py, double sh,
                                                               double* __restrict__ part) {
  __shared__ double red[64];
  const int b = blockIdx.x, WW = W * W;
  double gy = 0.0, gx = 0.0;
  for (int u = threadIdx.x; u < WW; u += blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    for (int k = 0; k < nm; ++k) {
      const size_t i = ((size_t)b * nm + k) * WW + u;
      acc = cadd(acc, cmulc(G[i], F[i]));   // conj(F) G
    }
    const float qx = fftfreq_f32(u % W, W, px), qy = fftfreq_f32(u / W, W, py);
    gy += (double)(qy * acc.y);
    gx += (double)(qx * acc.y);
  }
  block_sum2(gy, gx, red);
  if (threadIdx.x == 0) {
    part[(size_t)b * 6 + 2] += sh * gy;
    part[(size_t)b * 6 + 3] += sh * gx;
  }
}

// near-field inside-tilt gradient (objective.py:605-619): rsc * defocus * sum (qy, qx)
// Im(FWG conj(FFT(exit)))   grid Bn, block 1024
__global__ void __launch_bounds__(1024) var_near_tilt_kernel(const float2* __restrict__ FWG, const float2* __restrict__ FE,
                                                             int nm, int W, float px, float py, float defocus,
                                                             const float* __restrict__ defoci,
                                                             const int* __restrict__ seq, double rsc,
                                                             double* __restrict__ part) {
  __shared__ double red[64];
  const int b = blockIdx.x, WW = W * W;
  if (defoci) defocus = defoci[seq[b]];
  double gy = 0.0, gx = 0.0;
  for (int u = threadIdx.x; u < WW; u += blockDim.x) {
    float im = 0.0f;
    for (int k = 0; k < nm; ++k) {
      const size_t i = ((size_t)b * nm + k) * WW + u;
      im += cmulc(FWG[i], FE[i]).y;
    }
    const float qx = fftfreq_f32(u % W, W, px), qy = fftfreq_f32(u / W, W, py);
    gy += (double)(im * qy * defocus);
    gx += (double)(im * qx * defocus);
  }
  block_sum2(gy, gx, red);
  if (threadIdx.x == 0) {
    part[(size_t)b * 6 + 2] += rsc * gy;
    part[(size_t)b * 6 + 3] += rsc * gx;
  }
}

// adjoint of a real-space tilt mask and its gradient (objective.py:620-634 after the
// specimen, 660-673 before it): x *= conj(mask); with grad, sum over modes and pixels of
// Re(-2 x conj(ref) * i grid) into part[b][col], part[b][col + 1] (y, x). xcol0: the x grid's
// first column for every x (the reference's indexing for one probe mode before the specimen)
// grid Bn, block 1024
__global__ void __launch_bounds__(1024) var_tilt_adj_kernel(float2* __restrict__ x, const float2* __restrict__ ref,
                                                            TiltArgs t, int nper, int col, int grad, int xcol0,
                                                            double* __restrict__ part) {
  __shared__ double red[64];
  const int b = blockIdx.x, W = t.W, WW = W * W;
  const float* row = tilt_row(t, b);
  double gy = 0.0, gx = 0.0;
  for (int u = threadIdx.x; u < WW; u += blockDim.x) {
    const float2 m = tilt_mask_at(t, row, col, u);
    const float yg = t.grid[W + u / W], xg = t.grid[xcol0 ? 0 : u % W];
    for (int k = 0; k < nper; ++k) {
      const size_t i = ((size_t)b * nper + k) * WW + u;
      const float2 v = cmulc(x[i], m);
      x[i] = v;
      if (grad) {
        // kern = -2 v conj(ref); Re(kern * i g) = -g Im(kern) = 2 g Im(v conj(ref))
        const float im = cmulc(v, ref[i]).y;
        gy += (double)(2.0f * yg * im);
        gx += (double)(2.0f * xg * im);
      }
    }
  }
  if (!grad) return;
  block_sum2(gy, gx, red);
  if (threadIdx.x == 0) {
    part[(size_t)b * 6 + col] = gy;
    part[(size_t)b * 6 + col + 1] = gx;
  }
}

// tilt gradient rows from the per-position partials, in sequence order
// (objective.py:616-619, 635-639, 668-673; multislice_core.py:181-182)   one block
__global__ void var_tilt_finalize_kernel(const double* __restrict__ part, const int* __restrict__ seq, int nseq,
                                         int n_rows, int single, int use_before, int use_inside, int use_after,
                                         float* __restrict__ grad) {
  if (threadIdx.x != 0) return;
  for (int i = 0; i < n_rows * 6; ++i) grad[i] = 0.0f;
  for (int s = 0; s < nseq; ++s) {
    float* g = grad + (single ? 0 : (size_t)seq[s] * 6);
    const double* pp = part + (size_t)s * 6;
    for (int c = 0; c < 6; ++c) {
      const bool on = c < 2 ? use_before : (c < 4 ? use_inside : use_after);
      if (!on) continue;
      // before / after: one row sums the positions, per-position rows are assigned; inside
      // terms accumulate
      if (single || (c >= 2 && c < 4)) g[c] += (float)pp[c];
      else g[c] = (float)pp[c];
    }
  }
}

// ------------------------------------------------------------------ plan
struct LPlan {
  int W, WW, Ny, Nx, Z, Mo, Mp, N, nseq, Bb, zm, ntx, nty, ntiles, chunk, nchunk, engine;
  size_t o_pos, o_corr, o_seq, o_tab_pyx, o_mask, o_mask_sc, o_prop, o_prop_edge, o_sx, o_sy, o_planes, o_pf;
  size_t o_obj, o_grad, o_ob, o_tmp, o_dob, o_stack, o_psi, o_psi2, o_pb, o_pbs, o_partial, o_lists, o_counts;
  size_t o_loss_part, o_pos_part, o_dft, dft_bytes, total;
  int per_step;     // per-slice distances: one propagator table per step
  size_t o_steps;
  int S;            // probe scenarios (1: one probe)
  // variants (pty_loss_and_direction_variants)
  int near, compressed, nmask, n_abs, n_sets, has_bc, step_static;
  size_t o_ctf, o_abasis, o_abidx, o_ibuf, o_coef, o_dco, o_bc_part, o_ab_part, o_sbg;
  // beam tilts
  int n_rows, single_tilt, same_prop, before, after, inside_grad, step_tilts;
  int pos_prop;   // per-position propagator tables (per-position inside tilts that apply)
  size_t o_tilts, o_tgrid, o_spec, o_fexit, o_exitb, o_pbt, o_pft, o_tpart, o_pprop, o_pprop_edge;
};

inline LPlan make_lplan(const pty_problem_t* p, int engine, const pty_variant_t* v = nullptr) {
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
  q.S = (v && v->n_probe_scenarios > 1) ? v->n_probe_scenarios : 1;
  q.o_planes = take((size_t)q.S * q.Mp * WWs * c8);
  q.o_pf = take((size_t)q.S * q.Mp * WWs * c8);
  q.o_obj = take((size_t)q.zm * q.Ny * q.Nx * c8);
  q.o_grad = take((size_t)q.zm * q.Ny * q.Nx * c8);
  const size_t nobw = (size_t)q.Bb * q.zm, nwave = (size_t)q.Bb * q.Mp * q.Mo;
  q.o_ob = take(nobw * WWs * c8);
  q.o_tmp = take(nobw * WWs * c8);
  q.o_dob = take(nobw * WWs * c8);
  q.o_stack = take((size_t)q.Z * nwave * WWs * c8);
  q.o_psi = take(nwave * WWs * c8);
  q.o_psi2 = take(nwave * WWs * c8);
  // pb / pbs also carry the S x Mp probe-gradient planes at the end
  const size_t npb = (size_t)(q.Bb > q.S ? q.Bb : q.S) * q.Mp;
  q.o_pb = take(npb * WWs * c8);
  q.o_pbs = take(npb * WWs * c8);
  q.o_partial = take((size_t)q.nchunk * q.S * q.Mp * WWs * c8);
  q.o_lists = take((size_t)q.ntiles * q.Bb * sizeof(int));
  q.o_counts = take((size_t)q.ntiles * sizeof(int));
  q.o_loss_part = take((size_t)q.nseq * 2 * sizeof(double));
  q.o_pos_part = take((size_t)q.nseq * q.Mp * 2 * sizeof(double));
  q.per_step = p->slice_distances && q.Z > 1;
  q.o_steps = take(q.per_step ? (size_t)(q.Z - 1) * WWs * c8 : 0);
  if (v) {
    q.near = v->recon_type == 1;
    q.compressed = p->algorithm >= PTY_LSQ_COMPRESSED;
    q.nmask = q.compressed ? v->n_masks : 0;
    q.n_abs = v->aberrations ? v->n_aberrations : 0;
    q.n_sets = v->aberrations ? v->n_aberration_sets : 0;
    q.has_bc = v->beam_current != nullptr;
    q.o_ctf = take(q.near ? WWs * c8 : 0);
    q.o_abasis = take((size_t)q.n_abs * WWs * sizeof(float));
    q.o_abidx = take((size_t)3 * q.n_abs * sizeof(int));
    q.o_ibuf = take((size_t)q.Bb * WWs * sizeof(float));
    q.o_coef = take((size_t)q.Bb * q.nmask * sizeof(float));
    q.o_dco = take((size_t)q.Bb * q.nmask * sizeof(float));
    q.o_bc_part = take(q.has_bc ? (size_t)q.nseq * q.Mp * sizeof(double) : 0);
    q.o_ab_part = take((size_t)q.nseq * q.Mp * q.n_abs * sizeof(double));
    q.step_static = v->static_background && v->step_static_background;
    q.o_sbg = take(q.step_static ? WWs * sizeof(double) : 0);
    const int tm = v->n_tilts > 0 ? v->tilt_mode : 0;
    q.n_rows = v->n_tilts > 0 ? v->n_tilts : 1;
    q.single_tilt = q.n_rows == 1;
    q.same_prop = q.single_tilt || tm == 1 || tm == 2;   // objective.py:330, 482
    q.before = tm == 2 || tm == 4;
    q.after = tm == 1 || tm == 3 || tm == 4;
    q.step_tilts = v->n_tilts > 0 && v->step_tilts && v->tilts_grad;
    q.inside_grad = q.step_tilts && (tm == 0 || tm == 3 || tm == 4);
    q.o_tilts = take((size_t)q.n_rows * 6 * sizeof(float));
    q.o_tgrid = take((size_t)2 * q.W * sizeof(float));
    q.o_spec = take(q.inside_grad && q.Z > 1 ? (size_t)(q.Z - 1) * nwave * WWs * c8 : 0);
    q.o_fexit = take(q.inside_grad && q.near ? nwave * WWs * c8 : 0);
    q.o_exitb = take(q.after ? nwave * WWs * c8 : 0);
    q.o_pbt = take(q.before ? (size_t)q.Bb * q.Mp * WWs * c8 : 0);
    // spectra of the tilted probes the shift is applied to (no plates): the position gradient's
    // probe spectrum (objective.py:471, 651)
    q.o_pft = take(q.before && p->probe_shift && !q.n_abs ? (size_t)q.Bb * q.Mp * WWs * c8 : 0);
    q.o_tpart = take((size_t)q.nseq * 6 * sizeof(double));
    const bool edge = p->edge_mult > 1.0f && q.Z > 1;
    // with per-slice distances the reference builds every step's propagator from the batch's
    // own inside tilts, in every tilt mode (multislice_core.py:69-71)
    q.pos_prop = !q.same_prop || (q.per_step && !q.single_tilt);
    q.o_pprop = take(q.pos_prop ? (size_t)q.Bb * WWs * c8 : 0);
    q.o_pprop_edge = take(q.pos_prop && edge ? (size_t)q.Bb * WWs * c8 : 0);
  }
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

// float32 division on the host (IEEE round to nearest, as the reference's float32 arithmetic)
inline float fdiv_host(float a, float b) {
  volatile float r = a / b;
  return r;
}

// Krivanek (n, m, a/b) order of the first n aberrations (pypty/utils.py:1272-1308):
// kind 0 for m = 0, 1 for the cos (a) term, 2 for the sin (b) term
inline void krivanek_order(int n_abs, int* n_out, int* m_out, int* kind_out) {
  int i = 0;
  for (int n = 1; i < n_abs; ++n)
    for (int m = (n + 1) % 2; m <= n + 1 && i < n_abs; m += 2) {
      if (m == 0) {
        n_out[i] = n, m_out[i] = 0, kind_out[i] = 0, ++i;
      } else {
        n_out[i] = n, m_out[i] = m, kind_out[i] = 1, ++i;
        if (i < n_abs) n_out[i] = n, m_out[i] = m, kind_out[i] = 2, ++i;
      }
    }
}

struct Run {
  const pty_problem_t* p;
  LPlan q;
  void* ws;
  cudaStream_t st;
  const pty_variant_t* v = nullptr;
  TableArgs ta{};

  int dft(const float2* in, float2* out, long long nwin, int inverse) {
    if (nwin <= 0) return PTY_OK;
    if (q.engine == PTY_DFT_BF16X3 || q.engine == PTY_DFT_BF16X6)
      return tc_fft2(in, out, nwin, q.W, inverse, q.engine == PTY_DFT_BF16X3 ? 2 : 3, at<void>(ws, q.o_dft),
                     q.dft_bytes, st);
    // the FP32 engine's twiddle tables are built by the first transform of the call and reused
    float2* tw = at<float2>(ws, q.o_dft);
    const int build = tw_built ? 0 : 1;
    tw_built = true;
    if (q.W == 64) return run_fft2<64>(in, out, (int)nwin, inverse, 0, tw, st, build);
    if (q.W == 128) return run_fft2<128>(in, out, (int)nwin, inverse, 0, tw, st, build);
    return run_fft2<256>(in, out, (int)nwin, inverse, 0, tw, st, build);
  }
  bool tw_built = false;

  // the tensor-core engines' error word (set when a bounded wait ran out in any transform of
  // the call; the loss then comes back NaN), or nullptr for the FP32 engine
  int* tc_err() {
    if (q.engine != PTY_DFT_BF16X3 && q.engine != PTY_DFT_BF16X6) return nullptr;
    return tc_err_word(at<void>(ws, q.o_dft), q.W, q.engine == PTY_DFT_BF16X3 ? 2 : 3);
  }

  // the FP32 engine's twiddle tables (the 128-point ones for 256 px windows), built once per call
  float2* fp32_twiddles() {
    float2* tw = at<float2>(ws, q.o_dft);
    if (!tw_built) {
      prof_mark(st, KID_TWIDDLES);
      if (q.W == 64) build_twiddles_kernel<64><<<1, 256, 0, st>>>(tw);
      else build_twiddles_kernel<128><<<1, 256, 0, st>>>(tw);
      tw_built = true;
    }
    return tw;
  }

  // one forward step of the batch in one pass (FP32 engine, 64 / 128 px windows)
  int fwd_prop(const float2* pin, size_t pin_stride, float2* psi, float2* stack, const float2* ob, int z, int Bn,
               const float2* tab, size_t tab_stride, float scale, float2* spec_out) {
    float2* tw = fp32_twiddles();
    if (q.W == 256)
      return layered_fwd256(pin, pin_stride, psi, stack, ob, z, q.Z, q.Mp, q.Mo, Bn, tab, tab_stride, scale, tw, st);
    prof_mark(st, KID_FUSED);
    const unsigned nwin = (unsigned)(Bn * q.Mp * q.Mo);
    if (q.W == 64) {
      if (set_smem(fwd_prop_kernel<64>, Smem<64>::bytes)) return PTY_ERR_CUDA;
      fwd_prop_kernel<64><<<nwin, Geo<64>::T, Smem<64>::bytes, st>>>(pin, pin_stride, psi, stack, ob, z, q.Z, q.Mp,
                                                                     q.Mo, tab, tab_stride, scale, tw, spec_out);
    } else {
      if (set_smem(fwd_prop_kernel<128>, Smem<128>::bytes)) return PTY_ERR_CUDA;
      fwd_prop_kernel<128><<<nwin, Geo<128>::T, Smem<128>::bytes, st>>>(pin, pin_stride, psi, stack, ob, z, q.Z,
                                                                       q.Mp, q.Mo, tab, tab_stride, scale, tw,
                                                                       spec_out);
    }
    return cuda_status();
  }

  // x <- IFFT(FFT(x) * mask) for nwin windows (the band limit, objective.py:436-441,
  // multislice_core.py:189-191), in one pass on the FP32 engine for 64 / 128 px windows
  int band_limit(float2* x, float2* tmp, long long nwin) {
    if (q.engine == PTY_DFT_FP32_FFT && q.W == 256) return layered_step256(x, nwin, nullptr, 0, 1, 0, 1.0f, ta.mask_sc,
                                                                             fp32_twiddles(), st);
    if (q.engine == PTY_DFT_FP32_FFT && q.W <= 128) {
      float2* tw = fp32_twiddles();
      prof_mark(st, KID_FFT2);
      const float inv = 1.0f / (float)q.WW;
      if (q.W == 64) {
        if (set_smem(prop_step_kernel<64>, Smem<64>::bytes)) return PTY_ERR_CUDA;
        prop_step_kernel<64><<<(unsigned)nwin, Geo<64>::T, Smem<64>::bytes, st>>>(x, x, nullptr, 0, 1, 0, inv, tw,
                                                                                 ta.mask);
      } else {
        if (set_smem(prop_step_kernel<128>, Smem<128>::bytes)) return PTY_ERR_CUDA;
        prop_step_kernel<128><<<(unsigned)nwin, Geo<128>::T, Smem<128>::bytes, st>>>(x, x, nullptr, 0, 1, 0, inv, tw,
                                                                                    ta.mask);
      }
      return cuda_status();
    }
    int rc;
    if ((rc = dft(x, tmp, nwin, 0))) return rc;
    prof_mark(st, KID_ELEMENTWISE);
    mask_kernel<<<grid((int)nwin, 1), EB, 0, st>>>(tmp, ta.mask, q.WW);
    return dft(tmp, x, nwin, 1);
  }

  // psi <- IFFT(FFT(psi) * P) through psi2 (or in one pass on the FP32 engine for 64 / 128 px
  // windows): the table per group of nper windows, tab_stride apart, 1/W^2 folded in or not.
  // keep_g: psi2 holds FFT(psi) * P afterwards (with the unfolded P), as the separate passes
  // leave it
  int prop_step(float2* psi, float2* psi2, long long nwin, const float2* tab, size_t tab_stride, int nper,
                int conj, bool folded, bool keep_g = false) {
    const float WWf = (float)q.WW;
    if (q.engine == PTY_DFT_FP32_FFT && q.W == 256 && !keep_g)   // the folded cluster exchange
      return layered_step256(psi, nwin, tab, tab_stride, nper, conj, folded ? 1.0f : 1.0f / WWf, nullptr,
                             fp32_twiddles(), st);
    if (q.engine == PTY_DFT_FP32_FFT && q.W <= 128) {
      float2* tw = fp32_twiddles();
      prof_mark(st, KID_FFT2);
      const float scale = folded ? 1.0f : 1.0f / WWf;
      float2* gout = keep_g ? psi2 : nullptr;
      const float gscale = folded ? WWf : 1.0f;
      if (q.W == 64) {
        if (set_smem(prop_step_kernel<64>, Smem<64>::bytes)) return PTY_ERR_CUDA;
        prop_step_kernel<64><<<(unsigned)nwin, Geo<64>::T, Smem<64>::bytes, st>>>(psi, psi, tab, tab_stride, nper,
                                                                                 conj, scale, tw, nullptr, gout,
                                                                                 gscale);
      } else {
        if (set_smem(prop_step_kernel<128>, Smem<128>::bytes)) return PTY_ERR_CUDA;
        prop_step_kernel<128><<<(unsigned)nwin, Geo<128>::T, Smem<128>::bytes, st>>>(psi, psi, tab, tab_stride,
                                                                                    nper, conj, scale, tw, nullptr,
                                                                                    gout, gscale);
      }
      return cuda_status();
    }
    int rc;
    if ((rc = dft(psi, psi2, nwin, 0))) return rc;
    prof_mark(st, KID_ELEMENTWISE);
    if (tab_stride == 0)
      prop_kernel<<<grid((int)nwin, 1), EB, 0, st>>>(psi2, tab, q.WW, conj, folded ? WWf : 1.0f);
    else
      var_pos_table_mul_kernel<<<grid(nper, (int)(nwin / nper)), EB, 0, st>>>(psi2, tab, nper, q.WW, conj);
    return dft(psi2, psi, nwin, 1);
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
    if (int* e = tc_err())   // cleared once per call: a failure in any transform of the call stays set
      if (cudaMemsetAsync(e, 0, sizeof(int), st) != cudaSuccess) return PTY_ERR_CUDA;
    prof_mark(st, KID_TABLES);
    if (W == 64) tables_kernel<64><<<(WW + 255) / 256, 256, 0, st>>>(ta);
    else if (W == 128) tables_kernel<128><<<(WW + 255) / 256, 256, 0, st>>>(ta);
    else tables_kernel<256><<<(WW + 255) / 256, 256, 0, st>>>(ta);
    if (v) {
      VarTableArgs va{};
      va.prop = ta.prop;
      va.prop_edge = ta.prop_edge;
      va.ctf = at<float2>(ws, q.o_ctf);
      va.abasis = at<float>(ws, q.o_abasis);
      va.mask = ta.mask;
      int* abidx = at<int>(ws, q.o_abidx);
      if (q.n_abs > 0) {
        int host[3 * 64];
        if (q.n_abs > 64) return PTY_ERR_UNSUPPORTED;
        krivanek_order(q.n_abs, host, host + q.n_abs, host + 2 * q.n_abs);
        if (cudaMemcpyAsync(abidx, host, (size_t)3 * q.n_abs * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess)
          return PTY_ERR_CUDA;
      }
      va.abn = abidx;
      va.abm = abidx + q.n_abs;
      va.abk = abidx + 2 * q.n_abs;
      va.W = W;
      va.use_edge = ta.use_edge;
      va.near = q.near;
      va.n_abs = q.n_abs;
      va.px = p->pixel_size_x;
      va.py = p->pixel_size_y;
      va.distance = p->slice_distance;
      va.wavelength = p->wavelength;
      va.edge_mult = p->edge_mult;
      va.tan_x = v->tan_x;
      va.tan_y = v->tan_y;
      va.tgrid = at<float>(ws, q.o_tgrid);
      if (v->n_tilts > 0) {   // the shared propagator / CTF take row 0's inside tilt (objective.py:339-345)
        const bool dev_rows = v->tilts_device != nullptr;
        if (cudaMemcpyAsync(at<float>(ws, q.o_tilts), dev_rows ? v->tilts_device : v->tilts_host,
                            (size_t)q.n_rows * 6 * sizeof(float),
                            dev_rows ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st) != cudaSuccess)
          return PTY_ERR_CUDA;
        va.tilt_row = at<float>(ws, q.o_tilts);   // read on the device: no host copy of a trial point
      } else {   // one row holding the inside tilt, for the per-position CTF kernels
        const float row[6] = {0.0f, 0.0f, v->tan_y, v->tan_x, 0.0f, 0.0f};
        if (cudaMemcpyAsync(at<float>(ws, q.o_tilts), row, sizeof(row), cudaMemcpyHostToDevice, st) != cudaSuccess)
          return PTY_ERR_CUDA;
      }
      if (cudaMemsetAsync(at<double>(ws, q.o_tpart), 0, (size_t)q.nseq * 6 * sizeof(double), st) != cudaSuccess)
        return PTY_ERR_CUDA;
      if (q.step_static && cudaMemsetAsync(at<double>(ws, q.o_sbg), 0, (size_t)WW * sizeof(double), st) != cudaSuccess)
        return PTY_ERR_CUDA;
      va.defocus = v->defocus;
      va.cs = v->cs;
      var_tables_kernel<<<(WW + 255) / 256, 256, 0, st>>>(va);
    }
    // per-slice distances: one table per step with the shared inside tilt (multislice_core.py:69-74)
    float2* steps = at<float2>(ws, q.o_steps);
    if (q.per_step) {
      const float tx = v ? v->tan_x : 0.0f;
      const float ty = v ? v->tan_y : 0.0f;
      const float* row = (v && v->n_tilts > 0) ? at<float>(ws, q.o_tilts) : nullptr;   // row 0's inside tilt
      if (W == 64)
        launch_step_props<64>(ta.mask, p->slice_distances, q.Z - 1, ta.px, ta.py, ta.wavelength, ta.edge_mult,
                              ta.use_edge, tx, ty, steps, st, row);
      else if (W == 128)
        launch_step_props<128>(ta.mask, p->slice_distances, q.Z - 1, ta.px, ta.py, ta.wavelength, ta.edge_mult,
                               ta.use_edge, tx, ty, steps, st, row);
      else
        launch_step_props<256>(ta.mask, p->slice_distances, q.Z - 1, ta.px, ta.py, ta.wavelength, ta.edge_mult,
                               ta.use_edge, tx, ty, steps, st, row);
    }
    // distance of slice step z (the step from slice z to z + 1)
    auto step_distance = [&](int z) { return q.per_step ? p->slice_distances[z] : p->slice_distance; };
    float2* planes = at<float2>(ws, q.o_planes);
    float2* pf = at<float2>(ws, q.o_pf);
    prof_mark(st, KID_LAYOUT);
    probe_to_planes_s_kernel<<<dim3((unsigned)(WW / EB), (unsigned)q.Mp, (unsigned)q.S), EB, 0, st>>>(
        probe, planes, q.Mp, q.S, WW);
    if ((rc = dft(planes, pf, (long long)q.S * q.Mp, 0))) return rc;
    const int nyx = q.Ny * q.Nx;
    prof_mark(st, KID_OBJ_TO_SLICES);
    obj_to_slices_kernel<<<(nyx + 255) / 256, 256, 0, st>>>(obj, at<float2>(ws, q.o_obj), nyx, q.zm);
    const int* d_pos = at<int>(ws, q.o_pos);
    const float* d_corr = at<float>(ws, q.o_corr);
    float2 *ob = at<float2>(ws, q.o_ob), *tmp = at<float2>(ws, q.o_tmp), *dob = at<float2>(ws, q.o_dob);
    float2 *stack = at<float2>(ws, q.o_stack), *psi = at<float2>(ws, q.o_psi), *psi2 = at<float2>(ws, q.o_psi2);
    float2 *pb = at<float2>(ws, q.o_pb), *pbs = at<float2>(ws, q.o_pbs);
    const int nm = q.Mp * q.Mo;
    VarProbeArgs pa{};
    pa.pf = pf;
    pa.planes = planes;
    pa.sx = ta.sx;
    pa.sy = ta.sy;
    pa.mask = ta.mask;
    pa.corr = d_corr;
    pa.bc = v ? v->beam_current : nullptr;
    pa.abasis = at<float>(ws, q.o_abasis);
    pa.coefs = v ? v->aberrations : nullptr;
    pa.marker = v ? v->aberration_marker : nullptr;
    pa.W = W;
    pa.Mp = q.Mp;
    pa.shift = shift ? 1 : 0;
    pa.n_abs = q.n_abs;
    pa.n_sets = q.n_sets;
    pa.pmarker = q.S > 1 ? v->probe_marker : nullptr;
    pa.S = q.S;
    const bool var_probe = v && (shift || pa.bc || pa.coefs || q.before || q.S > 1);
    TiltArgs tg{};
    tg.rows = at<float>(ws, q.o_tilts);
    tg.grid = at<float>(ws, q.o_tgrid);
    tg.single = q.single_tilt;
    tg.W = W;
    PropArgs pr{};
    pr.mask = ta.mask;
    pr.distance = p->slice_distance;
    pr.wavelength = p->wavelength;
    pr.px = p->pixel_size_x;
    pr.py = p->pixel_size_y;
    pr.edge_mult = p->edge_mult;
    pr.defocus = v ? v->defocus : 0.0f;
    pr.cs = v ? v->cs : 0.0f;
    pr.defoci = v ? v->defocus_per_position : nullptr;
    pr.W = W;
    const bool tilted_prop = v && q.pos_prop;
    float2* spec = at<float2>(ws, q.o_spec);
    const size_t spec_stride = (size_t)q.Bb * nm * WWs;   // one forward step of the batch
    for (int i0 = 0, ib = 0; i0 < q.nseq; i0 += q.Bb, ++ib) {
      const int Bn = q.nseq - i0 < q.Bb ? q.nseq - i0 : q.Bb;
      const int* seq_b = at<int>(ws, q.o_seq) + i0;
      // object windows, band-limited (objective.py:436-441)
      prof_mark(st, KID_OBJECT_WINDOWS);
      gather_kernel<<<grid(q.zm, Bn), EB, 0, st>>>(at<float2>(ws, q.o_obj), ob, d_pos, seq_b, W, q.Ny, q.Nx, q.zm);
      if ((rc = band_limit(ob, tmp, (long long)Bn * q.zm))) return rc;
      // incoming probe per position (objective.py:469-476)
      const float2* pin = planes;
      size_t pin_stride = 0;
      pa.seq = seq_b;
      tg.seq = seq_b;
      float2* pprop = at<float2>(ws, q.o_pprop);
      float2* pprop_edge = ta.use_edge ? at<float2>(ws, q.o_pprop_edge) : nullptr;
      // the positions' propagators (objective.py:482-484): once per batch, or per step with
      // per-slice distances (multislice_core.py:69-74)
      auto pos_props = [&](int zstep) {
        PropArgs pz = pr;
        pz.distance = step_distance(zstep);
        prof_mark(st, KID_ELEMENTWISE);
        var_pos_prop_table_kernel<<<dim3((unsigned)(WW / EB), (unsigned)Bn), EB, 0, st>>>(
            tg, pz, pprop, (zstep == 0 && ta.use_edge) ? pprop_edge : nullptr);
      };
      if (tilted_prop && !q.per_step) pos_props(0);
      if (var_probe && q.before) {
        // the probe before the tilt (after beam current and plates), then the tilt mask, then
        // the shift: from the pre-plate spectrum with plates, else the tilted probe's
        // (objective.py:448-476)
        prof_mark(st, KID_ELEMENTWISE);
        float2* pbt = at<float2>(ws, q.o_pbt);
        VarProbeArgs p0 = pa;
        p0.shift = 0;
        var_probe_in_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(p0, p0.coefs ? pbs : pbt);
        if (p0.coefs && (rc = dft(pbs, pbt, (long long)Bn * q.Mp, 1))) return rc;
        if (cudaMemcpyAsync(pb, pbt, (size_t)Bn * q.Mp * WWs * sizeof(float2), cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess)
          return PTY_ERR_CUDA;
        var_tilt_mul_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(pb, tg, q.Mp, 0, 0);
        if (shift) {
          if (pa.coefs) {
            var_probe_in_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(pa, pbs);
          } else {
            if ((rc = dft(pb, pbs, (long long)Bn * q.Mp, 0))) return rc;
            if (cudaMemcpyAsync(at<float2>(ws, q.o_pft), pbs, (size_t)Bn * q.Mp * WWs * sizeof(float2),
                                cudaMemcpyDeviceToDevice, st) != cudaSuccess)
              return PTY_ERR_CUDA;
            var_ramp_mul_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(pbs, ta.sx, ta.sy, ta.mask, d_corr, seq_b, W, q.Mp);
          }
          if ((rc = dft(pbs, pb, (long long)Bn * q.Mp, 1))) return rc;
        }
        pin = pb;
        pin_stride = (size_t)q.Mp * WWs;
      } else if (var_probe) {
        prof_mark(st, KID_ELEMENTWISE);
        const bool spectral = shift || pa.coefs;
        var_probe_in_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(pa, spectral ? pbs : pb);
        if (spectral && (rc = dft(pbs, pb, (long long)Bn * q.Mp, 1))) return rc;
        pin = pb;
        pin_stride = (size_t)q.Mp * WWs;
      } else if (shift) {
        prof_mark(st, KID_ELEMENTWISE);
        probe_spec_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(pbs, pf, ta.sx, ta.sy, ta.mask, d_corr, seq_b, W, q.Mp);
        if ((rc = dft(pbs, pb, (long long)Bn * q.Mp, 1))) return rc;
        pin = pb;
        pin_stride = (size_t)q.Mp * WWs;
      }
      // forward multislice (multislice_core.py:61-82)
      // one-pass forward steps: the FP32 engine (at 256 px only where no step spectrum is kept)
      const bool one_pass = q.engine == PTY_DFT_FP32_FFT && !(W == 256 && v && q.inside_grad);
      for (int z = 0; z < q.Z; ++z) {
        if (z < q.Z - 1 && one_pass) {
          // slice, stack and propagation in one pass (multislice_core.py:61-80); FFT(psi O) kept
          // for the inside-tilt gradient
          if (tilted_prop && q.per_step) pos_props(z);
          const bool edge = z == 0 && ta.use_edge;
          const float2* tab = tilted_prop ? (edge ? pprop_edge : pprop)
                                          : (q.per_step ? steps + (size_t)z * WWs : (edge ? ta.prop_edge : ta.prop));
          const size_t tstride = tilted_prop ? WWs : 0;
          const float scale = tilted_prop ? 1.0f / (float)WW : 1.0f;
          float2* spec_out = (v && q.inside_grad) ? spec + z * spec_stride : nullptr;
          if ((rc = fwd_prop(pin, pin_stride, psi, stack, ob, z, Bn, tab, tstride, scale, spec_out))) return rc;
          continue;
        }
        prof_mark(st, KID_FUSED);
        fwd_slice_kernel<<<grid(nm, Bn), EB, 0, st>>>(pin, pin_stride, psi, stack, ob, z, q.Z, q.Mp, q.Mo, WW);
        if (z < q.Z - 1 && !(v && q.inside_grad)) {   // 256 px or the tensor-core engines
          if (tilted_prop && q.per_step) pos_props(z);
          const bool edge = z == 0 && ta.use_edge;
          if (tilted_prop)
            rc = prop_step(psi, psi2, (long long)Bn * nm, edge ? pprop_edge : pprop, WWs, nm, 0, false);
          else
            rc = prop_step(psi, psi2, (long long)Bn * nm,
                           q.per_step ? steps + (size_t)z * WWs : (edge ? ta.prop_edge : ta.prop), 0, 1, 0, true);
          if (rc) return rc;
        } else if (z < q.Z - 1) {   // separate transforms that keep the step's spectrum
          if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
          if (v && q.inside_grad &&   // FFT(psi O) of the step, for the inside-tilt gradient
              cudaMemcpyAsync(spec + z * spec_stride, psi2, (size_t)Bn * nm * WWs * sizeof(float2),
                              cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return PTY_ERR_CUDA;
          if (tilted_prop && q.per_step) pos_props(z);
          prof_mark(st, KID_ELEMENTWISE);
          if (tilted_prop)
            var_pos_table_mul_kernel<<<grid(nm, Bn), EB, 0, st>>>(psi2, (z == 0 && ta.use_edge) ? pprop_edge : pprop,
                                                                  nm, WW, 0);
          else
            prop_kernel<<<grid(Bn * nm, 1), EB, 0, st>>>(
                psi2, q.per_step ? steps + (size_t)z * WWs : ((z == 0 && ta.use_edge) ? ta.prop_edge : ta.prop), WW,
                0, unfold);
          if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
        }
      }
      if (v && q.after) {
        // tilt after the specimen (objective.py:490-499): one slice band-limits the exit first
        prof_mark(st, KID_ELEMENTWISE);
        if (q.Z == 1) {
          if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
          mask_kernel<<<grid(Bn * nm, 1), EB, 0, st>>>(psi2, ta.mask, WW);
          if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
        }
        if (cudaMemcpyAsync(at<float2>(ws, q.o_exitb), psi, (size_t)Bn * nm * WWs * sizeof(float2),
                            cudaMemcpyDeviceToDevice, st) != cudaSuccess)
          return PTY_ERR_CUDA;
        var_tilt_mul_kernel<<<grid(nm, Bn), EB, 0, st>>>(psi, tg, nm, 4, 0);
      }
      if (v && v->exit_waves &&   // the exit waves (objective.py:518-520, data_simulation_exitwave)
          cudaMemcpyAsync(static_cast<float2*>(v->exit_waves) + (size_t)i0 * nm * WWs, psi,
                          (size_t)Bn * nm * WWs * sizeof(float2), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return PTY_ERR_CUDA;
      // far field, loss, dL/dPsi (objective.py:501-597)
      if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
      if (v && q.inside_grad && q.near &&   // FFT(exit) for the near-field inside-tilt gradient
          cudaMemcpyAsync(at<float2>(ws, q.o_fexit), psi2, (size_t)Bn * nm * WWs * sizeof(float2),
                          cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return PTY_ERR_CUDA;
      if (!v) {
        prof_mark(st, KID_FINALIZE);
        loss_kernel<<<Bn, 1024, 0, st>>>(psi2, ta.mask, measured, seq_b, W, q.Mp, q.Mo, p->algorithm,
                                         p->loss_weight * (float)WW, at<double>(ws, q.o_loss_part) + 2 * i0);
        if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
      } else if ((rc = variant_loss(psi, psi2, measured, seq_b, Bn, i0, tg, pr))) {
        return rc;
      }
      double* tpart = at<double>(ws, q.o_tpart) + (size_t)i0 * 6;
      if (v && q.after) {
        // adjoint of the tilt after the specimen and its gradient (objective.py:620-639)
        prof_mark(st, KID_ELEMENTWISE);
        var_tilt_adj_kernel<<<Bn, 1024, 0, st>>>(psi, at<float2>(ws, q.o_exitb), tg, nm, 4, q.step_tilts, 0, tpart);
        if (q.Z == 1) {
          if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
          mask_kernel<<<grid(Bn * nm, 1), EB, 0, st>>>(psi2, ta.mask, WW);
          if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
        }
      }
      // adjoint multislice (multislice_core.py:158-200)
      for (int z = q.Z - 1; z >= 0; --z) {
        prof_mark(st, KID_FUSED);
        adj_slice_kernel<<<grid(q.Mo, Bn), EB, 0, st>>>(psi, stack, ob, dob, z, q.Z, q.Mp, q.Mo, WW);
        if (z > 0) {
          // adjoint propagation (multislice_core.py:164-183); psi2 keeps FFT(g) conj(P) for the
          // inside-tilt gradient
          const bool edge = z == 1 && ta.use_edge;
          const bool keep = v && q.inside_grad;
          if (tilted_prop && q.per_step) pos_props(z - 1);
          if (tilted_prop)
            rc = prop_step(psi, psi2, (long long)Bn * nm, edge ? pprop_edge : pprop, WWs, nm, 1, false, keep);
          else
            rc = prop_step(psi, psi2, (long long)Bn * nm,
                           q.per_step ? steps + (size_t)(z - 1) * WWs : (edge ? ta.prop_edge : ta.prop), 0, 1, 1,
                           true, keep);
          if (rc) return rc;
          if (keep) {
            // sh = -4 pi d / W^2 in float32, d (the step's distance) times the edge multiplier on
            // the thick step (multislice_core.py:164-180)
            const float dist = edge ? step_distance(z - 1) * p->edge_mult : step_distance(z - 1);
            const float shf = fdiv_host((float)-12.566370614359172 * dist, (float)WW);
            prof_mark(st, KID_ELEMENTWISE);
            var_inside_tilt_kernel<<<Bn, 1024, 0, st>>>(psi2, spec + (size_t)(z - 1) * spec_stride, nm, W,
                                                        p->pixel_size_x, p->pixel_size_y, (double)shf, tpart);
          }
        }
      }
      if (p->step_obj) {
        // band-limited gradient windows (multislice_core.py:189-191), deterministic scatter
        if ((rc = band_limit(dob, tmp, (long long)Bn * q.zm))) return rc;
        int* lists = at<int>(ws, q.o_lists);
        int* counts = at<int>(ws, q.o_counts);
        prof_mark(st, KID_TILE_LISTS);
        tile_lists_kernel<<<q.ntiles, 256, 0, st>>>(d_pos, seq_b, Bn, W, q.ntx, lists, counts);
        prof_mark(st, KID_SCATTER);
        scatter_tiles_kernel<<<dim3(q.ntiles, q.zm), dim3(32, 8), 0, st>>>(
            dob, d_pos, seq_b, lists, counts, at<float2>(ws, q.o_grad), Bn, W, q.Ny, q.Nx, q.ntx, q.zm, ib > 0);
      }
      const bool step_bc = v && v->beam_current && v->step_beam_current;
      const bool step_ab = v && v->aberrations && v->step_aberrations;
      const bool step_tb = v && q.before && q.step_tilts;
      if (p->step_probe || p->step_pos || step_bc || step_ab || step_tb) {
        // probe-gradient spectra with the shift adjoint and the position gradient (objective.py:641-703)
        prof_mark(st, KID_PROBE_PARTIAL);
        probe_sum_kernel<<<grid(q.Mp, Bn), EB, 0, st>>>(psi, pbs, q.Mp, q.Mo, WW);
        if ((rc = dft(pbs, pb, (long long)Bn * q.Mp, 0))) return rc;
        prof_mark(st, KID_ELEMENTWISE);
        double* pos_part = at<double>(ws, q.o_pos_part) + (size_t)i0 * q.Mp * 2;
        double* bc_part = at<double>(ws, q.o_bc_part) + (size_t)i0 * q.Mp;
        double* ab_part = at<double>(ws, q.o_ab_part) + (size_t)i0 * q.Mp * q.n_abs;
        if (var_probe && q.before) {
          // shift adjoint, then the tilt adjoint in real space (objective.py:660-673), then
          // plates and beam current
          VarProbeArgs p1 = pa;
          if (shift && !pa.coefs) p1.pspec = at<float2>(ws, q.o_pft);
          var_probe_adj_kernel<<<dim3(q.Mp, Bn), 1024, 0, st>>>(pb, p1, p->step_pos, step_bc, step_ab,
                                                                p->step_probe, 1, 0, pos_part, bc_part, ab_part);
          if ((rc = dft(pb, pbs, (long long)Bn * q.Mp, 1))) return rc;
          var_tilt_adj_kernel<<<Bn, 1024, 0, st>>>(pbs, at<float2>(ws, q.o_pbt), tg, q.Mp, 0, q.step_tilts,
                                                   q.Mp == 1, tpart);
          if ((rc = dft(pbs, pb, (long long)Bn * q.Mp, 0))) return rc;
          var_probe_adj_kernel<<<dim3(q.Mp, Bn), 1024, 0, st>>>(pb, pa, p->step_pos, step_bc, step_ab,
                                                                p->step_probe, 0, 1, pos_part, bc_part, ab_part);
        } else if (var_probe)
          var_probe_adj_kernel<<<dim3(q.Mp, Bn), 1024, 0, st>>>(pb, pa, p->step_pos, step_bc, step_ab,
                                                                p->step_probe, 1, 1, pos_part, bc_part, ab_part);
        else if (shift)
          probe_adj_kernel<<<dim3(q.Mp, Bn), 1024, 0, st>>>(pb, pf, ta.sx, ta.sy, ta.mask, d_corr, seq_b, W, q.Mp,
                                                           p->step_pos, at<double>(ws, q.o_pos_part) + (size_t)i0 * q.Mp * 2);
        if (p->step_probe) {
          const int nch = (Bn + q.chunk - 1) / q.chunk;
          prof_mark(st, KID_PROBE_PARTIAL);
          if (q.S > 1)
            probe_partial_s_kernel<<<dim3((unsigned)((WW + 255) / 256), (unsigned)(q.Mp * q.S), nch), 256, 0, st>>>(
                pb, at<float2>(ws, q.o_partial), Bn, q.Mp, q.S, WW, q.chunk, ib > 0 ? 1 : 0, pa.pmarker, seq_b);
          else
            probe_partial_kernel<<<dim3((unsigned)((WW + 255) / 256), q.Mp, nch), 256, 0, st>>>(
                pb, at<float2>(ws, q.o_partial), Bn, q.Mp, WW, q.chunk, ib > 0 ? 1 : 0);
        }
      }
    }
    // probe gradient: IFFT(mask * sum_b spectra) (objective.py:703, 927-933)
    if (p->step_probe) {
      prof_mark(st, KID_PROBE_FINAL);
      probe_total_kernel<<<grid(q.Mp * q.S, 1), EB, 0, st>>>(at<float2>(ws, q.o_partial), q.nchunk, q.Mp * q.S,
                                                             ta.mask, pbs, WW);
      if ((rc = dft(pbs, pb, (long long)q.Mp * q.S, 1))) return rc;
      prof_mark(st, KID_LAYOUT);
      planes_to_probe_s_kernel<<<dim3((unsigned)(WW / EB), (unsigned)q.Mp, (unsigned)q.S), EB, 0, st>>>(
          pb, probe_grad, q.Mp, q.S, WW);
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
                                               p->step_pos && shift, tc_err(), loss_sse, pos_grad);
    if (v && q.step_tilts)
      var_tilt_finalize_kernel<<<1, 32, 0, st>>>(at<double>(ws, q.o_tpart), at<int>(ws, q.o_seq), q.nseq, q.n_rows,
                                                 q.single_tilt, q.before, q.inside_grad, q.after, v->tilts_grad);
    if (v && q.step_static)
      var_static_final_kernel<<<(WW + 255) / 256, 256, 0, st>>>(at<double>(ws, q.o_sbg), WW,
                                                               v->static_background_grad);
    if (v && ((v->beam_current && v->step_beam_current) || (v->aberrations && v->step_aberrations))) {
      const bool gb = v->beam_current && v->step_beam_current, ga = v->aberrations && v->step_aberrations;
      var_finalize_kernel<<<1, 256, 0, st>>>(at<double>(ws, q.o_bc_part), at<double>(ws, q.o_ab_part),
                                             at<int>(ws, q.o_seq), q.nseq, q.Mp, W, q.N, v->beam_current,
                                             gb ? v->beam_current_grad : nullptr, q.n_sets, q.n_abs,
                                             v->aberration_marker, ga ? v->aberrations_grad : nullptr);
    }
    prof_mark(st, -1);
    return cuda_status();
  }

  // pattern, loss and dL/d(exit wave) of one batch for the variant branches: psi2 holds the
  // spectra of the exit waves; on return psi holds dL/d(exit wave) (objective.py:501-604)
  int variant_loss(float2* psi, float2* psi2, const float* measured, const int* seq_b, int Bn, int i0,
                   const TiltArgs& tg, const PropArgs& pr) {
    int rc;
    const int W = q.W, WW = q.WW, nm = q.Mp * q.Mo;
    float* ibuf = at<float>(ws, q.o_ibuf);
    double* lpart = at<double>(ws, q.o_loss_part) + 2 * (size_t)i0;
    const float2* ctf = at<float2>(ws, q.o_ctf);
    float2* field = psi2;
    prof_mark(st, KID_FINALIZE);
    if (q.near) {   // wave = IFFT(FFT(exit) * CTF) (objective.py:506-508)
      if (q.single_tilt && !v->defocus_per_position)
        prop_kernel<<<grid(Bn * nm, 1), EB, 0, st>>>(psi2, ctf, WW, 0, 1.0f);
      else   // the position's inside tilt
        var_tilted_mul_kernel<<<grid(nm, Bn), EB, 0, st>>>(psi2, tg, pr, nm, 0, 1, 0, 1.0f);
      if ((rc = dft(psi2, psi, (long long)Bn * nm, 1))) return rc;
      field = psi;
    }
    prof_mark(st, KID_FINALIZE);
    var_intensity_kernel<<<dim3((unsigned)(WW / EB), (unsigned)Bn), EB, 0, st>>>(field, ta.mask, ibuf, W, nm, q.near);
    if (v->static_background)
      var_add_static_kernel<<<dim3((unsigned)(WW / EB), (unsigned)Bn), EB, 0, st>>>(ibuf, v->static_background, ta.mask,
                                                                                    W);
    if (q.compressed) {
      float* coef = at<float>(ws, q.o_coef);
      float* dco = at<float>(ws, q.o_dco);
      var_coef_kernel<<<dim3((unsigned)q.nmask, (unsigned)Bn), 256, 0, st>>>(ibuf, v->masks, WW, q.nmask, coef);
      var_closs_kernel<<<Bn, 32, 0, st>>>(coef, measured, seq_b, q.nmask, p->algorithm, dco, lpart);
      var_cdldi_kernel<<<dim3((unsigned)(WW / EB), (unsigned)Bn), EB, 0, st>>>(ibuf, v->masks, dco, WW, q.nmask, nm);
    } else {
      MeasPrep mp{W, v->data_pad, v->use_padded_intensity != 0, v->shift_y, v->shift_x,
                  v->data_multiplier == 0.0f ? 1.0f : v->data_multiplier,
                  v->upsample_pattern > 1 ? v->upsample_pattern : 1};
      var_pixel_loss_kernel<<<Bn, 1024, 0, st>>>(ibuf, measured, seq_b, mp, nm, p->algorithm, lpart);
    }
    if (q.step_static)
      var_static_grad_kernel<<<(WW + 255) / 256, 256, 0, st>>>(ibuf, v->static_background, Bn, WW, p->loss_weight,
                                                              at<double>(ws, q.o_sbg));
    var_apply_kernel<<<grid(nm, Bn), EB, 0, st>>>(field, ibuf, ta.mask, W, nm, q.near, p->loss_weight * (float)WW);
    if (q.near) {   // dL/d(exit) = IFFT(loss_weight FFT(wave dL/dI) conj(CTF)) (objective.py:602-604)
      if ((rc = dft(psi, psi2, (long long)Bn * nm, 0))) return rc;
      prof_mark(st, KID_ELEMENTWISE);
      if (q.single_tilt && !v->defocus_per_position)
        prop_kernel<<<grid(Bn * nm, 1), EB, 0, st>>>(psi2, ctf, WW, 1, p->loss_weight);
      else
        var_tilted_mul_kernel<<<grid(nm, Bn), EB, 0, st>>>(psi2, tg, pr, nm, 0, 1, 1, p->loss_weight);
      if (q.inside_grad)   // near-field inside-tilt gradient (objective.py:605-619)
        var_near_tilt_kernel<<<Bn, 1024, 0, st>>>(psi2, at<float2>(ws, q.o_fexit), nm, W, p->pixel_size_x,
                                                  p->pixel_size_y, v->defocus, v->defocus_per_position, seq_b,
                                                  -12.566370614359172 / (double)WW,
                                                  at<double>(ws, q.o_tpart) + (size_t)i0 * 6);
    }
    return dft(psi2, psi, (long long)Bn * nm, 1);
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

namespace {

// the problem with a compressed algorithm mapped onto a pixel one for the shared checks
int validate_variant(const pty_problem_t* p, const pty_variant_t* v) {
  if (!p || !v) return PTY_ERR_INVALID;
  pty_problem_t base = *p;
  const bool compressed = p->algorithm >= PTY_LSQ_COMPRESSED && p->algorithm <= PTY_POISSON_COMPRESSED;
  if (compressed) base.algorithm = PTY_LSQ;
  int rc = validate(&base);
  if (rc) return rc;
  if (v->recon_type != 0 && v->recon_type != 1) return PTY_ERR_UNSUPPORTED;
  if (v->data_pad < 0 || 2 * v->data_pad >= p->window) return PTY_ERR_INVALID;
  if (compressed && v->data_pad != 0) return PTY_ERR_UNSUPPORTED;
  if (v->n_tilts < 0 ||
      (v->n_tilts > 0 && ((!v->tilts_host && !v->tilts_device) || (v->n_tilts != 1 && v->n_tilts != p->n_positions))))
    return PTY_ERR_INVALID;
  if (v->n_tilts > 0 && (v->tilt_mode < 0 || v->tilt_mode > 4)) return PTY_ERR_UNSUPPORTED;
  if (compressed && (v->n_masks <= 0 || !v->masks)) return PTY_ERR_INVALID;
  if (v->beam_current && v->step_beam_current && !v->beam_current_grad) return PTY_ERR_INVALID;
  if (v->aberrations) {
    if (v->n_aberrations <= 0 || v->n_aberrations > 64 || v->n_aberration_sets <= 0 || !v->aberration_marker)
      return PTY_ERR_INVALID;
    if (v->step_aberrations && !v->aberrations_grad) return PTY_ERR_INVALID;
  }
  // detector upsampling: the cropped pattern side must be a multiple of the factor (the
  // reference's repeat / pad back to W fails otherwise); the compressed losses take masks at
  // the model pattern's size
  const int up = v->upsample_pattern > 1 ? v->upsample_pattern : 1;
  if (v->upsample_pattern < 0) return PTY_ERR_INVALID;
  const int S = v->use_padded_intensity ? p->window : p->window - 2 * v->data_pad;
  if (up > 1 && (compressed || S % up != 0)) return PTY_ERR_UNSUPPORTED;
  if (up > 1 && S / up - 2 * (v->use_padded_intensity ? v->data_pad / up : 0) <= 0) return PTY_ERR_INVALID;
  // static background: W x W, added to the full pattern (the reference's shapes only
  // broadcast without a crop and without upsampling)
  if (v->static_background && (S != p->window || up > 1)) return PTY_ERR_UNSUPPORTED;
  if (v->static_background && v->step_static_background && !v->static_background_grad) return PTY_ERR_INVALID;
  if (v->n_probe_scenarios < 0 || (v->n_probe_scenarios > 1 && !v->probe_marker)) return PTY_ERR_INVALID;
  return PTY_OK;
}

}  // namespace

extern "C" {

int pty_variants_workspace_bytes(const pty_problem_t* problem, const pty_variant_t* variant, size_t* bytes) {
  int rc = validate_variant(problem, variant);
  if (rc) return rc;
  if (!bytes) return PTY_ERR_INVALID;
  *bytes = lay::make_lplan(problem, PTY_DFT_FP32_FFT, variant).total;
  return PTY_OK;
}

int pty_loss_and_direction_variants(const pty_problem_t* problem, const pty_variant_t* variant, const void* obj,
                                    const void* probe, const int32_t* positions_host, const float* pos_correction,
                                    const int32_t* sequence_host, const float* measured, double* loss_sse,
                                    void* object_grad, void* probe_grad, float* pos_grad, void* workspace,
                                    size_t workspace_bytes, void* stream) {
  int rc = validate_variant(problem, variant);
  if (rc) return rc;
  if (!obj || !probe || !positions_host || !sequence_host || !measured || !loss_sse || !workspace)
    return PTY_ERR_INVALID;
  if ((problem->step_obj && !object_grad) || (problem->step_probe && !probe_grad) || (problem->step_pos && !pos_grad))
    return PTY_ERR_INVALID;
  if ((rc = check_geometry(problem, positions_host, sequence_host))) return rc;
  const lay::LPlan q = lay::make_lplan(problem, PTY_DFT_FP32_FFT, variant);
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
  lay::Run r{problem, q, workspace, st, variant};
  return r.run(static_cast<const float2*>(obj), static_cast<const float2*>(probe), measured, loss_sse,
               static_cast<float2*>(object_grad), static_cast<float2*>(probe_grad), pos_grad);
}

}  // extern "C"

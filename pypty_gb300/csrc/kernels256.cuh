// Kernels of the loss-and-gradient path for 256 x 256 windows: every window is a cluster of
// 4 blocks (window_fft256.cuh). The probe and object modes of a position are processed one
// after another inside that cluster, so the mode sums (intensity, probe-mode sum of the
// object gradient, object-mode sum of the probe gradient) are plain ordered accumulations
// in shared or global memory: deterministic, no cross-cluster reduction.
#pragma once
#include "ptycho_kernels.cuh"
#include "window_fft256.cuh"

namespace pty {

// element-pair (16-byte) helpers on one block's native part: no whole-window temporaries,
// so the window stays the only large register array
__device__ __forceinline__ void st_native128_conj(float2* base, const float2 (&v)[32]) {
  float4* p = reinterpret_cast<float4*>(base);
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 16; ++j) p[j * 512 + t] = make_float4(v[2 * j].x, -v[2 * j].y, v[2 * j + 1].x, -v[2 * j + 1].y);
}

// v *= w (conj_w: v *= conj(w)) for w in native order at base
__device__ __forceinline__ void mul_native128(float2 (&v)[32], const float2* base, bool conj_w) {
  const float4* p = reinterpret_cast<const float4*>(base);
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float4 q = p[j * 512 + t];
    const float2 w0 = make_float2(q.x, q.y), w1 = make_float2(q.z, q.w);
    v[2 * j] = conj_w ? cmulc(v[2 * j], w0) : cmul(v[2 * j], w0);
    v[2 * j + 1] = conj_w ? cmulc(v[2 * j + 1], w1) : cmul(v[2 * j + 1], w1);
    if ((j & 7) == 7) asm volatile("" ::: "memory");
  }
}

// out = (accumulate ? out : 0) + a * v with a, out in native order
__device__ __forceinline__ void madd_native128(float2* out, const float2* a_, const float2 (&v)[32], bool accumulate) {
  float4* o = reinterpret_cast<float4*>(out);
  const float4* a = reinterpret_cast<const float4*>(a_);
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float4 q = a[j * 512 + t];
    float2 g0 = cmul(make_float2(q.x, q.y), v[2 * j]);
    float2 g1 = cmul(make_float2(q.z, q.w), v[2 * j + 1]);
    if (accumulate) {
      const float4 r = o[j * 512 + t];
      g0 = cadd(make_float2(r.x, r.y), g0);
      g1 = cadd(make_float2(r.z, r.w), g1);
    }
    o[j * 512 + t] = make_float4(g0.x, g0.y, g1.x, g1.y);
    if ((j & 3) == 3) asm volatile("" ::: "memory");   // bound the loads in flight
  }
}

// v += w (native order)
__device__ __forceinline__ void add_native128(float2 (&v)[32], const float2* base) {
  const float4* p = reinterpret_cast<const float4*>(base);
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float4 q = p[j * 512 + t];
    v[2 * j] = cadd(v[2 * j], make_float2(q.x, q.y));
    v[2 * j + 1] = cadd(v[2 * j + 1], make_float2(q.z, q.w));
  }
}

// shared memory of the 256 kernels (per block)
struct Smem256 {
  using G = Geo<128>;
  static constexpr size_t xbuf_off = 0;
  static constexpr size_t tw1_off = xbuf_off + sizeof(float2) * G::XBUF;
  static constexpr size_t tw2_off = tw1_off + sizeof(float2) * G::TW1;
  static constexpr size_t tw256_off = tw2_off + sizeof(float2) * G::TW2;
  static constexpr size_t red_off = tw256_off + sizeof(float2) * 256;
  static constexpr size_t small = red_off + sizeof(double) * 72;              // FFT-only kernels
  static constexpr size_t pyx_off = small;
  static constexpr size_t bits_off = pyx_off + sizeof(float2) * 512;
  static constexpr size_t acc_off = bits_off + sizeof(uint32_t) * G::T * 4;
  static constexpr size_t fused = acc_off + sizeof(float) * G::XBUF;         // the fused kernel
};

struct Carve256 {
  float2 *xbuf, *tw1, *tw2, *tw256;
  double* red;
  __device__ explicit Carve256(unsigned char* smem) {
    xbuf = reinterpret_cast<float2*>(smem + Smem256::xbuf_off);
    tw1 = reinterpret_cast<float2*>(smem + Smem256::tw1_off);
    tw2 = reinterpret_cast<float2*>(smem + Smem256::tw2_off);
    tw256 = reinterpret_cast<float2*>(smem + Smem256::tw256_off);
    red = reinterpret_cast<double*>(smem + Smem256::red_off);
  }
};

// ------------------------------------------------------------------ probe spectrum
// probe (256, 256, Mp) reference layout -> FFT per mode; grid = Mp * 4, cluster of 4
__global__ void __launch_bounds__(512, 1) probe_fft256_kernel(const float2* __restrict__ probe, int Mp,
                                                             const float2* __restrict__ g_tw,
                                                             float2* __restrict__ probe_f) {
  using G = Geo256;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x, p = blockIdx.x / 4;
  load_twiddles<128>(s.tw1, s.tw2, g_tw);
  load_tw256(s.tw256);
  __syncthreads();
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = probe[(size_t)(G::ry(c, t) * 256 + G::rx(c, t, i)) * Mp + p];
  WinFFT256::forward(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
  st_native<128>(probe_f + (size_t)p * 65536 + c * G::PART, v);
}

// ------------------------------------------------------------------ object windows
// gather + band limit; grid = Bb * zm * 4, cluster of 4
__global__ void __launch_bounds__(512, 1) object_windows256_kernel(WindowArgs a) {
  using G = Geo256;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  const int win = blockIdx.x / 4, b = win / a.zm, k = win % a.zm;
  load_twiddles<128>(s.tw1, s.tw2, a.tw);
  load_tw256(s.tw256);
  const int gi = a.seq[b];
  const int y0 = a.pos[2 * gi], x0 = a.pos[2 * gi + 1];
  const float2* src = a.obj + (size_t)k * a.Ny * a.Nx + (size_t)(y0 + G::ry(c, t)) * a.Nx + x0;
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = src[G::rx(c, t, i)];
  __syncthreads();
  WinFFT256::band_limit(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl, a.mask_sc);
  st_native<128>(a.out + (size_t)win * 65536 + c * G::PART, v);
}

// ------------------------------------------------------------------ gradient windows
// band limit of the summed gradient window, native in, natural (y, x) out, in place
__global__ void __launch_bounds__(512, 1) grad_windows256_kernel(float2* buf, const float* __restrict__ mask_sc,
                                                                const float2* __restrict__ g_tw) {
  using G = Geo256;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  float2* win = buf + (size_t)(blockIdx.x / 4) * 65536;
  load_twiddles<128>(s.tw1, s.tw2, g_tw);
  load_tw256(s.tw256);
  float2 v[32];
  ld_native<128>(win + c * G::PART, v);
  __syncthreads();
  // the cluster barriers inside the transforms order every block's reads before any write
  WinFFT256::band_limit(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl, mask_sc);
#pragma unroll
  for (int i = 0; i < 32; ++i) win[G::ry(c, t) * 256 + G::rx(c, t, i)] = v[i];
}

// ------------------------------------------------------------------ probe gradient
__global__ void __launch_bounds__(512, 1) probe_final256_kernel(const float2* __restrict__ partial, int nchunk, int Mp,
                                                               const float* __restrict__ mask_sc,
                                                               const float2* __restrict__ g_tw,
                                                               float2* __restrict__ probe_grad) {
  using G = Geo256;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x, p = blockIdx.x / 4;
  load_twiddles<128>(s.tw1, s.tw2, g_tw);
  load_tw256(s.tw256);
  __syncthreads();
  // chunks outer, elements inner: each chunk's 32 loads are in flight together (the chunk
  // order of every element's sum is unchanged)
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = make_float2(0.f, 0.f);
  for (int ch = 0; ch < nchunk; ++ch) {
    const float2* src = partial + ((size_t)ch * Mp + p) * 65536 + c * G::PART;
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = cadd(v[i], src[nidx<128>(i, t)]);
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = cscale(v[i], mask_sc[G::fky(c, t, i) * 256 + G::fkx(c, t, i)]);
  WinFFT256::inverse(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
#pragma unroll
  for (int i = 0; i < 32; ++i) probe_grad[(size_t)(G::ry(c, t) * 256 + G::rx(c, t, i)) * Mp + p] = v[i];
}

// ------------------------------------------------------------------ plain batched FFT
__global__ void __launch_bounds__(512, 1) fft2_batch256_kernel(const float2* __restrict__ in, float2* __restrict__ out,
                                                              int inverse, int shift, const float2* __restrict__ g_tw) {
  using G = Geo256;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  load_twiddles<128>(s.tw1, s.tw2, g_tw);
  load_tw256(s.tw256);
  __syncthreads();
  const float2* src = in + (size_t)(blockIdx.x / 4) * 65536;
  float2* dst = out + (size_t)(blockIdx.x / 4) * 65536;
  const int h = shift ? 128 : 0;
  float2 v[32];
  if (!inverse) {
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = src[G::ry(c, t) * 256 + G::rx(c, t, i)];
    WinFFT256::forward(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
#pragma unroll
    for (int i = 0; i < 32; ++i)
      dst[((G::fky(c, t, i) + h) & 255) * 256 + ((G::fkx(c, t, i) + h) & 255)] = v[i];
  } else {
    const float inv = 1.0f / 65536.0f;
#pragma unroll
    for (int i = 0; i < 32; ++i)
      v[i] = cscale(src[((G::fky(c, t, i) + h) & 255) * 256 + ((G::fkx(c, t, i) + h) & 255)], inv);
    WinFFT256::inverse(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
#pragma unroll
    for (int i = 0; i < 32; ++i) dst[G::ry(c, t) * 256 + G::rx(c, t, i)] = v[i];
  }
}

// ------------------------------------------------------------------ layered steps, 256
// One propagation step (P given, one table per group of nper windows, tab_stride apart) or,
// with rtab, one band limit by a real mask, of a batch of natural-layout 256-px windows in
// place: the folded butterfly-table-butterfly exchange of the fused kernel.   4 blocks / window
__global__ void __launch_bounds__(512, 1) layered_step256_kernel(float2* x, const float2* __restrict__ tab,
                                                                size_t tab_stride, int nper, int conj, float scale,
                                                                const float* __restrict__ rtab,
                                                                const float2* __restrict__ g_tw) {
  using G = Geo256;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  const size_t w = blockIdx.x / 4;
  float2* win = x + w * 65536;
  load_twiddles<128>(s.tw1, s.tw2, g_tw);
  load_tw256(s.tw256);
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = win[G::ry(c, t) * 256 + G::rx(c, t, i)];
  __syncthreads();
  // the cluster barriers inside the transforms order every block's reads before any write
  if (rtab)
    WinFFT256::band_limit(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl, rtab);
  else
    WinFFT256::propagate(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl, tab + (w / nper) * tab_stride, conj != 0, scale);
#pragma unroll
  for (int i = 0; i < 32; ++i) win[G::ry(c, t) * 256 + G::rx(c, t, i)] = v[i];
}

// One forward multislice step of the layered path for 256-px windows (multislice_core.py:61-80)
// in one pass: in = z == 0 ? the incoming probe (mode p) : psi; stack = conj(in);
// psi = IFFT(FFT(in * O[b][z][m]) * P) with the folded exchange.   4 blocks / window
__global__ void __launch_bounds__(512, 1) layered_fwd256_kernel(const float2* __restrict__ pin, size_t pin_stride,
                                                               float2* psi, float2* __restrict__ stack,
                                                               const float2* __restrict__ ob, int z, int Z, int Mp,
                                                               int Mo, const float2* __restrict__ tab,
                                                               size_t tab_stride, float scale,
                                                               const float2* __restrict__ g_tw) {
  using G = Geo256;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  const size_t WW = 65536;
  const int nm = Mp * Mo, wi = blockIdx.x / 4, b = wi / nm, pm = wi % nm, p = pm / Mo, m = pm % Mo;
  const float2* src = z == 0 ? pin + (size_t)b * pin_stride + (size_t)p * WW : psi + (size_t)wi * WW;
  float2* stw = stack + (((size_t)b * Z + z) * nm + pm) * WW;
  const float2* o = ob + (((size_t)b * Z + z) * Mo + m) * WW;
  load_twiddles<128>(s.tw1, s.tw2, g_tw);
  load_tw256(s.tw256);
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int u = G::ry(c, t) * 256 + G::rx(c, t, i);
    const float2 in = src[u];
    stw[u] = cconj(in);
    v[i] = cmul(in, o[u]);
  }
  __syncthreads();
  WinFFT256::propagate(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl, tab + (size_t)b * tab_stride, false, scale);
  float2* dst = psi + (size_t)wi * WW;
#pragma unroll
  for (int i = 0; i < 32; ++i) dst[G::ry(c, t) * 256 + G::rx(c, t, i)] = v[i];
}

// ------------------------------------------------------------------ fused multislice, 256
// One cluster of 4 blocks per position; modes one after another (forward: k = m*Mp + p
// ascending; adjoint: probe mode outer, object mode inner). Extra buffers (FusedArgs): psi
// [Bb][Mp*Mo] far-field waves, dldi [Bb] dL/dI (split passes), pgr [Bb][Mp] object-mode sum
// of the probe gradient (Mo > 1), seg [Bb][ckpt] recomputed waves and gpark [Bb] the parked
// adjoint wave (ckpt > 1).
//
// Per-slice recomputation: with ckpt = K > 1 the forward keeps conj(psi_z) only for
// z % K == 0; the adjoint, on reaching a segment [z0, zl], parks its wave, re-runs the
// forward from the checkpoint z0 (same arithmetic, so the same waves bit for bit) into seg,
// and reloads its wave. The stack then holds ceil(Z/K) instead of Z waves per mode.
//
// Steps form a small state machine, each "real-space op -> FFT -> frequency op -> inverse
// FFT" with the two transforms inlined once:
//   F_START  load the shifted probe           F_SLICE  * O_z, FFT, * P (or far field), IFFT
//   LOSS     dL/dI (no transform)             A_START  dL/dI * Psi_k -> IFFT
//   A_RECOMP segment recomputation            A_SLICE  gradient, * conj O_z, FFT, * conj P, IFFT
//
// The kernel is compiled twice: PH = 1 runs the forward stages and the loss and leaves dL/dI
// in dldi; PH = 2 starts from dldi and runs the adjoint stages. Each instance carries only
// its own stages' code and live state (the one-kernel state machine spilled ~400 B per
// thread; the two instances spill under 100 B). Propagation steps fold the forward cross
// butterfly, the propagator and the inverse cross butterfly into one cluster exchange
// (WinFFT256::cross_propagate).
enum Stage256 : int { F_START = 0, F_SLICE, S_LOSS, A_START, A_RECOMP, A_SLICE, S_DONE };

template <int PH>
__global__ void __launch_bounds__(512, 1) fused256_kernel(FusedArgs a) {
  static_assert(PH == 1 || PH == 2, "phase 1: forward + loss, phase 2: adjoint");
  constexpr bool FWD = PH == 1, ADJ = PH == 2;
  using G = Geo256;
  constexpr int T = G::T;
  constexpr size_t WW = 65536;
  constexpr size_t PART = G::PART;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  float2* spy = reinterpret_cast<float2*>(smem + Smem256::pyx_off);   // [256] y factor, [256] x factor
  const float2* spx = spy + 256;
  uint32_t* sbits = reinterpret_cast<uint32_t*>(smem + Smem256::bits_off);
  float* facc = reinterpret_cast<float*>(smem + Smem256::acc_off);     // I accumulator, then dL/dI
  double* xch = s.red + 64;                                            // cluster exchange slots
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  const int b = blockIdx.x / 4;
  const int Z = a.Z, Mp = a.Mp, Mo = a.Mo, nmodes = Mp * Mo;
  const bool store_stack = a.step_obj && !a.simulate;
  const int K = (a.ckpt > 1 && store_stack) ? a.ckpt : 1;   // no stack, nothing to recompute
  const int nck = (Z + K - 1) / K;
  load_twiddles<128>(s.tw1, s.tw2, a.tw);
  load_tw256(s.tw256);
  for (int i = t; i < 512; i += T) spy[i] = a.pyx[i];
  for (int q = 0; q < 4; ++q) {   // band-limit bits of this thread's elements in every quadrant
    uint32_t mb = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) mb |= (a.mask[G::fky(q, t, i) * 256 + G::fkx(q, t, i)] != 0.0f ? 1u : 0u) << i;
    sbits[q * T + t] = mb;
  }
  for (int i = 0; i < 32; ++i) facc[i * T + t] = 0.0f;
  const bool want_probe = a.step_probe || a.step_pos;
  auto part = [&](const float2* base, size_t win) { return base + win * WW + c * PART; };
  auto wpart = [&](float2* base, size_t win) { return base + win * WW + c * PART; };
  auto stack_win = [&](int z, int p, int m) { return (((size_t)b * nck + z / K) * Mp + p) * Mo + m; };

  int stage = FWD ? F_START : A_START, k = 0, z = 0, z0 = 0, zl = 0;
  if (ADJ) {
    for (int i = 0; i < 32; ++i) facc[i * T + t] = a.dldi[(size_t)b * WW + c * PART + i * T + t];
  }
  __syncthreads();

  float2 v[32];
  while (stage != S_DONE) {
    const bool fwd_stage = FWD;
    const int p = fwd_stage ? k % Mp : k / Mo;
    const int m = fwd_stage ? k / Mp : k % Mo;
    const int kidx = m * Mp + p;

    if (FWD && stage == S_LOSS) {
      // ------------------------------------------------ loss and dL/dI of this quadrant
      const int gi = a.seq[b];
      const float inv_modes = 1.0f / (float)nmodes;
      const float* meas = a.measured + (size_t)gi * WW;
      double lsum = 0.0, ssum = 0.0;
#pragma unroll 1
      for (int i = 0; i < 32; ++i) {
        const float acc = facc[i * T + t];
        const float I = (nmodes == 1) ? acc : acc * inv_modes;
        const int ky = G::fky(c, t, i), kx = G::fkx(c, t, i);
        const int didx = ((ky + 128) & 255) * 256 + ((kx + 128) & 255);
        if (a.simulate) {
          a.sim_out[(size_t)b * WW + didx] = I;
          continue;
        }
        float d = loss_pixel(a.algorithm, I, meas[didx], lsum, ssum);
        if (nmodes > 1) d = d / (float)nmodes;
        facc[i * T + t] = d;
      }
      if (a.simulate) return;
      block_sum2(lsum, ssum, s.red);
      if (t == 0) {
        xch[0] = lsum;
        xch[1] = ssum;
      }
      cl.sync();
      if (c == 0 && t == 0) {
        double l = 0.0, q = 0.0;
        for (int rr = 0; rr < 4; ++rr) {
          const double* rx = cl.map_shared_rank(xch, rr);
          l += rx[0];
          q += rx[1];
        }
        a.loss_part[2 * b] = l;
        a.loss_part[2 * b + 1] = q;
      }
      cl.sync();
      for (int i = 0; i < 32; ++i) a.dldi[(size_t)b * WW + c * PART + i * T + t] = facc[i * T + t];
      return;
    }

    // ------------------------------------------------ L2 prefetch of the next step's operands
    // (this block's part of each window), one FFT pair ahead of their loads
    if (t == 0) {
      constexpr uint32_t PB = (uint32_t)(PART * sizeof(float2));
      if (FWD) {
        const int zn = stage == F_START ? 0 : z + 1;
        if (zn < Z) prefetch_l2(part(a.obl, ((size_t)b * Z + zn) * Mo + m), PB);
      } else if (stage == A_SLICE || (stage == A_START && K == 1)) {
        const int zn = stage == A_START ? Z - 1 : z - 1;
        if (zn >= 0 && (K == 1 || zn >= z0)) {   // the next step stays in this segment
          prefetch_l2(part(a.obl, ((size_t)b * Z + zn) * Mo + m), PB);
          if (store_stack) {
            prefetch_l2(K == 1 ? part(a.stack, stack_win(zn, p, m)) : part(a.seg, (size_t)b * K + (zn - z0)), PB);
            if (p > 0) prefetch_l2(part(a.gsum, ((size_t)b * Z + zn) * Mo + m), PB);
          }
        }
      } else if (stage == A_RECOMP && z < zl) {
        prefetch_l2(part(a.obl, ((size_t)b * Z + z + 1) * Mo + m), PB);
      }
    }

    // ------------------------------------------------ real-space op
    bool do_fwd = false, do_inv = false, skip = false;
    if (FWD && stage == F_START) {
      ld_native<128>(part(a.fprobe, (size_t)b * Mp + p), v);   // the shifted incoming probe
    } else if (ADJ && stage == A_START) {
      do_inv = true;
    } else if (FWD) {   // F_SLICE
      if (store_stack && z % K == 0) st_native128_conj(wpart(a.stack, stack_win(z, p, m)), v);
      mul_native128(v, part(a.obl, ((size_t)b * Z + z) * Mo + m), false);
      do_fwd = true;
      do_inv = z < Z - 1;
    } else if (stage == A_RECOMP) {
      if (z == z0) {
        st_native<128>(wpart(a.gpark, b), v);                 // park the adjoint wave
        ld_native<128>(part(a.stack, stack_win(z0, p, m)), v);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = cconj(v[i]);     // the checkpoint holds conj(psi)
      }
      st_native128_conj(wpart(a.seg, (size_t)b * K + (z - z0)), v);
      if (z < zl) {
        mul_native128(v, part(a.obl, ((size_t)b * Z + z) * Mo + m), false);
        do_fwd = true;
        do_inv = true;
      } else {
        ld_native<128>(part(a.gpark, b), v);                  // the adjoint wave back
      }
    } else {   // A_SLICE
      if (store_stack) {
        // conj(psi_z) * g, summed over probe modes in order p = 0, 1, ... (multislice_core.py:186-188)
        const float2* src = K == 1 ? part(a.stack, stack_win(z, p, m)) : part(a.seg, (size_t)b * K + (z - z0));
        madd_native128(wpart(a.gsum, ((size_t)b * Z + z) * Mo + m), src, v, p > 0);
      }
      mul_native128(v, part(a.obl, ((size_t)b * Z + z) * Mo + m), true);
      if (z > 0) {
        do_fwd = true;
        do_inv = true;
      } else if (want_probe) {
        if (Mo > 1) {
          // sum over object modes (multislice_core.py:193-197), in order m = 0, 1, ...
          float2* pr = wpart(a.pgr, (size_t)b * Mp + p);
          if (m > 0) add_native128(v, pr);
          if (m < Mo - 1) {
            st_native<128>(pr, v);
            skip = true;
          }
        }
        // the probe-gradient wave; probe_spectrum256_kernel takes its spectrum
        if (!skip) st_native<128>(wpart(a.fprobe, (size_t)b * Mp + p), v);
      }
    }

    // ------------------------------------------------ transforms and frequency op
    // forward: twiddled sub-transform, then either the full cross butterfly or (propagation
    // steps) the folded butterfly-propagator-butterfly exchange; inverse: conjugate twiddle
    // and sub-transform. Each sub-transform is inlined once.
    const bool prop_step = do_fwd && do_inv;
    if (do_fwd) {
      WinFFT<128>::forward(v, s.xbuf, s.tw1, s.tw2);
      WinFFT256::twiddle(v, s.tw256, c, false);
    }
    if (prop_step) {
      // propagator (conjugated in the adjoint); the thick first slice uses the table
      const bool adjoint = ADJ && stage == A_SLICE;
      const int zstep = adjoint ? z - 1 : z;
      const bool edge = a.use_edge && zstep == 0;
      const bool tab = !a.use_sep || edge;
      const float2* pr = a.prop_steps ? a.prop_steps + (size_t)zstep * (256 * 256) : (edge ? a.prop_edge : a.prop);
      WinFFT256::cross_propagate(v, s.xbuf, cl, c, adjoint, [&](int i, int q) {
        const int ky = G::fky(q, t, i), kx = G::fkx(q, t, i);
        if (tab) return pr[ky * 256 + kx];
        return ((sbits[q * T + t] >> i) & 1u) ? cmul(spy[ky], spx[kx]) : make_float2(0.f, 0.f);
      });
    } else {
      // outside the propagation steps only the far field (forward) transforms forward: the
      // adjoint instance carries no copy of that butterfly
      if (FWD && do_fwd) WinFFT256::cross(v, s.xbuf, cl, c);
      if (ADJ && stage == A_START) {
        // dL/dPsi = dL/dI * Psi * w (objective.py:595-597)
        ld_native<128>(part(a.psi, (size_t)b * nmodes + kidx), v);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = cscale(cscale(v[i], facc[i * T + t]), a.loss_weight);
      } else if (FWD && stage == F_SLICE && z == Z - 1) {   // the exit plane
        // far field of this mode: Psi = FFT(exit) * mask; accumulate |Psi|^2
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          v[i] = cscale(v[i], a.mask[G::fky(c, t, i) * 256 + G::fkx(c, t, i)]);
          facc[i * T + t] += cabs2(v[i]);
        }
        if (!a.simulate) st_native<128>(wpart(a.psi, (size_t)b * nmodes + kidx), v);
      }
      if (do_inv) WinFFT256::cross(v, s.xbuf, cl, c);
    }
    if (do_inv) {
      WinFFT256::twiddle(v, s.tw256, c, true);
      WinFFT<128>::inverse(v, s.xbuf, s.tw1, s.tw2);
    }

    // ------------------------------------------------ next step
    if (FWD) {
      if (stage == F_START) {
        stage = F_SLICE;
        z = 0;
      } else if (z < Z - 1) {
        ++z;
      } else if (++k < nmodes) {
        stage = F_START;
      } else {
        stage = S_LOSS;
      }
    } else if (stage == A_START || (stage == A_SLICE && z > 0 && K > 1 && z == z0)) {
      // enter the segment below (from A_START: the top segment)
      zl = stage == A_START ? Z - 1 : z0 - 1;
      z0 = (zl / K) * K;
      if (K > 1) {
        stage = A_RECOMP;
        z = z0;
      } else {
        stage = A_SLICE;
        z = zl;
      }
    } else if (stage == A_RECOMP) {
      if (z < zl) {
        ++z;
      } else {
        stage = A_SLICE;
      }
    } else {   // A_SLICE
      if (z > 0) {
        --z;
      } else if (++k < nmodes) {
        stage = A_START;
      } else {
        stage = S_DONE;
      }
    }
  }
}


// ------------------------------------------------------------------ shifted incoming probes
// Real-space probe of every (position, probe mode): IFFT(FFT(P) * shift ramp * mask) / W^2
// (objective.py:469-476); without a shift the probe comes back unchanged (FFT(P) / W^2).
// Written to fprobe in native order for the forward stages; grid = Bn * Mp clusters of 4.
__global__ void __launch_bounds__(512, 1) shifted_probes256_kernel(FusedArgs a) {
  using G = Geo256;
  constexpr size_t WW = 65536;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  const int win = blockIdx.x / 4, b = win / a.Mp, p = win % a.Mp;
  load_twiddles<128>(s.tw1, s.tw2, a.tw);
  load_tw256(s.tw256);
  __syncthreads();
  const float2* pf = a.probe_f + (size_t)p * WW + c * G::PART;
  const float inv = 1.0f / (float)WW;
  const int gi = a.seq[b];
  const float dy = a.corr[2 * gi], dx = a.corr[2 * gi + 1];
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    float2 w = make_float2(inv, 0.f);
    if (a.probe_shift) {
      const int ky = G::fky(c, t, i), kx = G::fkx(c, t, i);
      const float mk = a.mask[ky * 256 + kx];
      const float th = __fadd_rn(__fmul_rn(__fmul_rn(a.sx[kx], mk), dx), __fmul_rn(__fmul_rn(a.sy[ky], mk), dy));
      float sn, cs;
      sincosf(th, &sn, &cs);
      w = make_float2(cs * mk * inv, sn * mk * inv);
    }
    v[i] = cmul(pf[nidx<128>(i, t)], w);
  }
  WinFFT256::inverse(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
  st_native<128>(a.fprobe + (size_t)win * WW + c * G::PART, v);
}

// ------------------------------------------------------------------ probe-gradient spectrum
// Spectrum of the probe-gradient wave of every (position, probe mode) that the adjoint left
// in fprobe (real space, native order), in place, with the shift adjoint and the position
// gradient (objective.py:641-656); grid = Bn * Mp clusters of 4.
__global__ void __launch_bounds__(512, 1) probe_spectrum256_kernel(FusedArgs a) {
  using G = Geo256;
  constexpr size_t WW = 65536;
  extern __shared__ __align__(16) unsigned char smem[];
  Carve256 s(smem);
  double* xch = s.red + 64;
  cg::cluster_group cl = cg::this_cluster();
  const int c = (int)cl.block_rank(), t = threadIdx.x;
  const int win = blockIdx.x / 4, b = win / a.Mp, p = win % a.Mp;
  load_twiddles<128>(s.tw1, s.tw2, a.tw);
  load_tw256(s.tw256);
  float2* dst = a.fprobe + (size_t)win * WW + c * G::PART;
  float2 v[32];
  ld_native<128>(dst, v);
  __syncthreads();
  WinFFT256::forward(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
  double gy = 0.0, gx = 0.0;
  if (a.probe_shift) {
    const float2* pf = a.probe_f + (size_t)p * WW + c * G::PART;
    const int gi = a.seq[b];
    const float dy = a.corr[2 * gi], dx = a.corr[2 * gi + 1];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int ky = G::fky(c, t, i), kx = G::fkx(c, t, i);
      const float mk = a.mask[ky * 256 + kx];
      const float th = __fadd_rn(__fmul_rn(__fmul_rn(a.sx[kx], mk), dx), __fmul_rn(__fmul_rn(a.sy[ky], mk), dy));
      float sn, cs;
      sincosf(th, &sn, &cs);
      v[i] = cmulc(v[i], make_float2(cs * mk, sn * mk));
      if (a.step_pos) {
        const float im = cmulc(v[i], pf[nidx<128>(i, t)]).y;
        gy += (double)(-(a.sy[ky] * mk) * im);
        gx += (double)(-(a.sx[kx] * mk) * im);
      }
    }
  }
  if (a.step_probe) st_native<128>(dst, v);
  if (a.step_pos) {
    block_sum2(gy, gx, s.red);
    if (t == 0) {
      xch[2] = gy;
      xch[3] = gx;
    }
    cl.sync();
    if (c == 0 && t == 0) {
      double sy_ = 0.0, sx_ = 0.0;
      for (int rr = 0; rr < 4; ++rr) {
        const double* rx = cl.map_shared_rank(xch, rr);
        sy_ += rx[2];
        sx_ += rx[3];
      }
      a.pos_part[(size_t)win * 2] = sy_;
      a.pos_part[(size_t)win * 2 + 1] = sx_;
    }
    cl.sync();
  }
}

}  // namespace pty

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
  static constexpr size_t acc_off = bits_off + sizeof(uint32_t) * G::T;
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
  WinFFT256::forward(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = cscale(v[i], a.mask_sc[G::fky(c, t, i) * 256 + G::fkx(c, t, i)]);
  WinFFT256::inverse(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
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
  WinFFT256::forward(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = cscale(v[i], mask_sc[G::fky(c, t, i) * 256 + G::fkx(c, t, i)]);
  WinFFT256::inverse(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
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
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    float2 acc = make_float2(0.f, 0.f);
    for (int ch = 0; ch < nchunk; ++ch)
      acc = cadd(acc, partial[((size_t)ch * Mp + p) * 65536 + c * G::PART + nidx<128>(i, t)]);
    v[i] = cscale(acc, mask_sc[G::fky(c, t, i) * 256 + G::fkx(c, t, i)]);
  }
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

// ------------------------------------------------------------------ fused multislice, 256
// One cluster of 4 blocks per position; modes k = m * Mp + p one after another.
// Extra buffers (FusedArgs): psi [Bb][Mp*Mo] far-field waves, dldi [Bb] dL/dI (split
// passes), pgr [Bb][Mp] real-space probe gradient summed over object modes (Mo > 1).
//
// The work is one flat loop of steps "real-space op -> FFT -> frequency op -> inverse FFT"
// (each transform inlined once):
//   forward, per mode k:   START (probe spectrum -> IFFT), SLICE z = 0..Z-1 (store conj psi,
//                          * O_z, FFT, * P, IFFT; the last slice ends with the far field)
//   LOSS                   dL/dI of the mode-mean intensity (no transform)
//   adjoint, per mode k:   ASTART (dL/dI * Psi_k -> IFFT), ASLICE z = Z-1..0 (gradient
//                          contribution, * conj O_z, FFT, * conj P, IFFT; after z = 0 the
//                          probe-gradient spectrum and the position gradient)
__global__ void __launch_bounds__(512, 1) fused256_kernel(FusedArgs a) {
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
  load_twiddles<128>(s.tw1, s.tw2, a.tw);
  load_tw256(s.tw256);
  for (int i = t; i < 512; i += T) spy[i] = a.pyx[i];
  {
    uint32_t mb = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) mb |= (a.mask[G::fky(c, t, i) * 256 + G::fkx(c, t, i)] != 0.0f ? 1u : 0u) << i;
    sbits[t] = mb;
  }
  for (int i = 0; i < 32; ++i) facc[i * T + t] = 0.0f;
  __syncthreads();
  const bool store_stack = a.step_obj && !a.simulate;
  const bool want_probe = a.step_probe || a.step_pos;
  auto part = [&](const float2* base, size_t win) { return base + win * WW + c * PART; };
  auto wpart = [&](float2* base, size_t win) { return base + win * WW + c * PART; };

  const int per_mode = Z + 1;
  const int n_fwd = nmodes * per_mode;           // steps [0, n_fwd): forward
  const int s_loss = n_fwd;                       // the loss step
  const int n_total = a.simulate ? n_fwd + 1 : n_fwd + 1 + nmodes * per_mode;
  int s_begin = 0, s_end = n_total;
  if (a.phase == 1) s_end = n_fwd + 1;
  if (a.phase == 2) {
    s_begin = n_fwd + 1;
    for (int i = 0; i < 32; ++i) facc[i * T + t] = a.dldi[(size_t)b * WW + c * PART + i * T + t];
    __syncthreads();
  }

  float2 v[32];
  for (int s_ = s_begin; s_ < s_end; ++s_) {
    // ------------------------------------------------ decode the step
    const bool is_loss = (s_ == s_loss);
    const bool fwd = s_ < s_loss;
    const int r = fwd ? s_ : s_ - s_loss - 1;
    const int kk = is_loss ? 0 : r / per_mode, j = is_loss ? 0 : r % per_mode;
    // forward: modes in order k = m*Mp + p; adjoint: probe mode outer, object mode inner
    const int p = fwd ? kk % Mp : kk / Mo;
    const int m = fwd ? kk / Mp : kk % Mo;
    const int k = m * Mp + p;
    const bool start = !is_loss && j == 0;
    const int z = fwd ? j - 1 : Z - j;        // slice of a SLICE / ASLICE step

    if (is_loss) {
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
      if (a.phase == 1) {
        for (int i = 0; i < 32; ++i) a.dldi[(size_t)b * WW + c * PART + i * T + t] = facc[i * T + t];
        return;
      }
      continue;
    }

    // ------------------------------------------------ real-space op
    bool do_fwd = false, do_inv = false;
    if (start) {
      do_inv = true;
    } else if (fwd) {
      if (store_stack) st_native128_conj(wpart(a.stack, (((size_t)b * Z + z) * Mp + p) * Mo + m), v);
      mul_native128(v, part(a.obl, ((size_t)b * Z + z) * Mo + m), false);
      do_fwd = true;
      do_inv = z < Z - 1;
    } else {
      if (store_stack) {
        // conj(psi_z) * g, summed over probe modes in order p = 0, 1, ... (multislice_core.py:186-188)
        madd_native128(wpart(a.gsum, ((size_t)b * Z + z) * Mo + m),
                       part(a.stack, (((size_t)b * Z + z) * Mp + p) * Mo + m), v, p > 0);
      }
      mul_native128(v, part(a.obl, ((size_t)b * Z + z) * Mo + m), true);
      if (z > 0) {
        do_fwd = true;
        do_inv = true;
      } else {
        if (!want_probe) continue;
        if (Mo > 1) {
          // sum over object modes (multislice_core.py:193-197), in order m = 0, 1, ...
          float2* pr = wpart(a.pgr, (size_t)b * Mp + p);
          if (m > 0) add_native128(v, pr);
          if (m < Mo - 1) {
            st_native<128>(pr, v);
            continue;
          }
        }
        do_fwd = true;   // probe-gradient spectrum
      }
    }

    // ------------------------------------------------ forward FFT
    if (do_fwd) WinFFT256::forward(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);

    // ------------------------------------------------ frequency op
    if (start && fwd) {
      // incoming probe: FFT(P) * shift ramp * mask / W^2 (objective.py:469-476); without a
      // shift the probe is taken back unchanged (FFT(P) / W^2)
      const float2* pf = part(a.probe_f, p);
      const float inv = 1.0f / (float)WW;
      const int gi = a.seq[b];
      const float dy = a.corr[2 * gi], dx = a.corr[2 * gi + 1];
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
    } else if (start) {
      // adjoint start: dL/dPsi = dL/dI * Psi * w (objective.py:595-597)
      ld_native<128>(part(a.psi, (size_t)b * nmodes + k), v);
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = cscale(cscale(v[i], facc[i * T + t]), a.loss_weight);
    } else if (fwd && z == Z - 1) {
      // far field of this mode: Psi = FFT(exit) * mask; accumulate |Psi|^2
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        v[i] = cscale(v[i], a.mask[G::fky(c, t, i) * 256 + G::fkx(c, t, i)]);
        facc[i * T + t] += cabs2(v[i]);
      }
      if (!a.simulate) st_native<128>(wpart(a.psi, (size_t)b * nmodes + k), v);
    } else if (do_inv) {
      // propagator (conjugated in the adjoint); the thick first slice uses the table
      const int zstep = fwd ? z : z - 1;
      const bool edge = a.use_edge && zstep == 0;
      if (a.use_sep && !edge) {
        const uint32_t mb = sbits[t];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float2 P = cmul(spy[G::fky(c, t, i)], spx[G::fkx(c, t, i)]);
          v[i] = ((mb >> i) & 1u) ? (fwd ? cmul(v[i], P) : cmulc(v[i], P)) : make_float2(0.f, 0.f);
        }
      } else {
        const float2* pr = edge ? a.prop_edge : a.prop;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float2 P = pr[G::fky(c, t, i) * 256 + G::fkx(c, t, i)];
          v[i] = fwd ? cmul(v[i], P) : cmulc(v[i], P);
        }
      }
    } else if (!fwd) {
      // probe-gradient spectrum with the shift adjoint, position gradient (objective.py:641-656)
      double gy = 0.0, gx = 0.0;
      if (a.probe_shift) {
        const float2* pf = part(a.probe_f, p);
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
      if (a.step_probe) st_native<128>(wpart(a.fprobe, (size_t)b * Mp + p), v);
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
          a.pos_part[((size_t)b * Mp + p) * 2] = sy_;
          a.pos_part[((size_t)b * Mp + p) * 2 + 1] = sx_;
        }
        cl.sync();
      }
    }

    // ------------------------------------------------ inverse FFT
    if (do_inv) WinFFT256::inverse(v, s.xbuf, s.tw1, s.tw2, s.tw256, cl);
  }
}

}  // namespace pty

// Kernels of the far-field multislice loss-and-gradient path (pypty objective /
// multislice_core restated for sm_103a). All kernels are templated on the window size W
// and use WinFFT<W> for their transforms. Windows that live only inside one call are
// stored in the "native" order of WinFFT (element i of thread t at offset i*T + t) so that
// every load/store of a window is a fully coalesced 256-byte warp access.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "window_fft.cuh"

namespace cg = cooperative_groups;

namespace pty {

enum Algorithm : int { ALG_LSQ_SQRT = 0, ALG_ML = 1, ALG_LSQ = 2, ALG_LSQ_SQRT_2 = 3 };

// Kernels that are not templates are declared static: each launch-path translation unit
// (one per window size) carries its own copy.

// ------------------------------------------------------------------ tables
// mask        exclude_mask_ishift of create_spatial_frequencies (pypty/utils.py:176-194)
// mask_sc     mask / W^2 (the ifft2 normalisation folded into the band limit; exact)
// prop        Fresnel propagator * mask / W^2 (pypty/objective.py:343), natural (ky,kx)
// prop_edge   prop^edge_mult / W^2 for the first slice step (multislice_core.py:73-74)
// sx, sy      float32(-6.2831855 * fftfreq(W)) : sub-pixel shift exponents
//             (pypty/objective.py:308-313), multiplied by mask where used
struct TableArgs {
  float2* pyx;          // separable propagator factors: exp(i a lambda qy^2) [W], exp(i a lambda qx^2)/W^2 [W]
  float* mask;
  float* mask_sc;
  float2* prop;
  float2* prop_edge;
  float* sx;
  float* sy;
  float px, py, cutoff, rolloff, distance, wavelength, edge_mult;
  int use_edge;
  float2* tw;           // W <= 128, not null: the window FFT's twiddle tables are written too
};

// scipy.fft.fftfreq(n, d) as the reference evaluates it with a float32 pixel size d:
// val = float32(1 / float32(n * d)); f_k = float64(k) * val; then cast to float32
// (pypty/utils.py:174-176). Replicated bit for bit so that the band-limit mask, whose edge
// is a <= comparison, selects exactly the same pixels.
__device__ __forceinline__ float fftfreq_f32(int k, int n, float d) {
  const int kk = (k < (n + 1) / 2) ? k : k - n;
  const float nd = __fmul_rn((float)n, d);
  const float val = __fdiv_rn(1.0f, nd);
  return (float)((double)kk * (double)val);
}

// One slice step's propagator for per-slice distances (multislice_core.py:69-74 with
// is_single_dist false): exp(-i pi d (lambda q^2 + 2 (qx tan_x + qy tan_y))) * mask, the phase
// rounded as tables_kernel rounds it, raised to edge_mult (principal branch, numpy's complex
// ** float) when edge, scaled by 1/W^2 like prop   grid (W^2 / 256), block 256
struct StepPropArgs {
  const float* mask;
  float px, py, wavelength, distance, tan_x, tan_y, edge_mult;
  int edge;
  float2* out;
  const float* tilt_row;   // device tilt row [6]: its inside tilt (2, 3) replaces tan_y, tan_x; or nullptr
};

template <int W>
__global__ void step_prop_kernel(StepPropArgs a) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= W * W) return;
  const int ky = idx / W, kx = idx % W;
  const float qx = fftfreq_f32(kx, W, a.px);
  const float qy = fftfreq_f32(ky, W, a.py);
  const float q2 = __fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy));
  const float tan_x = a.tilt_row ? a.tilt_row[3] : a.tan_x, tan_y = a.tilt_row ? a.tilt_row[2] : a.tan_y;
  const float tilt = __fmul_rn(2.0f, __fadd_rn(__fmul_rn(qx, tan_x), __fmul_rn(qy, tan_y)));
  const float x = __fadd_rn(__fmul_rn(a.wavelength, q2), tilt);
  const float phase = __fmul_rn(__fmul_rn(-3.141592654f, a.distance), x);
  const float mk = a.mask[idx];
  float s, c;
  sincosf(phase, &s, &c);
  float2 p = make_float2(c * mk, s * mk);
  if (a.edge) {
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
  const float inv = 1.0f / (float)(W * W);
  a.out[idx] = make_float2(p.x * inv, p.y * inv);
}

// the Z - 1 per-step tables of a problem with slice_distances (host), one launch per step
template <int W>
inline void launch_step_props(const float* mask, const float* distances_host, int nsteps, float px, float py,
                              float wavelength, float edge_mult, int use_edge, float tan_x, float tan_y,
                              float2* out, cudaStream_t st, const float* tilt_row = nullptr) {
  for (int z = 0; z < nsteps; ++z) {
    StepPropArgs sa{mask, px, py, wavelength, distances_host[z], tan_x, tan_y, edge_mult, (z == 0 && use_edge) ? 1 : 0,
                    out + (size_t)z * W * W, tilt_row};
    step_prop_kernel<W><<<(W * W + 255) / 256, 256, 0, st>>>(sa);
  }
}

template <int W>
__global__ void tables_kernel(TableArgs a) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if constexpr (W <= 128) {
    if (a.tw && idx < Geo<W>::TW1 + Geo<W>::TW2) a.tw[idx] = twiddle_entry<W>(idx);
  }
  if (idx < W) {
    // fftfreq(W) with d = 1 is exact in float64: k / W
    const int kk = (idx < W / 2) ? idx : idx - W;
    a.sx[idx] = (float)(-6.2831855 * ((double)kk / (double)W));
    a.sy[idx] = a.sx[idx];
    // exp(-i pi d lambda (qx^2 + qy^2)) = exp(-i pi d lambda qy^2) * exp(-i pi d lambda qx^2); the
    // factored phases differ from the reference's single float32 phase by one rounding
    const float a_pd = __fmul_rn(-3.141592654f, a.distance);
    const float qyk = fftfreq_f32(idx, W, a.py), qxk = fftfreq_f32(idx, W, a.px);
    float sy_, cy_, sx_, cx_;
    sincosf(__fmul_rn(a_pd, __fmul_rn(a.wavelength, __fmul_rn(qyk, qyk))), &sy_, &cy_);
    sincosf(__fmul_rn(a_pd, __fmul_rn(a.wavelength, __fmul_rn(qxk, qxk))), &sx_, &cx_);
    const float inv_ww = 1.0f / (float)(W * W);
    a.pyx[idx] = make_float2(cy_, sy_);
    a.pyx[W + idx] = make_float2(cx_ * inv_ww, sx_ * inv_ww);
  }
  if (idx >= W * W) return;
  const int ky = idx / W, kx = idx % W;
  const float qx = fftfreq_f32(kx, W, a.px);
  const float qy = fftfreq_f32(ky, W, a.py);
  const float q2 = __fadd_rn(__fmul_rn(qx, qx), __fmul_rn(qy, qy));
  const float max_x = fftfreq_f32((W - 1) / 2, W, a.px);
  const float mc = __fmul_rn(max_x, a.cutoff);
  const float r_max = __fmul_rn(mc, mc);
  float mk = (q2 <= r_max) ? 1.0f : 0.0f;
  if (a.rolloff != 0.0f) {
    const float m0 = __fmul_rn(max_x, __fsub_rn(a.cutoff, a.rolloff));
    const float r0 = __fmul_rn(m0, m0);
    if (q2 > r0)
      mk *= 0.5f * (1.0f + cosf(__fdiv_rn(__fmul_rn(3.141592654f, __fsub_rn(q2, r0)), __fsub_rn(r_max, r0))));
  }
  const float inv = 1.0f / (float)(W * W);
  a.mask[idx] = mk;
  a.mask_sc[idx] = mk * inv;
  // exp(-i*pi*d*(lambda*q2)) * mask, evaluated as the reference does in complex64:
  // the phase is (-pi_trunc * d) * (lambda * q2) rounded to float32 first
  const float phase = __fmul_rn(__fmul_rn(-3.141592654f, a.distance), __fmul_rn(a.wavelength, q2));
  float s, c;
  sincosf(phase, &s, &c);
  const float2 p = make_float2(c * mk, s * mk);
  a.prop[idx] = make_float2(p.x * inv, p.y * inv);
  if (a.use_edge) {
    // principal-branch power, as numpy's complex ** float (|p|^e * exp(i e arg p))
    float r = sqrtf(p.x * p.x + p.y * p.y);
    float2 pe = make_float2(0.f, 0.f);
    if (r > 0.f) {
      float ang = atan2f(p.y, p.x) * a.edge_mult;
      float re = powf(r, a.edge_mult);
      float se, ce;
      sincosf(ang, &se, &ce);
      pe = make_float2(re * ce, re * se);
    }
    a.prop_edge[idx] = make_float2(pe.x * inv, pe.y * inv);
  }
}

// ------------------------------------------------------------------ layout transposes
// (Ny, Nx, Z*Mo) reference layout  <->  (Z*Mo, Ny, Nx) slice-major working layout
static __global__ void obj_to_slices_kernel(const float2* __restrict__ src, float2* __restrict__ dst,
                                     int nyx, int zm) {
  const int yx = blockIdx.x * blockDim.x + threadIdx.x;
  if (yx >= nyx) return;
  for (int k = 0; k < zm; ++k) dst[(size_t)k * nyx + yx] = src[(size_t)yx * zm + k];
}

static __global__ void slices_to_obj_kernel(const float2* __restrict__ src, float2* __restrict__ dst,
                                     int nyx, int zm) {
  const int yx = blockIdx.x * blockDim.x + threadIdx.x;
  if (yx >= nyx) return;
  for (int k = 0; k < zm; ++k) dst[(size_t)yx * zm + k] = src[(size_t)k * nyx + yx];
}

// ------------------------------------------------------------------ shared-memory plan
template <int W>
struct Smem {
  using G = Geo<W>;
  static constexpr size_t bytes = sizeof(float2) * (G::XBUF + G::TW1 + G::TW2) + sizeof(double) * 64;
};

template <int W>
__device__ __forceinline__ void carve(unsigned char* smem, float2*& xbuf, float2*& tw1,
                                      float2*& tw2, double*& red) {
  using G = Geo<W>;
  xbuf = reinterpret_cast<float2*>(smem);
  tw1 = xbuf + G::XBUF;
  tw2 = tw1 + G::TW1;
  red = reinterpret_cast<double*>(tw2 + G::TW2);
}

// sum of (a, b) over the block; result valid in thread 0
__device__ __forceinline__ void block_sum2(double& a, double& b, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) {
    red[warp] = a;
    red[32 + warp] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int w = 0; w < nw; ++w) {
      sa += red[w];
      sb += red[32 + w];
    }
    a = sa;
    b = sb;
  }
}

// ------------------------------------------------------------------ probe spectrum
// probe (W, W, Mp) reference layout -> FFT per mode, native frequency layout [Mp]
template <int W>
__global__ void __launch_bounds__(Geo<W>::T) probe_fft_kernel(const float2* __restrict__ probe, int Mp,
                                                              const float2* __restrict__ g_tw,
                                                              float2* __restrict__ probe_f) {
  using G = Geo<W>;
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  load_twiddles<W>(tw1, tw2, g_tw);
  __syncthreads();
  const int t = threadIdx.x, p = blockIdx.x;
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = probe[(size_t)(G::ry(t) * W + G::rx(t, i)) * Mp + p];
  WinFFT<W>::forward(v, xbuf, tw1, tw2);
  st_native<W>(probe_f + (size_t)p * W * W, v);
}

// ------------------------------------------------------------------ object windows
// Gather the W x W window of every (position, slice, object mode) from the slice-major
// object and band-limit it: O_b = IFFT(FFT(window) * mask)  (pypty/objective.py:436-441).
struct WindowArgs {
  const float2* obj;      // (Z*Mo, Ny, Nx)
  const int* pos;         // (N, 2) int [y, x]
  const int* seq;         // batch's sequence entries
  const float* mask_sc;
  const float2* tw;
  float2* out;            // native real layout [Bb*Z*Mo]
  int Ny, Nx, zm;
};

template <int W>
__global__ void __launch_bounds__(Geo<W>::T) object_windows_kernel(WindowArgs a) {
  using G = Geo<W>;
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  load_twiddles<W>(tw1, tw2, a.tw);
  const int t = threadIdx.x;
  const int win = blockIdx.x;             // (b * zm + k)
  const int b = win / a.zm, k = win % a.zm;
  const int gi = a.seq[b];
  const int y0 = a.pos[2 * gi], x0 = a.pos[2 * gi + 1];
  const float2* src = a.obj + (size_t)k * a.Ny * a.Nx + (size_t)(y0 + G::ry(t)) * a.Nx + x0;
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = src[G::rx(t, i)];
  __syncthreads();
  WinFFT<W>::forward(v, xbuf, tw1, tw2);
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = cscale(v[i], a.mask_sc[G::fky(t, i) * W + G::fkx(t, i)]);
  WinFFT<W>::inverse(v, xbuf, tw1, tw2);
  st_native<W>(a.out + (size_t)win * W * W, v);
}

// ------------------------------------------------------------------ fused multislice
struct FusedArgs {
  int Z, Mp, Mo, algorithm, step_obj, step_probe, step_pos, probe_shift, simulate, use_edge;
  int phase;                // 0: whole pass; 1: forward half; 2: adjoint half;
                            // 3: forward multislice only (exit wave out); 4: adjoint from a given
                            //    exit-wave gradient with a real-space probe gradient out
  const float2* probe_b;    // per-position incoming probes, native real [Bb*Mp] (phase 3)
  float2* exit_out;         // exit waves, native real [Bb*Mp*Mo] (phase 3)
  float loss_weight;
  const float2* probe;      // (W, W, Mp) reference layout (used without probe shift)
  const float2* probe_f;    // native frequency layout [Mp]
  const float2* obl;        // band-limited object windows, native real [Bb*Z*Mo]
  const float2* prop;       // natural (ky, kx), scaled by 1/W^2
  const float2* prop_edge;
  const float2* pyx;        // separable propagator factors (used when the mask is binary)
  int use_sep;
  int mask_bin;             // the band-limit mask is 0/1 (no smooth roll-off): the mask bits and
                            // the separable shift ramp stand in for the float mask
  const float2* prop_steps; // per-step tables [Z-1] (slice distances), step 0 with the edge
                            // power; nullptr: prop / prop_edge for every step
  const float* mask;        // natural, unscaled
  const float* sx;
  const float* sy;
  const float* corr;        // (N, 2) [dy, dx]
  const int* seq;           // batch's sequence entries
  const float* measured;    // (N, W, W) detector (fftshifted) order
  const float2* tw;
  float2* stack;            // conj input waves, native real [Bb*Z*Mp*Mo]
  float2* gsum;             // object-gradient contributions, native real [Bb*Z*Mo*Mp] (probe mode innermost)
  float2* fprobe;           // FFT of the per-position probe gradient, native freq [Bb*Mp]
  float2* gbuf;             // dL/d(exit wave) between the two halves, native real [Bb*Mp*Mo]
  float2* psi;              // 256 windows: far-field wave per mode [Bb*Mp*Mo]
  float* dldi;              // 256 windows: dL/dI between the two halves [Bb]
  float2* pgr;              // 256 windows: object-mode sum of the probe gradient [Bb*Mp]
  int ckpt;                 // 256 windows: keep every ckpt-th slice's wave, recompute the rest
  float2* seg;              // 256 windows: recomputed waves of one segment [Bb*ckpt]
  float2* gpark;            // 256 windows: adjoint wave parked during a recomputation [Bb]
  double* loss_part;        // [Bb][2]
  double* pos_part;         // [Bb][Mp][2]
  float* sim_out;           // [Bb][W][W] simulated mean intensity (detector order)
  int* err;                 // set to 1 if a bounded wait on an async copy ran out
};

template <int W>
__device__ __forceinline__ float2 shift_ramp(const FusedArgs& a, int ky, int kx, float mk,
                                             float dy, float dx) {
  // exp(smx*dx + smy*dy) * mask with smx = i * sx[kx] * mask (pypty/objective.py:473)
  const float th = __fadd_rn(__fmul_rn(__fmul_rn(a.sx[kx], mk), dx),
                             __fmul_rn(__fmul_rn(a.sy[ky], mk), dy));
  float s, c;
  sincosf(th, &s, &c);
  return make_float2(c * mk, s * mk);
}

// The same ramp for a binary mask, inside the mask: exp(i sx[kx] dx) * exp(i sy[ky] dy). A
// thread's 32 frequency-layout elements i = q*Bq + r span Q distinct kx (by q) and Bq distinct
// ky (by r), so Q + Bq sincos evaluations serve all 32 (the caller zeroes the elements outside
// the mask). f(i, ky, kx, ramp) is called for every element, i a compile-time constant.
template <int W, typename Fn>
__device__ __forceinline__ void visit_sep_ramp(const FusedArgs& a, int t, float dy, float dx, Fn&& f) {
  using G = Geo<W>;
  constexpr int Q = G::Q, Bq = G::Bq;
  auto phase = [](float s, float d) {
    float sn, cs;
    sincosf(__fmul_rn(s, d), &sn, &cs);
    return make_float2(cs, sn);
  };
  if constexpr (Q <= Bq) {   // the Q x factors kept, one y factor at a time
    float2 ex[Q];
    static_for<0, Q>([&](auto QQ) {
      constexpr int q = decltype(QQ)::value;
      ex[q] = phase(a.sx[G::fkx(t, q * Bq)], dx);
    });
    static_for<0, Bq>([&](auto RR) {
      constexpr int r = decltype(RR)::value;
      const int ky = G::fky(t, r);
      const float2 ey = phase(a.sy[ky], dy);
      static_for<0, Q>([&](auto QQ) {
        constexpr int q = decltype(QQ)::value;
        f(std::integral_constant<int, q * Bq + r>{}, ky, G::fkx(t, q * Bq), cmul(ex[q], ey));
      });
    });
  } else {                   // the Bq y factors kept, one x factor at a time
    float2 ey[Bq];
    static_for<0, Bq>([&](auto RR) {
      constexpr int r = decltype(RR)::value;
      ey[r] = phase(a.sy[G::fky(t, r)], dy);
    });
    static_for<0, Q>([&](auto QQ) {
      constexpr int q = decltype(QQ)::value;
      const int kx = G::fkx(t, q * Bq);
      const float2 ex = phase(a.sx[kx], dx);
      static_for<0, Bq>([&](auto RR) {
        constexpr int r = decltype(RR)::value;
        f(std::integral_constant<int, q * Bq + r>{}, G::fky(t, r), kx, cmul(ex, ey[r]));
      });
    });
  }
}

// A thread's running sum of float32 terms, compensated: every add is Knuth's TwoSum, so hi + lo
// holds the exact sum to ~2^-44 relative, read out in FP64 for the FP64 block and grid sums.
// (Per-element FP64 adds would run at the GPU's much lower FP64 rate.)
struct FSum {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ FSum& operator+=(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
    return *this;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// dL/dI of one detector pixel for the loss `alg` (pypty/objective.py:527-559), with the
// per-pixel loss and squared error added to the accumulators (double, or FSum). Float32
// arithmetic per pixel, as the reference's arrays; only the sums are wider.
template <typename Acc>
__device__ __forceinline__ float loss_pixel(int alg, float I, float Mv, Acc& lsum, Acc& ssum) {
  float d, lp, sp;
  if (alg == ALG_LSQ_SQRT) {
    const float sI = sqrtf(I), sM = sqrtf(Mv);
    const float df = sI - sM;
    sp = (Mv - I) * (Mv - I);
    lp = df * df;
    d = df / (sI == 0.0f ? 1.0f : sI);
  } else if (alg == ALG_ML) {
    const float df = I - Mv;
    sp = df * df;
    lp = I - Mv * logf(I + (I == 0.0f ? 1.0f : 0.0f));
    d = df / (I == 0.0f ? 1.0f : I);
  } else if (alg == ALG_LSQ) {
    const float df = I - Mv;
    sp = df * df;
    lp = sp;
    d = 2.0f * df;
  } else {
    const float df = Mv - I;
    sp = df * df;
    if (Mv > 0.5f) {
      lp = 0.5f * (sp / Mv);
      d = I / Mv - 1.0f;
    } else {
      lp = I;
      d = 1.0f;
    }
  }
  lsum += lp;
  ssum += sp;
  return d;
}

// Shared memory of the fused kernel: the FFT exchange buffer (which also receives each
// step's main operand by TMA bulk copy), twiddles, reduction scratch, a side buffer for the
// first NST elements per thread of the adjoint step's object window, and two mbarriers.
template <int W>
struct FusedSmem {
  static constexpr int NST = (W == 128) ? 22 : 16;
  static constexpr size_t side_off = Smem<W>::bytes;
  static constexpr size_t pyx_off = side_off + sizeof(float2) * NST * Geo<W>::T;
  static constexpr size_t bits_off = pyx_off + sizeof(float2) * 2 * W;
  static constexpr size_t bar_off = bits_off + sizeof(uint32_t) * Geo<W>::T;
  // W = 64: the position's measured pattern (W^2 floats, detector order), copied in at the
  // start, and the probe-shift ramp of the first step (frequency layout), reused by the last
  static constexpr size_t meas_off = (bar_off + 2 * sizeof(uint64_t) + 15) & ~(size_t)15;
  static constexpr size_t ramp_off = meas_off + (W == 64 ? sizeof(float) * W * W : 0);
  static constexpr size_t bytes = ramp_off + (W == 64 ? sizeof(float2) * W * W : 0);
};

// One thread block per (position, probe mode, object mode); the Mp*Mo blocks of a position
// form a thread-block cluster and exchange intensities / gradients through distributed
// shared memory. Forward multislice (multislice_core.py:61-82), far field + loss
// (objective.py:501-597), adjoint multislice (multislice_core.py:158-199), probe-shift
// adjoint and position gradient (objective.py:641-658).
//
// The whole computation is one loop of steps, each "real-space op -> FFT -> frequency op ->
// inverse FFT", so the forward and inverse transforms are each inlined once and the window
// never leaves the registers:
//   step 0          incoming probe (shift ramp in frequency, inverse FFT)
//   steps 1..Z      slice z = s-1: store conj(psi_z), psi *= O_z, FFT, *= P (or the far
//                   field, loss and dL/dPsi after the last slice), IFFT
//   steps Z+1..2Z   slice z = 2Z-s: object-gradient contribution, g *= conj(O_z), FFT,
//                   *= conj(P), IFFT (z = 0: probe-gradient spectrum and position gradient)
// Operands: the side buffer (each thread's first NST elements, a prefix of the native layout)
// takes every step's streamed window by TMA one step ahead -- O_z in the forward, conj(psi_z)
// from the stack in the adjoint -- and the rest of that window is loaded at the step. The step
// writes its outgoing window (conj(psi_z) in the forward, this mode's gradient contribution in
// the adjoint) into the side buffer in place of what it read, and a TMA bulk store takes it out
// behind the forward transform. The adjoint's O_z lands in the exchange buffer while the
// inverse transform finishes its last register-only round; the adjoint's first step finds
// conj(psi_{Z-1}) still in the side buffer.
// PH = 0: the whole pass (phase 0) with every phase branch compiled out; PH = 1: a.phase at
// run time (the split halves and the multislice_core phases).
template <int W, int PH>
__global__ void __launch_bounds__(Geo<W>::T, Geo<W>::MINB) fused_multislice_kernel(FusedArgs a) {
  using G = Geo<W>;
  using F = WinFFT<W>;
  using S = FusedSmem<W>;
  constexpr int T = G::T;
  constexpr int NST = S::NST;
  constexpr size_t WW = (size_t)W * W;
  // W = 64 (few slices, latency-bound far field and probe steps): mask bits instead of the
  // float mask, the separable shift ramp, the measured pattern copied into shared memory at the
  // start. At W = 128 the extra live values spill and shared memory is full, so these stay
  // compiled out there.
  constexpr bool kLean = (W == 64);
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  float2* side = reinterpret_cast<float2*>(smem + S::side_off);
  float2* spy = reinterpret_cast<float2*>(smem + S::pyx_off);   // [W] y factor, then [W] x factor
  const float2* spx = spy + W;
  uint32_t* sbits = reinterpret_cast<uint32_t*>(smem + S::bits_off);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S::bar_off);   // [0]: xbuf, [1]: side
  float* fs0 = reinterpret_cast<float*>(xbuf);   // WW floats: this block's |Psi|^2
  float* fs1 = fs0 + WW;                          // WW floats: mode-summed I, then dL/dI
  cg::cluster_group cluster = cg::this_cluster();
  const int t = threadIdx.x;
  const int nmodes = a.Mp * a.Mo;
  const int crank = (int)cluster.block_rank();
  const int p = crank % a.Mp, m = crank / a.Mp;
  const int b = blockIdx.x / nmodes;
  const int gi = a.seq[b];
  const float dy = a.corr[2 * gi], dx = a.corr[2 * gi + 1];
  const int Z = a.Z;
  const bool adj_stack = a.step_obj && !a.simulate;   // the adjoint reads conj(psi_z)
  const int phase = PH == 0 ? 0 : a.phase;
  if (t == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_async_shared();
  }
  load_twiddles<W>(tw1, tw2, a.tw);
  for (int i = t; i < 2 * W; i += T) spy[i] = a.pyx[i];
  // bit i: element i (frequency layout) of this thread lies inside the band limit
  {
    uint32_t mbits = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) mbits |= (a.mask[G::fky(t, i) * W + G::fkx(t, i)] != 0.0f ? 1u : 0u) << i;
    sbits[t] = mbits;   // kept in shared memory: registers are needed for the window
  }
  __syncthreads();
  float* smeas = reinterpret_cast<float*>(smem + S::meas_off);    // W = 64 only
  float2* sramp = reinterpret_cast<float2*>(smem + S::ramp_off);  // W = 64 only
  if constexpr (kLean) {
    // only passes that reach the far field (which waits for these copies) issue them
    if (!a.simulate && a.measured && (phase <= 1)) {
      const float* src = a.measured + (size_t)gi * WW;
      if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
        for (int e = 4 * t; e < (int)WW; e += 4 * T) cp_async16(smeas + e, src + e);
      } else {
        for (int e = t; e < (int)WW; e += T) cp_async4(smeas + e, src + e);
      }
      cp_async_commit();
    }
  }
  uint32_t ph_x = 0, ph_side = 0;

  auto obl_ptr = [&](int z) { return a.obl + (((size_t)b * Z + z) * a.Mo + m) * WW; };
  auto stack_ptr = [&](int z) { return a.stack + ((((size_t)b * Z + z) * a.Mp + p) * a.Mo + m) * WW; };
  // O_z of step s >= 1: the adjoint steps read it from the exchange buffer, the forward steps
  // through the side buffer
  auto xsrc = [&](int s) -> const float2* { return obl_ptr(s <= Z ? s - 1 : 2 * Z - s); };
  auto issue_x = [&](int s) {
    if (t == 0) {
      fence_async_shared();
      bulk_load(xbuf, xsrc(s), (uint32_t)(WW * sizeof(float2)), &bars[0]);
    }
  };
  constexpr uint32_t kSideBytes = (uint32_t)(NST * T * sizeof(float2));
  // the side buffer takes the first NST elements per thread (a prefix of the native layout) of
  // a window: O_z in the forward, conj(psi_z) from the stack in the adjoint
  auto issue_side = [&](const float2* src) {
    if (t == 0) {
      fence_async_shared();
      bulk_load(side, src, kSideBytes, &bars[1]);
    }
  };
  // the window that the staged side buffer goes to: code z < Z is the stack window of slice z
  // (forward), code Z + z this mode's gradient contribution of slice z (adjoint)
  auto contrib_ptr = [&](int z) { return a.gsum + ((((size_t)b * Z + z) * a.Mo + m) * a.Mp + p) * WW; };
  auto store_ptr = [&](int code) { return code < Z ? stack_ptr(code) : contrib_ptr(code - Z); };

  float2 v[32];
  int side_next = -1;        // the slice whose window prefix the side buffer takes next
  bool side_held = false;    // the side buffer holds the next step's operand, waited for
  int store_code = -1;       // the side buffer is staged for a bulk store to store_ptr(store_code)
  float2* gb = a.gbuf + (((size_t)b * a.Mp + p) * a.Mo + m) * WW;
  const bool adjoint_only = (phase == 2 || phase == 4);
  const int s_begin = adjoint_only ? Z + 1 : 0;
  const int s_end = (a.simulate || phase == 1 || phase == 3) ? Z + 1 : 2 * Z + 1;
  if (adjoint_only) {
    // adjoint half: resume from dL/d(exit wave) kept by the forward half
    ld_native<W>(gb, v);
    issue_x(Z + 1);
    if (adj_stack) issue_side(stack_ptr(Z - 1));
  } else {
    issue_side(obl_ptr(0));
  }
  for (int s = s_begin; s < s_end; ++s) {
    const bool fwd = (s >= 1 && s <= Z);
    const int z = fwd ? s - 1 : 2 * Z - s;

    // ------------------------------------------------ real-space op
    if (s == 0) {
      if (PH != 0 && a.probe_b) {
        ld_native<W>(a.probe_b + ((size_t)b * a.Mp + p) * WW, v);
      } else if (!a.probe_shift) {
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = a.probe[(size_t)(G::ry(t) * W + G::rx(t, i)) * a.Mp + p];
      }
    } else if (fwd) {
      // O_z: elements NST.. straight from global memory (issued first), the rest from the side
      // buffer, copied in during the previous step; the exchange buffer is not refilled
      float4 otail[(32 - NST) / 2];
      {
        const float4* og = reinterpret_cast<const float4*>(obl_ptr(z));
#pragma unroll
        for (int j = NST / 2; j < 16; ++j) otail[j - NST / 2] = og[j * T + t];
      }
      float4* sd = reinterpret_cast<float4*>(side);
      float4* st = adj_stack ? reinterpret_cast<float4*>(stack_ptr(z)) : nullptr;
      mbar_wait(&bars[1], ph_side, a.err);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const float4 q = (j < NST / 2) ? sd[j * T + t] : otail[j - NST / 2];
        if (adj_stack) {
          // conj(psi_z) to the stack: elements < NST in place of O_z in the side buffer, whence
          // a bulk copy takes them out behind the transform; the rest straight from the registers
          const float4 c = make_float4(v[2 * j].x, -v[2 * j].y, v[2 * j + 1].x, -v[2 * j + 1].y);
          if (j < NST / 2) sd[j * T + t] = c;
          else st[j * T + t] = c;
        }
        v[2 * j] = cmul(v[2 * j], make_float2(q.x, q.y));
        v[2 * j + 1] = cmul(v[2 * j + 1], make_float2(q.z, q.w));
      }
      if (adj_stack) {
        fence_async_shared();
        // the adjoint's first step (the same slice) reads conj(psi_z) from the side buffer itself
        if (!(z == Z - 1 && phase == 0)) store_code = z;
      }
      if (z + 1 < Z) side_next = z + 1;
      else side_held = true;
      if (phase == 3 && z == Z - 1) {
        st_native<W>(a.exit_out + (((size_t)b * a.Mp + p) * a.Mo + m) * WW, v);   // the exit wave
        break;
      }
    } else {
      if (adj_stack) {
        // conj(psi_z): elements NST.. straight from global memory (this thread stored them in
        // the forward), the rest in the side buffer
        float4 stail[(32 - NST) / 2];
        {
          const float4* sg = reinterpret_cast<const float4*>(stack_ptr(z));
#pragma unroll
          for (int j = NST / 2; j < 16; ++j) stail[j - NST / 2] = sg[j * T + t];
        }
        if (side_held) side_held = false;
        else mbar_wait(&bars[1], ph_side, a.err);
        // contribution conj(psi_z) * g of this probe mode, to its own window of the gradient
        // buffer ([position][slice][object mode][probe mode]); grad_windows_kernel adds the
        // probe modes in ascending order before the band limit (multislice_core.py:184-191), so
        // the adjoint needs no cluster barrier and no remote reads. Elements < NST replace
        // conj(psi_z) in the side buffer, whence a bulk copy takes them out behind the transform.
        float4* g4 = reinterpret_cast<float4*>(contrib_ptr(z));
        float4* sd = reinterpret_cast<float4*>(side);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float4 q = (j < NST / 2) ? sd[j * T + t] : stail[j - NST / 2];
          const float2 g0 = cmul(make_float2(q.x, q.y), v[2 * j]);
          const float2 g1 = cmul(make_float2(q.z, q.w), v[2 * j + 1]);
          if (j < NST / 2) sd[j * T + t] = make_float4(g0.x, g0.y, g1.x, g1.y);
          else g4[j * T + t] = make_float4(g0.x, g0.y, g1.x, g1.y);
        }
        fence_async_shared();
        store_code = Z + z;
        if (z > 0) side_next = z - 1;
      }
      // g *= conj(O_z), O_z in the exchange buffer
      mbar_wait(&bars[0], ph_x, a.err);
      {
        const float4* ob = reinterpret_cast<const float4*>(xbuf);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float4 q = ob[j * T + t];
          v[2 * j] = cmulc(v[2 * j], make_float2(q.x, q.y));
          v[2 * j + 1] = cmulc(v[2 * j + 1], make_float2(q.z, q.w));
        }
      }
      if (z == 0) {
        if (!(a.step_probe || a.step_pos)) break;
        if (a.Mo > 1) {
          // probe gradient: sum over object modes (multislice_core.py:193-197)
          __syncthreads();
#pragma unroll
          for (int i = 0; i < 32; ++i) xbuf[i * T + t] = v[i];
          cluster.sync();
          if (m == 0) {
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              float2 acc = make_float2(0.f, 0.f);
              for (int mm = 0; mm < a.Mo; ++mm)
                acc = cadd(acc, cluster.map_shared_rank(xbuf, p + mm * a.Mp)[i * T + t]);
              v[i] = acc;
            }
          }
          cluster.sync();
          if (m != 0) break;
        }
        if (phase == 4) {   // interm_probe_grad of multislice_core.py:193-197, real space
          if (a.step_probe) st_native<W>(a.fprobe + ((size_t)b * a.Mp + p) * WW, v);
          break;
        }
      }
    }

    // ------------------------------------------------ forward FFT
    if (s > 0) {
      F::forward_round1(v, tw1);
      const bool staged = store_code >= 0;
      auto side_src = [&](int zz) { return fwd ? obl_ptr(zz) : stack_ptr(zz); };
      F::forward_rest(v, xbuf, tw1, tw2, [&] {
        // every thread has finished with the side buffer: copy its staged part out, or refill it
        if (staged) {
          if (t == 0) bulk_store(store_ptr(store_code), side, kSideBytes);
          store_code = -1;
        } else if (side_next >= 0) {
          issue_side(side_src(side_next));
          side_next = -1;
        }
      });
      if (side_next >= 0) {   // refill the side buffer once the bulk store has read it
        if (t == 0) bulk_wait_read();
        issue_side(side_src(side_next));
        side_next = -1;
      }
    }

    // ------------------------------------------------ frequency op
    if (s == 0) {
      if (!a.probe_shift) continue;   // the unshifted probe is already in real space
      const float2* pf = a.probe_f + (size_t)p * WW;
      const float inv = 1.0f / (float)WW;
      if (kLean && a.mask_bin) {
        const uint32_t mbits = sbits[t];
        visit_sep_ramp<W>(a, t, dy, dx, [&](auto I, int, int, float2 ramp) {
          constexpr int i = decltype(I)::value;
          v[i] = ((mbits >> i) & 1u) ? cscale(cmul(pf[nidx<W>(i, t)], ramp), inv) : make_float2(0.f, 0.f);
          sramp[i * T + t] = ramp;   // the same ramp serves the probe-gradient step (phase 0)
        });
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int ky = G::fky(t, i), kx = G::fkx(t, i);
          v[i] = cscale(cmul(pf[nidx<W>(i, t)], shift_ramp<W>(a, ky, kx, a.mask[ky * W + kx], dy, dx)), inv);
        }
      }
    } else if (fwd && z < Z - 1) {
      if (a.use_sep && !(z == 0 && a.use_edge)) {
        const uint32_t mbits = sbits[t];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float2 P = cmul(spy[G::fky(t, i)], spx[G::fkx(t, i)]);
          v[i] = ((mbits >> i) & 1u) ? cmul(v[i], P) : make_float2(0.f, 0.f);
        }
      } else {
        const float2* pr = a.prop_steps ? a.prop_steps + (size_t)z * WW
                                        : ((z == 0 && a.use_edge) ? a.prop_edge : a.prop);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = cmul(v[i], pr[G::fky(t, i) * W + G::fkx(t, i)]);
      }
    } else if (fwd) {
      // far field: Psi = FFT(exit) * mask, I = mean over modes |Psi|^2 (objective.py:501-512)
      if constexpr (kLean) cp_async_wait_all();   // the measured pattern; the cluster barrier below
                                                  // makes every thread's part visible
      __syncthreads();
      if (kLean && a.mask_bin) {
        const uint32_t mbits = sbits[t];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          if (!((mbits >> i) & 1u)) v[i] = make_float2(0.f, 0.f);
          fs0[i * T + t] = cabs2(v[i]);
        }
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          v[i] = cscale(v[i], a.mask[G::fky(t, i) * W + G::fkx(t, i)]);
          fs0[i * T + t] = cabs2(v[i]);
        }
      }
      cluster.sync();
#pragma unroll 1
      for (int i0 = 0; i0 < 32; i0 += 8) {
        float acc[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] = 0.0f;
#pragma unroll
        for (int r = 0; r < 8; ++r) {      // ranks in ascending order: a fixed summation order
          if (r < nmodes) {
            const float* rb = cluster.map_shared_rank(fs0, r);
#pragma unroll
            for (int k = 0; k < 8; ++k) acc[k] += rb[(i0 + k) * T + t];
          }
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) fs1[(i0 + k) * T + t] = acc[k];
      }
      cluster.sync();   // every block is done reading this block's intensities
      const float inv_modes = 1.0f / (float)nmodes;
      const float* meas = a.measured + (size_t)gi * WW;
      FSum lsum_c, ssum_c;
      // eight pixels at a time, used in order (W = 64: the next eight measured values are
      // loaded while the current ones are used)
      auto load8 = [&](int i0, float (&dst)[8]) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int i = i0 + k;
          const int ky = G::fky(t, i), kx = G::fkx(t, i);
          const int didx = ((ky + W / 2) & (W - 1)) * W + ((kx + W / 2) & (W - 1));
          dst[k] = a.simulate ? 0.0f : (kLean ? smeas[didx] : meas[didx]);
        }
      };
      float mv[8], nx[8];
      if constexpr (kLean) load8(0, mv);
#pragma unroll 1
      for (int i0 = 0; i0 < 32; i0 += 8) {
        if constexpr (kLean) {
          if (i0 + 8 < 32) load8(i0 + 8, nx);
        } else {
          load8(i0, mv);
        }
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int i = i0 + k;
          const float acc = fs1[i * T + t];
          const float I = (nmodes == 1) ? acc : acc * inv_modes;
          if (a.simulate) {
            const int ky = G::fky(t, i), kx = G::fkx(t, i);
            const int didx = ((ky + W / 2) & (W - 1)) * W + ((kx + W / 2) & (W - 1));
            if (crank == 0) a.sim_out[(size_t)b * WW + didx] = I;
            continue;
          }
          float d = loss_pixel(a.algorithm, I, mv[k], lsum_c, ssum_c);
          if (nmodes > 1) d = d / (float)nmodes;           // objective.py:586-587
          fs1[i * T + t] = d;
        }
        if constexpr (kLean) {
#pragma unroll
          for (int k = 0; k < 8; ++k) mv[k] = nx[k];
        }
      }
      if (a.simulate) return;
      double lsum = lsum_c.value(), ssum = ssum_c.value();
      block_sum2(lsum, ssum, red);
      if (t == 0 && crank == 0) {
        a.loss_part[2 * b] = lsum;
        a.loss_part[2 * b + 1] = ssum;
      }
      // dL/dPsi = dLdI * Psi * (w * W^2); the W^2 cancels the 1/W^2 of ifft2 (objective.py:595-597)
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = cscale(cscale(v[i], fs1[i * T + t]), a.loss_weight);
    } else if (z > 0) {
      if (a.use_sep && !(z == 1 && a.use_edge)) {
        const uint32_t mbits = sbits[t];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const float2 P = cmul(spy[G::fky(t, i)], spx[G::fkx(t, i)]);
          v[i] = ((mbits >> i) & 1u) ? cmulc(v[i], P) : make_float2(0.f, 0.f);
        }
      } else {
        const float2* pr = a.prop_steps ? a.prop_steps + (size_t)(z - 1) * WW
                                        : ((z == 1 && a.use_edge) ? a.prop_edge : a.prop);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = cmulc(v[i], pr[G::fky(t, i) * W + G::fkx(t, i)]);
      }
    } else {
      // probe-gradient spectrum with the shift adjoint, position gradient (objective.py:641-656)
      const float2* pf = a.probe_f + (size_t)p * WW;
      FSum gy_c, gx_c;
      if (kLean && a.probe_shift && a.mask_bin && phase == 0) {
        // the first step's ramp, kept in shared memory by this thread
        const uint32_t mbits = sbits[t];
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int ky = G::fky(t, i), kx = G::fkx(t, i);
          const float mk = ((mbits >> i) & 1u) ? 1.0f : 0.0f;
          v[i] = cmulc(v[i], cscale(sramp[i * T + t], mk));
          if (a.step_pos) {   // as below
            const float im = cmulc(v[i], pf[nidx<W>(i, t)]).y;
            gy_c += -(a.sy[ky] * mk) * im;
            gx_c += -(a.sx[kx] * mk) * im;
          }
        }
      } else if (a.probe_shift) {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int ky = G::fky(t, i), kx = G::fkx(t, i);
          const float mk = a.mask[ky * W + kx];
          v[i] = cmulc(v[i], shift_ramp<W>(a, ky, kx, mk, dy, dx));
          if (a.step_pos) {
            // Re(smyx * conj(Pf) * F) with smyx = i*s*mask  ->  -(s*mask) * Im(conj(Pf) * F)
            const float im = cmulc(v[i], pf[nidx<W>(i, t)]).y;
            gy_c += -(a.sy[ky] * mk) * im;
            gx_c += -(a.sx[kx] * mk) * im;
          }
        }
      }
      if (a.step_probe) st_native<W>(a.fprobe + ((size_t)b * a.Mp + p) * WW, v);
      if (a.step_pos) {
        double gy = gy_c.value(), gx = gx_c.value();
        block_sum2(gy, gx, red);
        if (t == 0) {
          a.pos_part[(b * a.Mp + p) * 2] = gy;
          a.pos_part[(b * a.Mp + p) * 2 + 1] = gx;
        }
      }
      break;
    }

    // ------------------------------------------------ inverse FFT (next operand copied in
    // behind its register-only last round)
    F::inverse_head(v, xbuf, tw1, tw2);
    if (s + 1 < s_end) {
      if (s + 1 > Z) {     // the adjoint steps read O_z from the exchange buffer
        __syncthreads();   // every thread has finished reading it
        // the adjoint's side-buffer copies read the stack's bulk-stored parts back
        if (s == Z && t == 0) bulk_wait_all();
        issue_x(s + 1);
      }
      // every block asks for its operands at about the same time: bring what the next steps
      // read late into L2 now, so that they read L2 instead of waiting for HBM -- the adjoint's
      // O_z two steps ahead (copied into the exchange buffer just in time) and the parts of the
      // side-buffer windows that are read by plain loads (their prefixes arrive by TMA a whole
      // step ahead)
      if (t == 0) {
        constexpr uint32_t kTailBytes = (uint32_t)((WW - (size_t)NST * T) * sizeof(float2));
        if (s + 2 < s_end) {
          if (s + 2 <= Z)   // forward: the side copy (a step ahead) takes the prefix; the tail is loaded
            prefetch_l2(xsrc(s + 2) + (size_t)NST * T, kTailBytes);
          else              // adjoint: O_z goes to the exchange buffer just in time
            prefetch_l2(xsrc(s + 2), (uint32_t)(WW * sizeof(float2)));
        }
        const int zs = 2 * Z - s - 2;
        if (adj_stack && s >= Z && zs >= 0) prefetch_l2(stack_ptr(zs) + (size_t)NST * T, kTailBytes);
      }
    }
    F::inverse_tail(v, tw1);
  }
  if (store_code >= 0) {   // staged by a step that left the loop before its forward transform
    __syncthreads();
    if (t == 0) bulk_store(store_ptr(store_code), side, kSideBytes);
  }
  if (t == 0) bulk_wait_all();   // the bulk stores are complete before the block exits
  if (phase == 1) st_native<W>(gb, v);   // forward half: keep dL/d(exit wave)
}

// ------------------------------------------------------------------ reference-layout windows
// (B, W, W, K) arrays with the mode axes innermost (the reference's layout) <-> the native
// window layout [B*K] used by the kernels; one block per window.
template <int W>
__global__ void __launch_bounds__(Geo<W>::T) ref_to_native_kernel(const float2* __restrict__ src,
                                                                  float2* __restrict__ dst, int K) {
  using G = Geo<W>;
  const int t = threadIdx.x, win = blockIdx.x, b = win / K, k = win % K;
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = src[(((size_t)b * W + G::ry(t)) * W + G::rx(t, i)) * K + k];
  st_native<W>(dst + (size_t)win * W * W, v);
}

template <int W>
__global__ void __launch_bounds__(Geo<W>::T) native_to_ref_kernel(const float2* __restrict__ src,
                                                                  float2* __restrict__ dst, int K) {
  using G = Geo<W>;
  const int t = threadIdx.x, win = blockIdx.x, b = win / K, k = win % K;
  float2 v[32];
  ld_native<W>(src + (size_t)win * W * W, v);
#pragma unroll
  for (int i = 0; i < 32; ++i) dst[(((size_t)b * W + G::ry(t)) * W + G::rx(t, i)) * K + k] = v[i];
}

// (B, W*W, K) -> (B, K, W*W): per-position windows to per-plane natural windows
static __global__ void ref_to_planes_kernel(const float2* __restrict__ src, float2* __restrict__ dst, int B,
                                            int WW, int K) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)B * WW) return;
  const size_t b = idx / WW, e = idx % WW;
  for (int k = 0; k < K; ++k) dst[(b * K + k) * WW + e] = src[idx * K + k];
}

// A caller-given propagator P (W x W, mask applied, the reference's
// master_propagator_phase_space) and band-limit mask as the kernels' tables: P / W^2,
// P^edge / W^2 (principal branch) and mask / W^2.
template <int W>
__global__ void external_tables_kernel(const float2* __restrict__ P, const float* __restrict__ mask_clean,
                                       float edge, int use_edge, float2* __restrict__ prop,
                                       float2* __restrict__ prop_edge, float* __restrict__ mask,
                                       float* __restrict__ mask_sc, float2* __restrict__ pyx) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < 2 * W) pyx[idx] = make_float2(0.f, 0.f);   // separable factors unused here
  if (idx >= W * W) return;
  const float inv = 1.0f / (float)(W * W);
  const float2 p = P[idx];
  prop[idx] = make_float2(p.x * inv, p.y * inv);
  if (use_edge) {
    const float r = sqrtf(p.x * p.x + p.y * p.y);
    float2 pe = make_float2(0.f, 0.f);
    if (r > 0.f) {
      const float ang = atan2f(p.y, p.x) * edge;
      const float re = powf(r, edge);
      float se, ce;
      sincosf(ang, &se, &ce);
      pe = make_float2(re * ce, re * se);
    }
    prop_edge[idx] = make_float2(pe.x * inv, pe.y * inv);
  }
  const float mk = mask_clean ? mask_clean[idx] : 1.0f;
  mask[idx] = mk;
  mask_sc[idx] = mk * inv;
}

// ------------------------------------------------------------------ gradient windows
// Sum the nsum probe-mode contributions of a gradient window in ascending mode order
// (multislice_core.py:184-188) and band-limit the sum: IFFT(FFT(G) * mask)
// (multislice_core.py:189-191). Window w's contributions are the nsum consecutive native
// windows at buf + w * nsum * W^2; the result, in natural (y, x) layout, overwrites the first.
template <int W>
__global__ void __launch_bounds__(Geo<W>::T) grad_windows_kernel(float2* buf, const float* __restrict__ mask_sc,
                                                                 const float2* __restrict__ g_tw, int nsum) {
  using G = Geo<W>;
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  load_twiddles<W>(tw1, tw2, g_tw);
  const int t = threadIdx.x;
  float2* win = buf + (size_t)blockIdx.x * nsum * W * W;
  float2 v[32];
  ld_native<W>(win, v);
  for (int p = 1; p < nsum; ++p) {
    const float4* src = reinterpret_cast<const float4*>(win + (size_t)p * W * W);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float4 q = src[j * G::T + t];
      v[2 * j] = cadd(v[2 * j], make_float2(q.x, q.y));
      v[2 * j + 1] = cadd(v[2 * j + 1], make_float2(q.z, q.w));
    }
  }
  __syncthreads();
  WinFFT<W>::forward(v, xbuf, tw1, tw2);
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = cscale(v[i], mask_sc[G::fky(t, i) * W + G::fkx(t, i)]);
  WinFFT<W>::inverse(v, xbuf, tw1, tw2);
  // all reads of this window finished before the first barrier of forward()
#pragma unroll
  for (int i = 0; i < 32; ++i) win[G::ry(t) * W + G::rx(t, i)] = v[i];
}

// ------------------------------------------------------------------ deterministic scatter
// Object-gradient accumulation without atomics: the object plane is cut into TS x TS tiles;
// for every tile the positions whose window overlaps it are listed in batch order, and the
// block owning the tile adds their contributions pixel by pixel in that order
// (the fixed order of np.add.at in multislice_core.py:226-227).
constexpr int TS = 32;

static __global__ void tile_lists_kernel(const int* __restrict__ pos, const int* __restrict__ seq, int Bb,
                                  int W, int ntx, int* __restrict__ lists, int* __restrict__ counts) {
  __shared__ int warp_tot[32];
  __shared__ int base_s;
  const int tile = blockIdx.x;
  const int ty0 = (tile / ntx) * TS, tx0 = (tile % ntx) * TS;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) base_s = 0;
  __syncthreads();
  int* my = lists + (size_t)tile * Bb;
  for (int b0 = 0; b0 < Bb; b0 += blockDim.x) {
    const int b = b0 + threadIdx.x;
    bool hit = false;
    if (b < Bb) {
      const int gi = seq[b];
      const int y = pos[2 * gi], x = pos[2 * gi + 1];
      hit = (y < ty0 + TS) && (y + W > ty0) && (x < tx0 + TS) && (x + W > tx0);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) warp_tot[warp] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < nw; ++w) {
      if (w < warp) before += warp_tot[w];
      total += warp_tot[w];
    }
    const int base = base_s;
    if (hit) my[base + before + __popc(bal & ((1u << lane) - 1u))] = b;
    __syncthreads();
    if (threadIdx.x == 0) base_s = base + total;
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[tile] = base_s;
}

// Window (b, k) of gw starts at ((b * zm + k) * wmul) * W^2 (wmul = probe modes when the
// windows hold per-mode contributions whose first slot carries the sum).
// blockDim = (32, 8); grid = (ntiles, Z*Mo, groups). With groups = 1 a block adds its tile's
// whole list onto the gradient plane. With groups > 1 (few tiles: a small object or a single
// slice) the list is cut into `groups` consecutive runs; block (tile, k, g) sums run g alone
// into part[g][k][tile], and the last of the tile's run blocks to finish (an integer counter per
// (slice, tile) in `done`, zero before the launch and reset by that block) adds the runs onto
// the plane in run order -- still a fixed order, now with groups x more blocks at work.
static __global__ void scatter_tiles_kernel(const float2* __restrict__ gw, const int* __restrict__ pos,
                                     const int* __restrict__ seq, const int* __restrict__ lists,
                                     const int* __restrict__ counts, float2* __restrict__ grad,
                                     int Bb, int W, int Ny, int Nx, int ntx, int zm, int accumulate,
                                     int groups = 1, float2* __restrict__ part = nullptr, int wmul = 1,
                                     int* __restrict__ done = nullptr) {
  __shared__ int s_b[256], s_y[256], s_x[256];
  __shared__ int s_last;
  const int tile = blockIdx.x, k = blockIdx.y, g = blockIdx.z;
  const int ty0 = (tile / ntx) * TS, tx0 = (tile % ntx) * TS;
  const int lx = threadIdx.x, ly = threadIdx.y, tid = ly * 32 + lx;
  const int x = tx0 + lx;
  float2 acc[4];
  float2* plane = grad + (size_t)k * Ny * Nx;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int y = ty0 + ly + 8 * r;
    acc[r] = (groups == 1 && accumulate && y < Ny && x < Nx) ? plane[(size_t)y * Nx + x] : make_float2(0.f, 0.f);
  }
  const int n_all = counts[tile];
  const int per = (n_all + groups - 1) / groups;
  const int jb = min(n_all, g * per), n = min(n_all, jb + per);
  const int* lst = lists + (size_t)tile * Bb;
  const size_t WW = (size_t)W * W;
  for (int j0 = jb; j0 < n; j0 += 256) {
    __syncthreads();
    if (j0 + tid < n) {
      const int b = lst[j0 + tid];
      const int gi = seq[b];
      s_b[tid] = b;
      s_y[tid] = pos[2 * gi];
      s_x[tid] = pos[2 * gi + 1];
    }
    __syncthreads();
    const int jn = min(256, n - j0);
    int j = 0;
    // groups of four windows: all their loads first, then the adds in window order (the
    // same order and the same skipped pixels as one window at a time)
    for (; j + 4 <= jn; j += 4) {
      float2 val[4][4];
      bool ok[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int ox = x - s_x[j + u];
        const bool inx = (unsigned)ox < (unsigned)W;
        const float2* src = gw + ((size_t)s_b[j + u] * zm + k) * wmul * WW + (inx ? ox : 0);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int oy = ty0 + ly + 8 * r - s_y[j + u];
          ok[u][r] = inx && (unsigned)oy < (unsigned)W;
          val[u][r] = ok[u][r] ? src[(size_t)oy * W] : make_float2(0.f, 0.f);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int r = 0; r < 4; ++r)
          if (ok[u][r]) acc[r] = cadd(acc[r], val[u][r]);
    }
    for (; j < jn; ++j) {
      const int b = s_b[j];
      const int ox = x - s_x[j];
      if ((unsigned)ox >= (unsigned)W) continue;
      const float2* src = gw + ((size_t)b * zm + k) * wmul * WW + ox;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int oy = ty0 + ly + 8 * r - s_y[j];
        if ((unsigned)oy < (unsigned)W) acc[r] = cadd(acc[r], src[(size_t)oy * W]);
      }
    }
  }
  if (groups > 1) {
    float2* pt = part + (((size_t)g * zm + k) * (gridDim.x) + tile) * (TS * TS);
#pragma unroll
    for (int r = 0; r < 4; ++r) pt[(ly + 8 * r) * TS + lx] = acc[r];
    // the last of the tile's run blocks to finish adds the runs in run order; the integer
    // counter only decides which block that is
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&done[k * gridDim.x + tile], 1) == groups - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    float2 sum[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int y = ty0 + ly + 8 * r;
      sum[r] = (accumulate && y < Ny && x < Nx) ? plane[(size_t)y * Nx + x] : make_float2(0.f, 0.f);
    }
    for (int gg = 0; gg < groups; ++gg) {
      const float2* pg = part + (((size_t)gg * zm + k) * gridDim.x + tile) * (TS * TS);
#pragma unroll
      for (int r = 0; r < 4; ++r) sum[r] = cadd(sum[r], __ldcg(pg + (ly + 8 * r) * TS + lx));
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int y = ty0 + ly + 8 * r;
      if (y < Ny && x < Nx) plane[(size_t)y * Nx + x] = sum[r];
    }
    if (tid == 0) done[k * gridDim.x + tile] = 0;   // ready for the next batch's launch
    return;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int y = ty0 + ly + 8 * r;
    if (y < Ny && x < Nx) plane[(size_t)y * Nx + x] = acc[r];
  }
}

// ------------------------------------------------------------------ probe gradient
// partial[c][p][e] (+)= sum over positions b of chunk c of fprobe[b][p][e], in order
static __global__ void probe_partial_kernel(const float2* __restrict__ fprobe, float2* __restrict__ partial,
                                     int Bb, int Mp, int WW, int chunk, int accumulate) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y, c = blockIdx.z;
  if (e >= WW) return;
  float2 s = make_float2(0.f, 0.f);
  const int b1 = min(Bb, (c + 1) * chunk);
  for (int b = c * chunk; b < b1; ++b) s = cadd(s, fprobe[((size_t)b * Mp + p) * WW + e]);
  float2* dst = partial + ((size_t)c * Mp + p) * WW + e;
  *dst = accumulate ? cadd(*dst, s) : s;
}

// partial[0][p][e] = sum over c of partial[c][p][e] in chunk order (0 + partial[0] + partial[1]
// + ..., the order probe_final_kernel would add them in), one thread per element: the chunk sum
// spread over the whole GPU instead of the final kernel's one block per mode.
static __global__ void probe_chunks_kernel(float2* __restrict__ partial, int nchunk, int Mp, int WW) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  if (e >= WW) return;
  float2 s = make_float2(0.f, 0.f);
  for (int c = 0; c < nchunk; ++c) s = cadd(s, partial[((size_t)c * Mp + p) * WW + e]);
  partial[(size_t)p * WW + e] = s;
}

// probe_grad = IFFT(mask * sum_c partial[c]) (objective.py:703 and :927-933), written in the
// reference layout (W, W, Mp)
template <int W>
__global__ void __launch_bounds__(Geo<W>::T) probe_final_kernel(const float2* __restrict__ partial, int nchunk,
                                                                int Mp, const float* __restrict__ mask_sc,
                                                                const float2* __restrict__ g_tw,
                                                                float2* __restrict__ probe_grad) {
  using G = Geo<W>;
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  load_twiddles<W>(tw1, tw2, g_tw);
  __syncthreads();
  const int t = threadIdx.x, p = blockIdx.x;
  const size_t WW = (size_t)W * W;
  // chunks outer, elements inner: each chunk's 32 loads are independent and in flight
  // together (the chunk order of every element's sum is unchanged)
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = make_float2(0.f, 0.f);
  for (int c = 0; c < nchunk; ++c) {
    const float2* src = partial + ((size_t)c * Mp + p) * WW;
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = cadd(v[i], src[nidx<W>(i, t)]);
  }
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = cscale(v[i], mask_sc[G::fky(t, i) * W + G::fkx(t, i)]);
  WinFFT<W>::inverse(v, xbuf, tw1, tw2);
#pragma unroll
  for (int i = 0; i < 32; ++i) probe_grad[(size_t)(G::ry(t) * W + G::rx(t, i)) * Mp + p] = v[i];
}

// ------------------------------------------------------------------ scalars
// loss = w * sum(loss_part), sse = sum(sse_part) in FP64 (fixed order); the position
// gradient pos_grad[seq[b]] = -2/W^2 * sum_p pos_part[b][p]  (objective.py:651-656)
static __global__ void finalize_scalars_kernel(const double* __restrict__ loss_part,
                                        const double* __restrict__ pos_part, const int* __restrict__ seq,
                                        int nseq, int Mp, int W, double loss_weight, int step_pos,
                                        const int* __restrict__ err, double* __restrict__ loss_sse,
                                        float* __restrict__ pos_grad) {
  __shared__ double red[64];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nseq; i += blockDim.x) {
    a += loss_part[2 * i];
    b += loss_part[2 * i + 1];
  }
  block_sum2(a, b, red);
  if (threadIdx.x == 0) {
    // a device-side wait that ran out leaves the result unusable: report it as a NaN loss
    const bool failed = err != nullptr && *err != 0;
    loss_sse[0] = failed ? __longlong_as_double(0x7ff8000000000000ll) : a * loss_weight;
    loss_sse[1] = b;
  }
  if (!step_pos) return;
  // A position that appears more than once in the sequence keeps the gradient of its last
  // occurrence, as the reference's batch-by-batch assignment pos_grad[tcs] = ... leaves it
  // (objective.py:655-656): the sequence is walked in rounds of blockDim.x entries separated
  // by barriers, and inside a round an entry writes only if no later entry of the round has
  // the same position.
  __shared__ int sseq[256];
  const double sh = -2.0 / ((double)W * (double)W);
  for (int base = 0; base < nseq; base += blockDim.x) {
    const int i = base + (int)threadIdx.x;
    const int s = i < nseq ? seq[i] : -1;
    __syncthreads();   // the previous round's comparisons are done
    sseq[threadIdx.x] = s;
    __syncthreads();
    if (i >= nseq) continue;
    const int nr = min((int)blockDim.x, nseq - base);
    bool later = false;
    for (int j = (int)threadIdx.x + 1; j < nr; ++j) later |= (sseq[j] == s);
    if (later) continue;
    double gy = 0.0, gx = 0.0;
    for (int p = 0; p < Mp; ++p) {
      gy += pos_part[((size_t)i * Mp + p) * 2];
      gx += pos_part[((size_t)i * Mp + p) * 2 + 1];
    }
    pos_grad[2 * s] = (float)(sh * gy);
    pos_grad[2 * s + 1] = (float)(sh * gx);
  }
}

// ------------------------------------------------------------------ plain batched FFT
// fft2 / ifft2 / shift_fft2 / ifft2_ishift of contiguous W x W windows (pypty/fft.py:91-178)
template <int W>
__global__ void __launch_bounds__(Geo<W>::T) fft2_batch_kernel(const float2* __restrict__ in, float2* __restrict__ out,
                                                               int inverse, int shift,
                                                               const float2* __restrict__ g_tw) {
  using G = Geo<W>;
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  load_twiddles<W>(tw1, tw2, g_tw);
  __syncthreads();
  const int t = threadIdx.x;
  const size_t WW = (size_t)W * W;
  const float2* src = in + (size_t)blockIdx.x * WW;
  float2* dst = out + (size_t)blockIdx.x * WW;
  float2 v[32];
  const int h = shift ? W / 2 : 0;
  if (!inverse) {
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = src[G::ry(t) * W + G::rx(t, i)];
    WinFFT<W>::forward(v, xbuf, tw1, tw2);
#pragma unroll
    for (int i = 0; i < 32; ++i)
      dst[((G::fky(t, i) + h) & (W - 1)) * W + ((G::fkx(t, i) + h) & (W - 1))] = v[i];
  } else {
    const float inv = 1.0f / (float)WW;
#pragma unroll
    for (int i = 0; i < 32; ++i)
      v[i] = cscale(src[((G::fky(t, i) + h) & (W - 1)) * W + ((G::fkx(t, i) + h) & (W - 1))], inv);
    WinFFT<W>::inverse(v, xbuf, tw1, tw2);
#pragma unroll
    for (int i = 0; i < 32; ++i) dst[G::ry(t) * W + G::rx(t, i)] = v[i];
  }
}

// One propagation step of a batch of windows (or, with rtab, one band limit by a real mask):
// out = IFFT(FFT(in) * P) (conj: conj(P)); gout, when given, receives FFT(in) * P * gscale with
// P = tab[k] (natural (ky, kx)) and the inverse's 1/W^2 applied as `scale` (1 for tables that
// fold it in already), one table per group of nper windows (tab_stride elements apart; 0: one
// table). The same products and rounding as fft2 -> multiply -> ifft2.   grid n windows
template <int W>
__global__ void __launch_bounds__(Geo<W>::T) prop_step_kernel(const float2* in, float2* out,   // may alias
                                                              const float2* __restrict__ tab, size_t tab_stride,
                                                              int nper, int conj, float scale,
                                                              const float2* __restrict__ g_tw,
                                                              const float* __restrict__ rtab = nullptr,
                                                              float2* __restrict__ gout = nullptr,
                                                              float gscale = 1.0f) {
  using G = Geo<W>;
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  load_twiddles<W>(tw1, tw2, g_tw);
  __syncthreads();
  const int t = threadIdx.x;
  const size_t WW = (size_t)W * W;
  const float2* src = in + (size_t)blockIdx.x * WW;
  float2* dst = out + (size_t)blockIdx.x * WW;
  const float2* P = tab + (size_t)(blockIdx.x / nper) * tab_stride;
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = src[G::ry(t) * W + G::rx(t, i)];
  WinFFT<W>::forward(v, xbuf, tw1, tw2);
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int k = G::fky(t, i) * W + G::fkx(t, i);
    if (rtab) {   // a real table (the band-limit mask)
      v[i] = cscale(cscale(v[i], rtab[k]), scale);
    } else {
      const float2 pk = P[k];
      const float2 prod = conj ? cmulc(v[i], pk) : cmul(v[i], pk);
      if (gout) gout[(size_t)blockIdx.x * WW + k] = cscale(prod, gscale);   // the product spectrum
      v[i] = cscale(prod, scale);
    }
  }
  __syncthreads();   // the inverse reuses the exchange buffer
  WinFFT<W>::inverse(v, xbuf, tw1, tw2);
#pragma unroll
  for (int i = 0; i < 32; ++i) dst[G::ry(t) * W + G::rx(t, i)] = v[i];
}

// One forward multislice step of a batch of windows (multislice_core.py:61-80) in one pass:
// in = z == 0 ? the position's incoming probe (mode p) : psi; stack[b][z][p][m] = conj(in);
// psi = IFFT(FFT(in * O[b][z][m]) * P), P as in prop_step_kernel; spec_out, when given,
// receives FFT(in * O).   grid Bn * Mp * Mo windows
template <int W>
__global__ void __launch_bounds__(Geo<W>::T) fwd_prop_kernel(const float2* __restrict__ pin, size_t pin_stride,
                                                             float2* psi, float2* __restrict__ stack,
                                                             const float2* __restrict__ ob, int z, int Z, int Mp,
                                                             int Mo, const float2* __restrict__ tab,
                                                             size_t tab_stride, float scale,
                                                             const float2* __restrict__ g_tw,
                                                             float2* __restrict__ spec_out) {
  using G = Geo<W>;
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *xbuf, *tw1, *tw2;
  double* red;
  carve<W>(smem, xbuf, tw1, tw2, red);
  load_twiddles<W>(tw1, tw2, g_tw);
  __syncthreads();
  const int t = threadIdx.x;
  const size_t WW = (size_t)W * W;
  const int nm = Mp * Mo, wi = blockIdx.x, b = wi / nm, pm = wi % nm, p = pm / Mo, m = pm % Mo;
  const float2* src = z == 0 ? pin + (size_t)b * pin_stride + (size_t)p * WW : psi + (size_t)wi * WW;
  float2* st = stack + (((size_t)b * Z + z) * nm + pm) * WW;
  const float2* o = ob + (((size_t)b * Z + z) * Mo + m) * WW;
  const float2* P = tab + (size_t)b * tab_stride;
  float2 v[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int u = G::ry(t) * W + G::rx(t, i);
    const float2 in = src[u];
    st[u] = cconj(in);
    v[i] = cmul(in, o[u]);
  }
  WinFFT<W>::forward(v, xbuf, tw1, tw2);
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int k = G::fky(t, i) * W + G::fkx(t, i);
    if (spec_out) spec_out[(size_t)wi * WW + k] = v[i];   // FFT(in O), kept for the inside-tilt gradient
    v[i] = cscale(cmul(v[i], P[k]), scale);
  }
  __syncthreads();   // the inverse reuses the exchange buffer
  WinFFT<W>::inverse(v, xbuf, tw1, tw2);
  float2* dst = psi + (size_t)wi * WW;
#pragma unroll
  for (int i = 0; i < 32; ++i) dst[G::ry(t) * W + G::rx(t, i)] = v[i];
}

}  // namespace pty

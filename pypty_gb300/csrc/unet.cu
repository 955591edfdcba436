// Learned warm start: the kernels of a small convolutional network (a 4-level U-Net) that
// predicts an object phase stack from per-position centre-of-mass and virtual-bright-field
// maps, trained on specimens simulated with this library's own forward model. No counterpart
// in the reference: its warm starts are non-learned (pypty/initialize.py:629
// get_ptycho_obj_from_scan; the centre-of-mass definition follows pypty/dpc.py:137-151).
//
// Activations and their gradients are BF16 (NCHW); every product accumulates in FP32; weights,
// weight gradients and the Adam state are FP32. Reductions over pixels (weight gradients, the
// loss) go through fixed per-block partial sums and a fixed-order final sum: training is
// deterministic run to run.
//
// conv3x3_kernel: a CTA computes a 32 x 32 pixel tile for 16 output channels; each thread a
// 2 x 2 pixel quad for those 16 channels (64 FP32 accumulators); input channels stream through
// shared memory 8 at a time with a one-pixel zero-padded halo; the weights of a chunk are read
// as float4 broadcasts (16 FMAs per weight load). The transposed-and-flipped weight view gives
// the data gradient with the same kernel.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"

namespace pty {
namespace nn {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ float ld(const bf16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ bf16 to_bf(float x) { return __float2bfloat16_rn(x); }

constexpr int TS = 32;    // output tile edge
constexpr int COT = 16;   // output channels per CTA
constexpr int CIT = 8;    // input channels per shared-memory chunk
constexpr int HALO = TS + 2;

// TRANS = 0: out[n][o] = act(b[o] + sum_i sum_t w[o][i][t] x[n][i][p + off(t)])   (forward)
// TRANS = 1: out[n][o] =          sum_i sum_t w[i][o][8 - t] x[n][i][p + off(t)]    (data gradient;
//            o runs over the layer's input channels, i over its output channels)
template <int TRANS, int RELU>
__global__ void __launch_bounds__(256) conv3x3_kernel(const bf16* __restrict__ x, const float* __restrict__ w,
                                                      const float* __restrict__ bias, bf16* __restrict__ out, int Ci,
                                                      int Co, int H, int Wd) {
  __shared__ float xs[CIT][HALO][HALO + 1];
  __shared__ __align__(16) float ws[CIT][9][COT];
  const int tiles_x = Wd / TS;
  const int ty0 = (blockIdx.x / tiles_x) * TS, tx0 = (blockIdx.x % tiles_x) * TS;
  const int o0 = blockIdx.y * COT, n = blockIdx.z;
  const int t = threadIdx.x, qx = (t & 15) * 2, qy = (t >> 4) * 2;
  float acc[4][COT];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int c = 0; c < COT; ++c) acc[p][c] = 0.f;
  const size_t plane = (size_t)H * Wd;
  for (int i0 = 0; i0 < Ci; i0 += CIT) {
    __syncthreads();
    for (int e = t; e < CIT * HALO * HALO; e += 256) {
      const int ci = e / (HALO * HALO), r = (e / HALO) % HALO, c = e % HALO;
      const int y = ty0 + r - 1, xx = tx0 + c - 1;
      float v = 0.f;
      if (i0 + ci < Ci && y >= 0 && y < H && xx >= 0 && xx < Wd) v = ld(x + ((size_t)n * Ci + i0 + ci) * plane + (size_t)y * Wd + xx);
      xs[ci][r][c] = v;
    }
    for (int e = t; e < CIT * 9 * COT; e += 256) {
      const int ci = e / (9 * COT), tap = (e / COT) % 9, co = e % COT;
      const int i = i0 + ci, o = o0 + co;
      float v = 0.f;
      if (i < Ci && o < Co) v = TRANS ? w[((size_t)i * Co + o) * 9 + (8 - tap)] : w[((size_t)o * Ci + i) * 9 + tap];
      ws[ci][tap][co] = v;
    }
    __syncthreads();
#pragma unroll 2
    for (int ci = 0; ci < CIT; ++ci) {
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
        const float v0 = xs[ci][qy + dy][qx + dx], v1 = xs[ci][qy + dy][qx + 1 + dx];
        const float v2 = xs[ci][qy + 1 + dy][qx + dx], v3 = xs[ci][qy + 1 + dy][qx + 1 + dx];
        const float4* wp = reinterpret_cast<const float4*>(&ws[ci][tap][0]);
#pragma unroll
        for (int c4 = 0; c4 < COT / 4; ++c4) {
          const float4 wv = wp[c4];
          const float wl[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            acc[0][4 * c4 + j] = fmaf(wl[j], v0, acc[0][4 * c4 + j]);
            acc[1][4 * c4 + j] = fmaf(wl[j], v1, acc[1][4 * c4 + j]);
            acc[2][4 * c4 + j] = fmaf(wl[j], v2, acc[2][4 * c4 + j]);
            acc[3][4 * c4 + j] = fmaf(wl[j], v3, acc[3][4 * c4 + j]);
          }
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < COT; ++c) {
    const int o = o0 + c;
    if (o >= Co) break;
    const float b = (!TRANS && bias) ? bias[o] : 0.f;
    bf16* op = out + ((size_t)n * Co + o) * plane;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      float v = acc[p][c] + b;
      if (RELU) v = fmaxf(v, 0.f);
      const int y = ty0 + qy + (p >> 1), xx = tx0 + qx + (p & 1);
      op[(size_t)y * Wd + xx] = to_bf(v);
    }
  }
}

// Weight and bias gradients of a 3x3 convolution, per (32 x 32 tile, image) partial sums:
//   part[blk][o][i][t] = sum_{p in tile} dy[n][o][p] x[n][i][p + off(t)],  pb[blk][o] = sum dy[n][o][p]
// grid (tiles * N, Co / COT, Ci / CIT); thread = (o, i) pair of the CTA's 16 x 8 block, half the rows.
struct WgradSmem {
  float xs[CIT][HALO][HALO + 1];
  float ds[COT][TS][TS + 1];
  float red[256][10];
};

__global__ void __launch_bounds__(256) conv3x3_wgrad_kernel(const bf16* __restrict__ dy, const bf16* __restrict__ x,
                                                            float* __restrict__ part, float* __restrict__ pbias,
                                                            int Ci, int Co, int H, int Wd, int N) {
  extern __shared__ __align__(16) unsigned char wg_smem[];
  WgradSmem& S = *reinterpret_cast<WgradSmem*>(wg_smem);
  auto& xs = S.xs;
  auto& ds = S.ds;
  auto& red = S.red;
  const int tiles_x = Wd / TS, tiles = (H / TS) * tiles_x;
  const int tile = blockIdx.x % tiles, n = blockIdx.x / tiles;
  const int ty0 = (tile / tiles_x) * TS, tx0 = (tile % tiles_x) * TS;
  const int o0 = blockIdx.y * COT, i0 = blockIdx.z * CIT;
  const int t = threadIdx.x;
  const size_t plane = (size_t)H * Wd;
  for (int e = t; e < CIT * HALO * HALO; e += 256) {
    const int ci = e / (HALO * HALO), r = (e / HALO) % HALO, c = e % HALO;
    const int y = ty0 + r - 1, xx = tx0 + c - 1;
    float v = 0.f;
    if (i0 + ci < Ci && y >= 0 && y < H && xx >= 0 && xx < Wd) v = ld(x + ((size_t)n * Ci + i0 + ci) * plane + (size_t)y * Wd + xx);
    xs[ci][r][c] = v;
  }
  for (int e = t; e < COT * TS * TS; e += 256) {
    const int co = e / (TS * TS), r = (e / TS) % TS, c = e % TS;
    float v = 0.f;
    if (o0 + co < Co) v = ld(dy + ((size_t)n * Co + o0 + co) * plane + (size_t)(ty0 + r) * Wd + tx0 + c);
    ds[co][r][c] = v;
  }
  __syncthreads();
  const int pair = t & 127, half = t >> 7;
  const int co = pair >> 3, ci = pair & 7;
  float a[9], sb = 0.f;
#pragma unroll
  for (int k = 0; k < 9; ++k) a[k] = 0.f;
  for (int r = half * 16; r < half * 16 + 16; ++r) {
    // sliding 3x3 window of x around (r, c): columns c-1, c, c+1 of rows r-1, r, r+1 (halo offset +1)
    float w0[3] = {xs[ci][r][0], xs[ci][r + 1][0], xs[ci][r + 2][0]};
    float w1[3] = {xs[ci][r][1], xs[ci][r + 1][1], xs[ci][r + 2][1]};
    for (int c = 0; c < TS; ++c) {
      const float w2[3] = {xs[ci][r][c + 2], xs[ci][r + 1][c + 2], xs[ci][r + 2][c + 2]};
      const float d = ds[co][r][c];
      sb += d;
#pragma unroll
      for (int dyy = 0; dyy < 3; ++dyy) {
        a[dyy * 3 + 0] = fmaf(d, w0[dyy], a[dyy * 3 + 0]);
        a[dyy * 3 + 1] = fmaf(d, w1[dyy], a[dyy * 3 + 1]);
        a[dyy * 3 + 2] = fmaf(d, w2[dyy], a[dyy * 3 + 2]);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        w0[k] = w1[k];
        w1[k] = w2[k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) red[t][k] = a[k];
  red[t][9] = sb;
  __syncthreads();
  if (half == 0) {
    const int o = o0 + co, i = i0 + ci;
    const size_t blk = blockIdx.x;
    if (o < Co && i < Ci) {
#pragma unroll
      for (int k = 0; k < 9; ++k) part[((blk * Co + o) * Ci + i) * 9 + k] = red[t][k] + red[t + 128][k];
    }
    if (ci == 0 && blockIdx.z == 0 && o < Co) pbias[blk * Co + o] = red[t][9] + red[t + 128][9];
  }
}

// dst[e] = sum_b src[b][e] in ascending b (the fixed-order reduction of per-block partials)
__global__ void reduce_blocks_kernel(const float* __restrict__ src, float* __restrict__ dst, int nblk, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  float s = 0.f;
  for (int b = 0; b < nblk; ++b) s += src[(size_t)b * n + e];
  dst[e] = s;
}

// 1x1 convolution (the output layer): out[n][o][p] = b[o] + sum_i w[o][i] x[n][i][p]
__global__ void conv1x1_kernel(const bf16* __restrict__ x, const float* __restrict__ w, const float* __restrict__ b,
                               bf16* __restrict__ out, int Ci, int Co, long long plane) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  if (p >= plane) return;
  float xv[64];
  for (int i = 0; i < Ci; ++i) xv[i] = ld(x + ((size_t)n * Ci + i) * plane + p);
  for (int o = 0; o < Co; ++o) {
    float s = b[o];
    for (int i = 0; i < Ci; ++i) s = fmaf(w[o * Ci + i], xv[i], s);
    out[((size_t)n * Co + o) * plane + p] = to_bf(s);
  }
}

// data gradient of the 1x1 convolution: dx[n][i][p] = sum_o w[o][i] dy[n][o][p]
__global__ void conv1x1_dgrad_kernel(const bf16* __restrict__ dy, const float* __restrict__ w, bf16* __restrict__ dx,
                                     int Ci, int Co, long long plane) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  if (p >= plane) return;
  float dv[64];
  for (int o = 0; o < Co; ++o) dv[o] = ld(dy + ((size_t)n * Co + o) * plane + p);
  for (int i = 0; i < Ci; ++i) {
    float s = 0.f;
    for (int o = 0; o < Co; ++o) s = fmaf(w[o * Ci + i], dv[o], s);
    dx[((size_t)n * Ci + i) * plane + p] = to_bf(s);
  }
}

// weight / bias gradient partials of the 1x1 convolution, one CTA per (pixel chunk of 4096, image),
// the chunk staged through shared memory 64 pixels at a time:
// part[blk][o * Ci + i] = sum_p dy[o][p] x[i][p], part[blk][Co * Ci + o] = sum_p dy[o][p]
constexpr int K1MAX = 17;   // outputs per thread: (64 * 64 + 64) / 256 rounded up
__global__ void __launch_bounds__(256) conv1x1_wgrad_kernel(const bf16* __restrict__ dy, const bf16* __restrict__ x,
                                                            float* __restrict__ part, int Ci, int Co, long long plane,
                                                            int chunks) {
  __shared__ float sdy[64][65], sx[64][65];
  const int n = blockIdx.x / chunks, ch = blockIdx.x % chunks;
  const long long p0 = (long long)ch * 4096;
  const int t = threadIdx.x;
  const int nout = Co * Ci + Co;
  float acc[K1MAX];
#pragma unroll
  for (int k = 0; k < K1MAX; ++k) acc[k] = 0.f;
  for (long long q0 = p0; q0 < p0 + 4096 && q0 < plane; q0 += 64) {
    __syncthreads();
    for (int e = t; e < 64 * 64; e += 256) {
      const int c = e / 64, j = e % 64;
      const long long p = q0 + j;
      sdy[c][j] = (c < Co && p < plane) ? ld(dy + ((size_t)n * Co + c) * plane + p) : 0.f;
      sx[c][j] = (c < Ci && p < plane) ? ld(x + ((size_t)n * Ci + c) * plane + p) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < K1MAX; ++kk) {
      const int k = t + 256 * kk;
      if (k < nout) {
        float s = 0.f;
        if (k < Co * Ci) {
          const int o = k / Ci, i = k % Ci;
          for (int j = 0; j < 64; ++j) s = fmaf(sdy[o][j], sx[i][j], s);
        } else {
          const int o = k - Co * Ci;
          for (int j = 0; j < 64; ++j) s += sdy[o][j];
        }
        acc[kk] += s;
      }
    }
  }
#pragma unroll
  for (int kk = 0; kk < K1MAX; ++kk) {
    const int k = t + 256 * kk;
    if (k < nout) part[(size_t)blockIdx.x * nout + k] = acc[kk];
  }
}

// dst += src (BF16, FP32 add)
__global__ void add_kernel(bf16* __restrict__ dst, const bf16* __restrict__ src, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) dst[e] = to_bf(ld(dst + e) + ld(src + e));
}

// dy *= (y > 0): the ReLU derivative from the post-activation output
__global__ void relu_mask_kernel(bf16* __restrict__ dy, const bf16* __restrict__ y, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n && !(ld(y + e) > 0.f)) dy[e] = to_bf(0.f);
}

// 2x2 average pooling and its adjoint
__global__ void avgpool2_kernel(const bf16* __restrict__ x, bf16* __restrict__ y, long long nplanes, int H, int Wd) {
  const int Ho = H / 2, Wo = Wd / 2;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nplanes * Ho * Wo) return;
  const long long pl = e / ((long long)Ho * Wo);
  const int r = (int)((e / Wo) % Ho), c = (int)(e % Wo);
  const bf16* xp = x + pl * H * Wd + (size_t)(2 * r) * Wd + 2 * c;
  y[e] = to_bf(0.25f * (ld(xp) + ld(xp + 1) + ld(xp + Wd) + ld(xp + Wd + 1)));
}
__global__ void avgpool2_back_kernel(const bf16* __restrict__ dy, bf16* __restrict__ dx, long long nplanes, int H, int Wd) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nplanes * H * Wd) return;
  const long long pl = e / ((long long)H * Wd);
  const int r = (int)((e / Wd) % H), c = (int)(e % Wd);
  dx[e] = to_bf(0.25f * ld(dy + pl * (H / 2) * (Wd / 2) + (size_t)(r / 2) * (Wd / 2) + c / 2));
}

// nearest 2x upsampling into channels [c_off, c_off + C) of a tensor with Ct channels, and its adjoint
__global__ void upsample2_kernel(const bf16* __restrict__ x, bf16* __restrict__ y, int N, int C, int Ct, int c_off, int H,
                                 int Wd) {
  const int Ho = 2 * H, Wo = 2 * Wd;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)N * C * Ho * Wo) return;
  const int c = (int)((e / ((long long)Ho * Wo)) % C), n = (int)(e / ((long long)C * Ho * Wo));
  const int r = (int)((e / Wo) % Ho), q = (int)(e % Wo);
  y[(((size_t)n * Ct + c_off + c) * Ho + r) * Wo + q] = x[(((size_t)n * C + c) * H + r / 2) * Wd + q / 2];
}
__global__ void upsample2_back_kernel(const bf16* __restrict__ dy, bf16* __restrict__ dx, int N, int C, int Ct, int c_off,
                                      int H, int Wd) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)N * C * H * Wd) return;
  const int c = (int)((e / ((long long)H * Wd)) % C), n = (int)(e / ((long long)C * H * Wd));
  const int r = (int)((e / Wd) % H), q = (int)(e % Wd);
  const bf16* p = dy + (((size_t)n * Ct + c_off + c) * 2 * H + 2 * r) * 2 * Wd + 2 * q;
  dx[e] = to_bf(ld(p) + ld(p + 1) + ld(p + 2 * Wd) + ld(p + 2 * Wd + 1));
}

// copy channels of x (N, C, plane) into / out of channels [c_off, c_off + C) of y (N, Ct, plane)
__global__ void channel_copy_kernel(const bf16* __restrict__ src, bf16* __restrict__ dst, int N, int C, int Ct,
                                    int c_off, long long plane, int into) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)N * C * plane) return;
  const long long p = e % plane;
  const int c = (int)((e / plane) % C), n = (int)(e / ((long long)C * plane));
  const size_t big = ((size_t)n * Ct + c_off + c) * plane + p;
  if (into) dst[big] = src[e];
  else dst[e] = src[big];
}

// dst (N, Cd, H, W) bf16, channel c < C: bilinear interpolation of src (N, C, h, w) float sampled
// at ((Y - oy) / sy, (X - ox) / sx) (the map grid placed in the output frame), zero outside the
// map; channels C .. Cd - 1 are zero
__global__ void bilinear_kernel(const float* __restrict__ src, bf16* __restrict__ dst, int N, int C, int Cd, int h,
                                int w, int H, int Wd, float oy, float ox, float sy, float sx) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)N * Cd * H * Wd) return;
  const int q = (int)(e % Wd), r = (int)((e / Wd) % H);
  const int c = (int)((e / ((long long)H * Wd)) % Cd), n = (int)(e / ((long long)Cd * H * Wd));
  float v = 0.f;
  const float fy = ((float)r - oy) / sy, fx = ((float)q - ox) / sx;
  if (c < C && fy >= 0.f && fx >= 0.f && fy <= (float)(h - 1) && fx <= (float)(w - 1)) {
    const int y0 = min((int)fy, h - 2), x0 = min((int)fx, w - 2);
    const float ay = fy - y0, ax = fx - x0;
    const float* s = src + ((size_t)n * C + c) * h * w;
    v = (1 - ay) * ((1 - ax) * s[y0 * w + x0] + ax * s[y0 * w + x0 + 1]) +
        ay * ((1 - ax) * s[(y0 + 1) * w + x0] + ax * s[(y0 + 1) * w + x0 + 1]);
  }
  dst[e] = to_bf(v);
}

// mean squared error: partial sums per CTA (FP64) and dpred = 2 (pred - target) / n
__global__ void __launch_bounds__(256) mse_kernel(const bf16* __restrict__ pred, const float* __restrict__ target,
                                                  bf16* __restrict__ dpred, double* __restrict__ part, long long n) {
  __shared__ double red[256];
  double s = 0.0;
  const float sc = 2.0f / (float)n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float d = ld(pred + e) - target[e];
    s += (double)d * d;
    dpred[e] = to_bf(sc * d);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Adam (Kingma & Ba 2015) with bias correction folded into the step size
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                            long long n, float lr_t, float b1, float b2, float eps) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float gg = g[e];
  const float mm = b1 * m[e] + (1.f - b1) * gg, vv = b2 * v[e] + (1.f - b2) * gg * gg;
  m[e] = mm;
  v[e] = vv;
  p[e] -= lr_t * mm / (sqrtf(vv) + eps);
}

// Per-pattern virtual detectors (pypty/dpc.py:137-151 centre of mass; a bright-field disk sum):
// out[3 * pos + 0] = sum k_x I / sum I, [1] = sum k_y I / sum I (pixels from the pattern centre,
// detector order), [2] = sum over k_x^2 + k_y^2 <= r_bf^2 of I.
__global__ void __launch_bounds__(256) virtual_detectors_kernel(const float* __restrict__ patterns, int W, float r_bf,
                                                                float* __restrict__ out) {
  __shared__ double red[4][256];
  const float* I = patterns + (size_t)blockIdx.x * W * W;
  double s = 0, sx = 0, sy = 0, sbf = 0;
  for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
    const float v = I[e];
    const int ky = e / W - W / 2, kx = e % W - W / 2;
    s += v;
    sx += (double)kx * v;
    sy += (double)ky * v;
    if ((float)(kx * kx + ky * ky) <= r_bf * r_bf) sbf += v;
  }
  red[0][threadIdx.x] = s;
  red[1][threadIdx.x] = sx;
  red[2][threadIdx.x] = sy;
  red[3][threadIdx.x] = sbf;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double tot = red[0][0] > 0 ? red[0][0] : 1.0;
    out[3 * blockIdx.x] = (float)(red[1][0] / tot);
    out[3 * blockIdx.x + 1] = (float)(red[2][0] / tot);
    out[3 * blockIdx.x + 2] = (float)red[3][0];
  }
}

// Phase slices of Gaussian atoms: phase[z][y][x] = sum_a amp_a exp(-((y - ya)^2 + (x - xa)^2) / (2 s^2))
// over the atoms of slice z (atoms: [z][a] = (y, x, amp) in pixels / rad); obj = exp(i phase).
__global__ void atoms_kernel(const float* __restrict__ atoms, int n_atoms, int Ny, int Nx, int Z, float sigma_px,
                             float* __restrict__ phase, float2* __restrict__ obj) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)Ny * Nx) return;
  const int y = (int)(e / Nx), x = (int)(e % Nx);
  const float inv = -0.5f / (sigma_px * sigma_px);
  const float cut = 5.f * sigma_px;
  for (int z = 0; z < Z; ++z) {
    const float* a = atoms + (size_t)z * n_atoms * 3;
    float s = 0.f;
    for (int k = 0; k < n_atoms; ++k) {
      const float dy = (float)y - a[3 * k], dx = (float)x - a[3 * k + 1];
      if (fabsf(dy) < cut && fabsf(dx) < cut) s += a[3 * k + 2] * __expf(inv * (dy * dy + dx * dx));
    }
    phase[(size_t)z * Ny * Nx + e] = s;
    if (obj) {
      float sn, cs;
      sincosf(s, &sn, &cs);
      obj[e * Z + z] = make_float2(cs, sn);   // (Ny, Nx, Z, 1) reference layout
    }
  }
}

inline int launch_ok() { return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA; }
inline unsigned nblk(long long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

}  // namespace nn
}  // namespace pty

using namespace pty;
using namespace pty::nn;

extern "C" {

int pty_nn_conv3x3(const void* x, const float* w, const float* bias, void* out, int32_t N, int32_t Ci, int32_t Co,
                   int32_t H, int32_t W, int32_t relu, int32_t transpose, void* stream) {
  if (!x || !w || !out || N <= 0 || Ci <= 0 || Co <= 0) return PTY_ERR_INVALID;
  if (H % TS || W % TS) return PTY_ERR_UNSUPPORTED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const dim3 grid((H / TS) * (W / TS), (Co + COT - 1) / COT, N);
  const bf16* xb = static_cast<const bf16*>(x);
  bf16* ob = static_cast<bf16*>(out);
  prof_mark(st, KID_NN);
  if (transpose) conv3x3_kernel<1, 0><<<grid, 256, 0, st>>>(xb, w, nullptr, ob, Ci, Co, H, W);
  else if (relu) conv3x3_kernel<0, 1><<<grid, 256, 0, st>>>(xb, w, bias, ob, Ci, Co, H, W);
  else conv3x3_kernel<0, 0><<<grid, 256, 0, st>>>(xb, w, bias, ob, Ci, Co, H, W);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_conv3x3_wgrad_workspace_floats(int32_t N, int32_t Ci, int32_t Co, int32_t H, int32_t W, int64_t* n) {
  if (!n || H % TS || W % TS) return PTY_ERR_INVALID;
  const long long blocks = (long long)N * (H / TS) * (W / TS);
  *n = blocks * ((long long)Co * Ci * 9 + Co);
  return PTY_OK;
}

int pty_nn_conv3x3_wgrad(const void* dy, const void* x, float* dw, float* db, int32_t N, int32_t Ci, int32_t Co,
                         int32_t H, int32_t W, float* workspace, void* stream) {
  if (!dy || !x || !dw || !db || !workspace) return PTY_ERR_INVALID;
  if (H % TS || W % TS) return PTY_ERR_UNSUPPORTED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int blocks = N * (H / TS) * (W / TS);
  float* part = workspace;
  float* pb = workspace + (size_t)blocks * Co * Ci * 9;
  if (cudaFuncSetAttribute(conv3x3_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(WgradSmem)) !=
      cudaSuccess)
    return PTY_ERR_CUDA;
  prof_mark(st, KID_NN);
  conv3x3_wgrad_kernel<<<dim3(blocks, (Co + COT - 1) / COT, (Ci + CIT - 1) / CIT), 256, sizeof(WgradSmem), st>>>(
      static_cast<const bf16*>(dy), static_cast<const bf16*>(x), part, pb, Ci, Co, H, W, N);
  const long long nw = (long long)Co * Ci * 9;
  prof_mark(st, KID_NN);
  reduce_blocks_kernel<<<nblk(nw), 256, 0, st>>>(part, dw, blocks, nw);
  prof_mark(st, KID_NN);
  reduce_blocks_kernel<<<nblk(Co), 256, 0, st>>>(pb, db, blocks, Co);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_conv1x1(const void* x, const float* w, const float* b, void* out, int32_t N, int32_t Ci, int32_t Co,
                   int64_t plane, void* stream) {
  if (!x || !w || !b || !out || Ci > 64 || Co > 64) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  conv1x1_kernel<<<dim3(nblk(plane), N), 256, 0, st>>>(static_cast<const bf16*>(x), w, b, static_cast<bf16*>(out), Ci,
                                                       Co, plane);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_conv1x1_backward(const void* dy, const void* x, const float* w, void* dx, float* dw, float* db, int32_t N,
                            int32_t Ci, int32_t Co, int64_t plane, float* workspace, void* stream) {
  if (!dy || !x || !w || !dw || !db || !workspace || Ci > 64 || Co > 64) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dx) {
    prof_mark(st, KID_NN);
    conv1x1_dgrad_kernel<<<dim3(nblk(plane), N), 256, 0, st>>>(static_cast<const bf16*>(dy), w, static_cast<bf16*>(dx),
                                                               Ci, Co, plane);
  }
  const int chunks = (int)((plane + 4095) / 4096);
  const int nout = Co * Ci + Co;
  prof_mark(st, KID_NN);
  conv1x1_wgrad_kernel<<<N * chunks, 256, 0, st>>>(static_cast<const bf16*>(dy), static_cast<const bf16*>(x), workspace,
                                                   Ci, Co, plane, chunks);
  float* sums = workspace + (size_t)N * chunks * nout;
  prof_mark(st, KID_NN);
  reduce_blocks_kernel<<<nblk(nout), 256, 0, st>>>(workspace, sums, N * chunks, nout);
  if (cudaMemcpyAsync(dw, sums, (size_t)Co * Ci * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(db, sums + (size_t)Co * Ci, (size_t)Co * sizeof(float), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return PTY_ERR_CUDA;
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_conv1x1_workspace_floats(int32_t N, int32_t Ci, int32_t Co, int64_t plane, int64_t* n) {
  if (!n) return PTY_ERR_INVALID;
  const long long chunks = (plane + 4095) / 4096;
  *n = ((long long)N * chunks + 1) * (Co * Ci + Co);
  return PTY_OK;
}

int pty_nn_add(void* dst, const void* src, int64_t n, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  add_kernel<<<nblk(n), 256, 0, st>>>(static_cast<bf16*>(dst), static_cast<const bf16*>(src), n);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_relu_mask(void* dy, const void* y, int64_t n, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  relu_mask_kernel<<<nblk(n), 256, 0, st>>>(static_cast<bf16*>(dy), static_cast<const bf16*>(y), n);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_avgpool2(const void* x, void* y, int64_t nplanes, int32_t H, int32_t W, int32_t backward, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  if (backward)
    avgpool2_back_kernel<<<nblk(nplanes * H * W), 256, 0, st>>>(static_cast<const bf16*>(x), static_cast<bf16*>(y),
                                                                nplanes, H, W);
  else
    avgpool2_kernel<<<nblk(nplanes * (H / 2) * (W / 2)), 256, 0, st>>>(static_cast<const bf16*>(x),
                                                                       static_cast<bf16*>(y), nplanes, H, W);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_upsample2(const void* x, void* y, int32_t N, int32_t C, int32_t Ct, int32_t c_off, int32_t H, int32_t W,
                     int32_t backward, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  if (backward)
    upsample2_back_kernel<<<nblk((long long)N * C * H * W), 256, 0, st>>>(
        static_cast<const bf16*>(x), static_cast<bf16*>(y), N, C, Ct, c_off, H, W);
  else
    upsample2_kernel<<<nblk((long long)N * C * 4 * H * W), 256, 0, st>>>(static_cast<const bf16*>(x),
                                                                          static_cast<bf16*>(y), N, C, Ct, c_off, H, W);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_channel_copy(const void* src, void* dst, int32_t N, int32_t C, int32_t Ct, int32_t c_off, int64_t plane,
                        int32_t into, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  channel_copy_kernel<<<nblk((long long)N * C * plane), 256, 0, st>>>(static_cast<const bf16*>(src),
                                                                      static_cast<bf16*>(dst), N, C, Ct, c_off, plane,
                                                                      into);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_bilinear(const float* src, void* dst, int32_t N, int32_t C, int32_t Cd, int32_t h, int32_t w, int32_t H,
                    int32_t W, float oy, float ox, float sy, float sx, void* stream) {
  if (h < 2 || w < 2 || H < 2 || W < 2 || sy <= 0.f || sx <= 0.f) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  bilinear_kernel<<<nblk((long long)N * Cd * H * W), 256, 0, st>>>(src, static_cast<bf16*>(dst), N, C, Cd, h, w, H, W,
                                                                    oy, ox, sy, sx);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_mse(const void* pred, const float* target, void* dpred, double* partials, int64_t n, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  mse_kernel<<<256, 256, 0, st>>>(static_cast<const bf16*>(pred), target, static_cast<bf16*>(dpred), partials, n);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_nn_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr_t, float b1, float b2, float eps,
                void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  adam_kernel<<<nblk(n), 256, 0, st>>>(p, g, m, v, n, lr_t, b1, b2, eps);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_virtual_detectors(const float* patterns, int32_t n_patterns, int32_t window, float r_bf, float* out,
                          void* stream) {
  if (!patterns || !out || n_patterns <= 0 || window <= 0) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  virtual_detectors_kernel<<<n_patterns, 256, 0, st>>>(patterns, window, r_bf, out);
  prof_mark(st, -1);
  return launch_ok();
}

int pty_atom_slices(const float* atoms, int32_t n_atoms, int32_t ny, int32_t nx, int32_t n_slices, float sigma_px,
                    float* phase, void* obj, void* stream) {
  if (!atoms || !phase || n_atoms <= 0) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_NN);
  atoms_kernel<<<nblk((long long)ny * nx), 256, 0, st>>>(atoms, n_atoms, ny, nx, n_slices, sigma_px, phase,
                                                         static_cast<float2*>(obj));
  prof_mark(st, -1);
  return launch_ok();
}

}  // extern "C"

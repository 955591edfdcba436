// 256 x 256 window FFT over a thread-block cluster of 4 blocks (512 threads each).
//
// Block c = (cy, cx) = (c >> 1, c & 1) owns, in real space, the polyphase component
// x[2y' + cy, 2x' + cx] (y', x' < 128) and, in frequency, the quadrant
// X[ky' + 128 cy, kx' + 128 cx]. A forward transform is
//   1. the register-resident 128 x 128 FFT of the block's component (WinFFT<128>),
//   2. the twiddle w_256^(ky' cy + kx' cx),
//   3. a radix-2 x 2 butterfly across the four blocks through distributed shared memory:
//      X_q = sum_r (-1)^(qy ry + qx rx) T_r  (block q keeps quadrant q);
// the inverse runs the same steps backwards with conjugate twiddles (unnormalised).
// Each block's part of a window is stored in the 128 native order (window_fft.cuh) at
// offset c * 128^2 of the window.
#pragma once
#include <cooperative_groups.h>

#include "window_fft.cuh"

namespace pty {

namespace cg256 = cooperative_groups;

struct Geo256 {
  using G = Geo<128>;
  static constexpr int W = 256;
  static constexpr int H = 128;
  static constexpr int T = G::T;                  // 512 threads per block
  static constexpr size_t PART = (size_t)H * H;    // elements per block
  static __device__ __forceinline__ int ry(int c, int t) { return 2 * G::ry(t) + (c >> 1); }
  static __device__ __forceinline__ int rx(int c, int t, int i) { return 2 * G::rx(t, i) + (c & 1); }
  static __device__ __forceinline__ int fky(int c, int t, int i) { return G::fky(t, i) + H * (c >> 1); }
  static __device__ __forceinline__ int fkx(int c, int t, int i) { return G::fkx(t, i) + H * (c & 1); }
};

// sign (-1)^(qy*ry + qx*rx) of the cross-block butterfly
__device__ __forceinline__ float quad_sign(int q, int r) {
  return (((q >> 1) & (r >> 1)) ^ ((q & 1) & (r & 1))) ? -1.0f : 1.0f;
}

// tw256[k] = exp(-2 pi i k / 256) into shared memory (256 entries)
__device__ __forceinline__ void load_tw256(float2* tw256) {
  for (int k = threadIdx.x; k < 256; k += blockDim.x) {
    float s, c;
    sincospif((float)k / 128.0f, &s, &c);   // exact argument: k/128 is dyadic
    tw256[k] = make_float2(c, -s);
  }
}

struct WinFFT256 {
  using G = Geo<128>;
  static constexpr int T = G::T;

  // Radix-2 x 2 butterfly across the four blocks, block `me` keeping output quadrant `me`:
  //   out_me = sum_r (-1)^(me_y r_y + me_x r_x) in_r.
  // It is separable: a stage with the x partner (me ^ 1) then a stage with the y partner
  // (me ^ 2). In each stage every block stores its values into the partner's exchange
  // buffer (remote shared-memory stores, which do not wait), the cluster synchronises, and
  // the block combines its own values with the partner's from its local buffer:
  //   bit of me clear: out = own + partner,  bit set: out = partner - own.
  static __device__ __forceinline__ void cross_stage(float2 (&v)[32], float2* xbuf, cg256::cluster_group& cl,
                                                     int me, int bit) {
    const int t = threadIdx.x;
    cl.sync();   // the partner has finished with its exchange buffer
    float2* dst = cl.map_shared_rank(xbuf, me ^ bit);
#pragma unroll
    for (int i = 0; i < 32; ++i) dst[nidx<128>(i, t)] = v[i];
    cl.sync();   // the partner's values have arrived
    const bool upper = (me & bit) != 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const float2 o = xbuf[nidx<128>(i, t)];
      v[i] = upper ? csub(o, v[i]) : cadd(v[i], o);
    }
  }

  static __device__ __forceinline__ void cross(float2 (&v)[32], float2* xbuf, cg256::cluster_group& cl, int me) {
    cross_stage(v, xbuf, cl, me, 1);
    cross_stage(v, xbuf, cl, me, 2);
    cl.sync();   // every block is done with the exchange buffers
  }

  static __device__ __forceinline__ void forward(float2 (&v)[32], float2* xbuf, const float2* tw1, const float2* tw2,
                                                 const float2* tw256, cg256::cluster_group& cl) {
    const int c = (int)cl.block_rank();
    const int t = threadIdx.x;
    WinFFT<128>::forward(v, xbuf, tw1, tw2);
    if (c != 0) {
      const int cy = c >> 1, cx = c & 1;
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = cmul(v[i], tw256[G::fky(t, i) * cy + G::fkx(t, i) * cx]);
    }
    cross(v, xbuf, cl, c);
  }

  static __device__ __forceinline__ void inverse(float2 (&v)[32], float2* xbuf, const float2* tw1, const float2* tw2,
                                                 const float2* tw256, cg256::cluster_group& cl) {
    const int c = (int)cl.block_rank();
    const int t = threadIdx.x;
    cross(v, xbuf, cl, c);
    if (c != 0) {
      const int cy = c >> 1, cx = c & 1;
#pragma unroll
      for (int i = 0; i < 32; ++i) v[i] = cmulc(v[i], tw256[G::fky(t, i) * cy + G::fkx(t, i) * cx]);
    }
    WinFFT<128>::inverse(v, xbuf, tw1, tw2);
  }
};

}  // namespace pty

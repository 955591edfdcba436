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

  // combine the four blocks' windows (held in their xbuf, native order) for block `me`:
  // out_i = sum_r sign(me, r) * block_r[i], r = 0, 1, 2, 3 in that order. The same code runs
  // in every block (only the signs differ); four elements per batch of shared-memory loads
  // keep the register footprint bounded.
  static __device__ __forceinline__ void cross(float2 (&v)[32], float2* xbuf, cg256::cluster_group& cl, int me) {
    const int t = threadIdx.x;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 32; ++i) xbuf[nidx<128>(i, t)] = v[i];
    cl.sync();
    const float2* r0 = cl.map_shared_rank(xbuf, 0);
    const float2* r1 = cl.map_shared_rank(xbuf, 1);
    const float2* r2 = cl.map_shared_rank(xbuf, 2);
    const float2* r3 = cl.map_shared_rank(xbuf, 3);
    const float s1 = quad_sign(me, 1), s2 = quad_sign(me, 2), s3 = quad_sign(me, 3);
#pragma unroll
    for (int i0 = 0; i0 < 32; i0 += 4) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int e = nidx<128>(i0 + k, t);
        const float2 a = r0[e], b = r1[e], c = r2[e], d = r3[e];
        v[i0 + k] = make_float2(fmaf(s3, d.x, fmaf(s2, c.x, fmaf(s1, b.x, a.x))),
                                fmaf(s3, d.y, fmaf(s2, c.y, fmaf(s1, b.y, a.y))));
      }
      asm volatile("" ::: "memory");   // keep the next batch's loads after this one
    }
    cl.sync();   // every block is done reading the others' xbuf
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

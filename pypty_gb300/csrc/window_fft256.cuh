// 256 x 256 window FFT over a thread-block cluster of 4 blocks (512 threads each).
//
// Block c = (cy, cx) = (c >> 1, c & 1) owns, in real space, the polyphase component
// x[2y' + cy, 2x' + cx] (y', x' < 128) and, in frequency, the quadrant
// X[ky' + 128 cy, kx' + 128 cx]. A forward transform is
//   1. the register-resident 128 x 128 FFT of the block's component (WinFFT<128>),
//   2. the twiddle w_256^(ky' cy + kx' cx),
//   3. a radix-2 x 2 butterfly across the four blocks through distributed shared memory:
//      X_q = sum_r (-1)^(qy ry + qx rx) T_r  (block q keeps quadrant q), one exchange in
//      which every block publishes its values and pulls the three partners' values;
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

// tw256[k] = exp(-2 pi i k / 256) into shared memory (256 entries)
__device__ __forceinline__ void load_tw256(float2* tw256) {
  for (int k = threadIdx.x; k < 256; k += blockDim.x) {
    float s, c;
    sincospif((float)k / 128.0f, &s, &c);   // exact argument: k/128 is dyadic
    tw256[k] = make_float2(c, -s);
  }
}

// shared::cluster address of `p` (this block's shared memory) in block `rank` of the cluster
__device__ __forceinline__ uint32_t cluster_map(const void* p, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}

__device__ __forceinline__ float4 ld_cluster_f4(uint32_t addr) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr)
               : "memory");
  return v;
}

struct WinFFT256 {
  using G = Geo<128>;
  static constexpr int T = G::T;

  // Every block stores its 32 values (element pairs as 16-byte words, native order) into its
  // own exchange buffer; after the cluster barrier the partners pull them with
  // ld.shared::cluster. The caller ends the exchange with end_exchange.
  static __device__ __forceinline__ void publish(const float2 (&v)[32], float2* xbuf, cg256::cluster_group& cl) {
    const int t = threadIdx.x;
    __syncthreads();   // this block's own transform has finished reading xbuf
    float4* p = reinterpret_cast<float4*>(xbuf);
#pragma unroll
    for (int j = 0; j < 16; ++j) p[j * T + t] = make_float4(v[2 * j].x, v[2 * j].y, v[2 * j + 1].x, v[2 * j + 1].y);
    cl.sync();   // every block's values are published
  }
  static __device__ __forceinline__ void end_exchange(cg256::cluster_group& cl) {
    cl.sync();   // every partner has read this block's buffer before it is reused
  }

  // Radix-2 x 2 butterfly across the four blocks, block `me` keeping output quadrant `me`:
  //   out_me = sum_r (-1)^(me_y r_y + me_x r_x) in_r.
  // With R_d = in_(me ^ d) (R_0 the block's own value) and s_x, s_y = -1 where bit x / y of
  // `me` is set: out_me = R_3 + s_x R_2 + s_y R_1 + s_x s_y R_0. One exchange: the block
  // publishes its values and pulls those of the three partners.
  static __device__ __forceinline__ void cross(float2 (&v)[32], float2* xbuf, cg256::cluster_group& cl, int me) {
    const int t = threadIdx.x;
    publish(v, xbuf, cl);
    const uint32_t a1 = cluster_map(xbuf, me ^ 1), a2 = cluster_map(xbuf, me ^ 2), a3 = cluster_map(xbuf, me ^ 3);
    const float sx = (me & 1) ? -1.0f : 1.0f, sy = (me & 2) ? -1.0f : 1.0f;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const uint32_t off = (uint32_t)(j * T + t) * 16u;
      const float4 q1 = ld_cluster_f4(a1 + off), q2 = ld_cluster_f4(a2 + off), q3 = ld_cluster_f4(a3 + off);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float2 r0 = v[2 * j + h];
        const float2 r1 = h ? make_float2(q1.z, q1.w) : make_float2(q1.x, q1.y);
        const float2 r2 = h ? make_float2(q2.z, q2.w) : make_float2(q2.x, q2.y);
        const float2 r3 = h ? make_float2(q3.z, q3.w) : make_float2(q3.x, q3.y);
        // (R_3 + s_x R_2) + s_y (R_1 + s_x R_0)
        const float2 u = make_float2(fmaf(sx, r2.x, r3.x), fmaf(sx, r2.y, r3.y));
        const float2 w = make_float2(fmaf(sx, r0.x, r1.x), fmaf(sx, r0.y, r1.y));
        v[2 * j + h] = make_float2(fmaf(sy, w.x, u.x), fmaf(sy, w.y, u.y));
      }
    }
    end_exchange(cl);
  }

  static __device__ __forceinline__ void twiddle(float2 (&v)[32], const float2* tw256, int c, bool conj) {
    if (c == 0) return;
    const int t = threadIdx.x;
    const int cy = c >> 1, cx = c & 1;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const float2 w = tw256[G::fky(t, i) * cy + G::fkx(t, i) * cx];
      v[i] = conj ? cmulc(v[i], w) : cmul(v[i], w);
    }
  }

  static __device__ __forceinline__ void forward(float2 (&v)[32], float2* xbuf, const float2* tw1, const float2* tw2,
                                                 const float2* tw256, cg256::cluster_group& cl) {
    const int c = (int)cl.block_rank();
    WinFFT<128>::forward(v, xbuf, tw1, tw2);
    twiddle(v, tw256, c, false);
    cross(v, xbuf, cl, c);
  }

  static __device__ __forceinline__ void inverse(float2 (&v)[32], float2* xbuf, const float2* tw1, const float2* tw2,
                                                 const float2* tw256, cg256::cluster_group& cl) {
    const int c = (int)cl.block_rank();
    cross(v, xbuf, cl, c);
    twiddle(v, tw256, c, true);
    WinFFT<128>::inverse(v, xbuf, tw1, tw2);
  }

  // The middle of one propagation step x -> IFFT(FFT(x) * P) (conj(P) if `adjoint`): the
  // forward cross butterfly, the multiply and the inverse cross butterfly folded into one
  // exchange, between the twiddled forward sub-transform and the conjugate twiddle of the
  // inverse. With T_r the twiddled sub-transform of block r and R_d = T_(me ^ d):
  //   X_q = sum_r s(q, r) T_r = s(q, me) Z_q,  Z_q = sum_d s(q, d) R_d,
  //   U_me = sum_q s(me, q) P_q X_q = sum_q P_q Z_q        (s(me, q) s(q, me) = 1),
  // where P_q is the propagator at frequency (ky + 128 q_y, kx + 128 q_x) of this thread's
  // element; pq(i, q) returns it (zero outside the band).
  template <typename PQ>
  static __device__ __forceinline__ void cross_propagate(float2 (&v)[32], float2* xbuf, cg256::cluster_group& cl,
                                                         int me, bool adjoint, PQ&& pq) {
    const int t = threadIdx.x;
    publish(v, xbuf, cl);
    const uint32_t a1 = cluster_map(xbuf, me ^ 1), a2 = cluster_map(xbuf, me ^ 2), a3 = cluster_map(xbuf, me ^ 3);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const uint32_t off = (uint32_t)(j * T + t) * 16u;
      const float4 q1 = ld_cluster_f4(a1 + off), q2 = ld_cluster_f4(a2 + off), q3 = ld_cluster_f4(a3 + off);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = 2 * j + h;
        const float2 r0 = v[i];
        const float2 r1 = h ? make_float2(q1.z, q1.w) : make_float2(q1.x, q1.y);
        const float2 r2 = h ? make_float2(q2.z, q2.w) : make_float2(q2.x, q2.y);
        const float2 r3 = h ? make_float2(q3.z, q3.w) : make_float2(q3.x, q3.y);
        const float2 e0 = cadd(r0, r1), e1 = csub(r0, r1), e2 = cadd(r2, r3), e3 = csub(r2, r3);
        const float2 z0 = cadd(e0, e2), z1 = cadd(e1, e3), z2 = csub(e0, e2), z3 = csub(e1, e3);
        const float2 p0 = pq(i, 0), p1 = pq(i, 1), p2 = pq(i, 2), p3 = pq(i, 3);
        v[i] = adjoint ? cadd(cadd(cmulc(z0, p0), cmulc(z1, p1)), cadd(cmulc(z2, p2), cmulc(z3, p3)))
                       : cadd(cadd(cmul(z0, p0), cmul(z1, p1)), cadd(cmul(z2, p2), cmul(z3, p3)));
      }
    }
    end_exchange(cl);
  }

  // x -> IFFT(FFT(x) * m) for a real multiplier m (256 x 256, unshifted frequency order)
  static __device__ __forceinline__ void band_limit(float2 (&v)[32], float2* xbuf, const float2* tw1,
                                                    const float2* tw2, const float2* tw256, cg256::cluster_group& cl,
                                                    const float* __restrict__ m) {
    const int c = (int)cl.block_rank();
    const int t = threadIdx.x;
    WinFFT<128>::forward(v, xbuf, tw1, tw2);
    twiddle(v, tw256, c, false);
    cross_propagate(v, xbuf, cl, c, false, [&](int i, int q) {
      return make_float2(m[(G::fky(t, i) + 128 * (q >> 1)) * 256 + G::fkx(t, i) + 128 * (q & 1)], 0.0f);
    });
    twiddle(v, tw256, c, true);
    WinFFT<128>::inverse(v, xbuf, tw1, tw2);
  }

  // x <- IFFT(FFT(x) * P * scale) (conj: conj(P)) for a (256, 256) table P in natural (ky, kx)
  // order, in the same single folded exchange
  static __device__ __forceinline__ void propagate(float2 (&v)[32], float2* xbuf, const float2* tw1,
                                                   const float2* tw2, const float2* tw256, cg256::cluster_group& cl,
                                                   const float2* __restrict__ P, bool conj, float scale) {
    const int c = (int)cl.block_rank();
    const int t = threadIdx.x;
    WinFFT<128>::forward(v, xbuf, tw1, tw2);
    twiddle(v, tw256, c, false);
    cross_propagate(v, xbuf, cl, c, conj, [&](int i, int q) {
      return cscale(P[(G::fky(t, i) + 128 * (q >> 1)) * 256 + G::fkx(t, i) + 128 * (q & 1)], scale);
    });
    twiddle(v, tw256, c, true);
    WinFFT<128>::inverse(v, xbuf, tw1, tw2);
  }
};

}  // namespace pty

// Register-resident 2D FFT of one W x W probe window per thread block (W = 64 or 128).
//
// Every thread owns 32 complex values. A 2D transform is three register rounds separated
// by two exchanges through shared memory:
//
//   round 1  thread (y, n2), n2 < A=W/32 : 32-point DFT along x over x = A*n1 + n2
//   round 2  thread (k1, m2), m2 < Bq    : twiddle w_W^(k1*n2), A-point DFT over n2 (finishes
//            kx = k1 + 32*k2), C-point DFT along y over y = Bq*m1 + m2, twiddle w_W^(j1*m2)
//   round 3  thread (j1, g), g < S3      : Bq-point DFT over m2 (finishes ky = j1 + C*j2),
//            the thread holds kx = g + S3*q
//
// with C = 32/A and Bq = W/C. The forward transform runs rounds 1-2-3 and leaves the
// spectrum in the "frequency layout"; the inverse runs 3-2-1 with conjugate twiddles and
// leaves the window in the "real layout" (round-1 ownership). Element-wise work (object
// slice, propagator, masks, loss) happens directly in those layouts, so a multislice step
// is FFT -> multiply -> IFFT without any extra data movement.
//
// Shared-memory exchanges use XOR swizzles chosen so that every half-warp of 8-byte accesses
// touches 16 distinct bank pairs and every quarter-warp of round 1's 16-byte accesses 8 distinct
// bank quads (no bank conflicts) for both W.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

namespace pty {

// ------------------------------------------------------------------ complex helpers
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }

// compile-time loop
template <int I, int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

// cos / sin of 2*pi*m/32, m in [0, 32)
__host__ __device__ constexpr float kcos32(int m) {
  constexpr float t[32] = {
      1.000000000e+00f, 9.807852507e-01f, 9.238795042e-01f, 8.314695954e-01f,
      7.071067691e-01f, 5.555702448e-01f, 3.826834261e-01f, 1.950903237e-01f,
      0.0f, -1.950903237e-01f, -3.826834261e-01f, -5.555702448e-01f,
      -7.071067691e-01f, -8.314695954e-01f, -9.238795042e-01f, -9.807852507e-01f,
      -1.000000000e+00f, -9.807852507e-01f, -9.238795042e-01f, -8.314695954e-01f,
      -7.071067691e-01f, -5.555702448e-01f, -3.826834261e-01f, -1.950903237e-01f,
      0.0f, 1.950903237e-01f, 3.826834261e-01f, 5.555702448e-01f,
      7.071067691e-01f, 8.314695954e-01f, 9.238795042e-01f, 9.807852507e-01f};
  return t[m];
}
__host__ __device__ constexpr float ksin32(int m) { return kcos32((m + 24) & 31); }

// a * exp(SIGN * 2*pi*i * E / N) with E, N compile-time (N divides 32)
template <int N, int E, int SIGN>
__device__ __forceinline__ float2 tw(float2 a) {
  static_assert(32 % N == 0, "twiddle table covers N | 32");
  constexpr int m = ((E % N) * (32 / N)) & 31;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (m == 16) {
    return make_float2(-a.x, -a.y);
  } else if constexpr (m == 8) {          // exp(SIGN * i*pi/2) = SIGN * i
    return SIGN > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
  } else if constexpr (m == 24) {         // exp(SIGN * i*3pi/2) = -SIGN * i
    return SIGN > 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
  } else if constexpr (m % 4 == 0) {      // odd multiples of pi/4
    constexpr float h = 7.071067691e-01f;
    constexpr float c = kcos32(m) > 0 ? h : -h;
    constexpr float s = (SIGN > 0 ? 1.0f : -1.0f) * (ksin32(m) > 0 ? h : -h);
    // (a.x + i a.y)(c + i s) with |c| = |s| = h
    constexpr float sc = (c > 0) == (s > 0) ? 1.0f : -1.0f;   // s = sc * c
    float u = a.x - sc * a.y;   // a.x - a.y*s/c
    float w = a.y + sc * a.x;   // a.y + a.x*s/c
    return make_float2(u * c, w * c);
  } else {
    constexpr float c = kcos32(m);
    constexpr float s = (SIGN > 0 ? 1.0f : -1.0f) * ksin32(m);
    return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
  }
}

// 4-point DFT butterfly: (t0..t3) -> X_q = sum_r t_r * exp(SIGN*2*pi*i*r*q/4)
template <int SIGN>
__device__ __forceinline__ void bfly4(float2& t0, float2& t1, float2& t2, float2& t3) {
  float2 u0 = cadd(t0, t2), u1 = csub(t0, t2), u2 = cadd(t1, t3), d = csub(t1, t3);
  // u3 = d * (SIGN * i)
  float2 u3 = SIGN > 0 ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
  t0 = cadd(u0, u2);
  t2 = csub(u0, u2);
  t1 = cadd(u1, u3);
  t3 = csub(u1, u3);
}

// In-register DFT of the N values v[OFF + STRIDE*i], i < N, written back in natural order.
// Radix-4 decimation in time, radix-2 for the last factor of 2.
template <int N, int SIGN>
struct DFT {
  template <int LEN, int STRIDE, int OFF>
  static __device__ __forceinline__ void run(float2 (&v)[LEN]) {
    if constexpr (N == 1) {
    } else if constexpr (N == 2) {
      float2 a = v[OFF], b = v[OFF + STRIDE];
      v[OFF] = cadd(a, b);
      v[OFF + STRIDE] = csub(a, b);
    } else if constexpr (N == 4) {
      bfly4<SIGN>(v[OFF], v[OFF + STRIDE], v[OFF + 2 * STRIDE], v[OFF + 3 * STRIDE]);
    } else {
      constexpr int M = N / 4;
      DFT<M, SIGN>::template run<LEN, 4 * STRIDE, OFF>(v);
      DFT<M, SIGN>::template run<LEN, 4 * STRIDE, OFF + STRIDE>(v);
      DFT<M, SIGN>::template run<LEN, 4 * STRIDE, OFF + 2 * STRIDE>(v);
      DFT<M, SIGN>::template run<LEN, 4 * STRIDE, OFF + 3 * STRIDE>(v);
      float2 out[N];
      static_for<0, M>([&](auto KK) {
        constexpr int k = decltype(KK)::value;
        float2 t0 = v[OFF + STRIDE * (4 * k)];
        float2 t1 = tw<N, 1 * k, SIGN>(v[OFF + STRIDE * (4 * k + 1)]);
        float2 t2 = tw<N, 2 * k, SIGN>(v[OFF + STRIDE * (4 * k + 2)]);
        float2 t3 = tw<N, 3 * k, SIGN>(v[OFF + STRIDE * (4 * k + 3)]);
        bfly4<SIGN>(t0, t1, t2, t3);
        out[k] = t0;
        out[k + M] = t1;
        out[k + 2 * M] = t2;
        out[k + 3 * M] = t3;
      });
#pragma unroll
      for (int i = 0; i < N; ++i) v[OFF + STRIDE * i] = out[i];
    }
  }
};

// ------------------------------------------------------------------ window geometry
template <int W>
struct Geo {
  static_assert(W == 64 || W == 128, "window FFT supports W = 64 and 128");
  static constexpr int E = 32;             // complex values per thread
  static constexpr int T = W * W / E;      // threads per window
  static constexpr int A = W / 32;         // x sub-factor owned by round-1 threads
  static constexpr int C = 32 / A;         // y factor done in round 2
  static constexpr int Bq = W / C;         // y factor done in round 3
  static constexpr int Q = 32 / Bq;        // kx values per round-3 thread
  static constexpr int S3 = W / Q;         // kx stride in round 3
  static constexpr int TW1 = A * 32;       // round-1 twiddle table size
  static constexpr int TW2 = W;            // round-2 twiddle table size
  static constexpr int XBUF = W * W;       // exchange buffer (float2)
  static constexpr int MINB = W == 64 ? 4 : 1;   // resident blocks per SM the kernels aim for

  // real layout: element i of thread t is pixel (y, x)
  static __device__ __forceinline__ int ry(int t) { return t / A; }
  static __device__ __forceinline__ int rx(int t, int i) { return A * i + (t % A); }
  // frequency layout: element i of thread t is frequency (ky, kx) (unshifted FFT index)
  static __device__ __forceinline__ int fky(int t, int i) { return (t / S3) + C * (i % Bq); }
  static __device__ __forceinline__ int fkx(int t, int i) { return (t % S3) + S3 * (i / Bq); }
};

// Twiddle tables (built once per launch into shared memory from a global copy):
//   tw1[n2*32 + (k1 ^ n2)] = w_W^(k1*n2),  tw2[m2*C + j1] = w_W^(j1*m2),  w_W = exp(-2 pi i/W)
// The x twiddle w_W^(k1*n2) between the 32-point and the A-point DFT along x is applied in round
// 2, where a thread holds one k1 and every n2: A - 1 distinct factors per thread (A - 1 table
// reads, C * (A - 1) multiplies) instead of 31 reads and multiplies per thread in round 1.
template <int W>
__device__ __forceinline__ void load_twiddles(float2* s_tw1, float2* s_tw2, const float2* g_tw) {
  using G = Geo<W>;
  for (int i = threadIdx.x; i < G::TW1 + G::TW2; i += blockDim.x) {
    float2 w = g_tw[i];
    if (i < G::TW1) s_tw1[i] = w; else s_tw2[i - G::TW1] = w;
  }
}

template <int W>
struct WinFFT {
  using G = Geo<W>;
  static constexpr int A = G::A, C = G::C, Bq = G::Bq, Q = G::Q, S3 = G::S3;

  // the XOR masks are even, so a row's elements 2j and 2j+1 stay adjacent: round 1 moves them
  // as one 16-byte word (round 2 reads single elements), conflict-free both ways
  static __device__ __forceinline__ int x1(int r, int k1) { return r * 32 + (k1 ^ ((r & 7) << 1)); }
  static __device__ __forceinline__ int x2(int s, int kx) { return s * W + (kx ^ ((s & 1) << 3)); }

  // real layout -> frequency layout, unnormalised, exp(-2 pi i ...) kernel
  static __device__ __forceinline__ void forward(float2 (&v)[32], float2* xbuf,
                                                 const float2* tw1, const float2* tw2) {
    forward_round1(v, tw1);
    forward_rest(v, xbuf, tw1, tw2, [] {});
  }

  // The forward transform in two parts, so that a caller can overlap work that must finish
  // before the exchange buffer is overwritten (a cluster barrier, a pending copy) with the
  // register-only first round. forward_round1 touches no shared memory besides the twiddles;
  // forward_rest calls after_first_sync() right after its first barrier, when every thread of
  // the block has finished everything it did before forward_rest.
  static __device__ __forceinline__ void forward_round1(float2 (&v)[32], const float2* tw1) {
    (void)tw1;   // the x twiddle is applied in round 2
    DFT<32, -1>::template run<32, 1, 0>(v);
  }

  template <typename AfterSync>
  static __device__ __forceinline__ void forward_rest(float2 (&v)[32], float2* xbuf, const float2* tw1,
                                                     const float2* tw2, AfterSync&& after_first_sync) {
    const int t = threadIdx.x;
    __syncthreads();
    after_first_sync();
#pragma unroll
    for (int j = 0; j < 16; ++j)
      reinterpret_cast<float4*>(xbuf)[x1(t, 2 * j) >> 1] =
          make_float4(v[2 * j].x, v[2 * j].y, v[2 * j + 1].x, v[2 * j + 1].y);
    __syncthreads();
    // ---- round 2
    {
      const int k1 = t % 32, m2 = t / 32;
#pragma unroll
      for (int m1 = 0; m1 < C; ++m1)
#pragma unroll
        for (int n2 = 0; n2 < A; ++n2) v[m1 * A + n2] = xbuf[x1((Bq * m1 + m2) * A + n2, k1)];
      {   // x twiddle w_W^(k1*n2): this thread's k1 is fixed
        float2 w[A];
#pragma unroll
        for (int n2 = 1; n2 < A; ++n2) w[n2] = tw1[n2 * 32 + (k1 ^ n2)];
#pragma unroll
        for (int m1 = 0; m1 < C; ++m1)
#pragma unroll
          for (int n2 = 1; n2 < A; ++n2) v[m1 * A + n2] = cmul(v[m1 * A + n2], w[n2]);
      }
      static_for<0, C>([&](auto M1) { DFT<A, -1>::template run<32, 1, decltype(M1)::value * A>(v); });
      static_for<0, A>([&](auto K2) { DFT<C, -1>::template run<32, A, decltype(K2)::value>(v); });
      if (m2 != 0) {
#pragma unroll
        for (int j1 = 1; j1 < C; ++j1) {
          float2 w = tw2[m2 * C + j1];
#pragma unroll
          for (int k2 = 0; k2 < A; ++k2) v[j1 * A + k2] = cmul(v[j1 * A + k2], w);
        }
      }
      __syncthreads();
#pragma unroll
      for (int j1 = 0; j1 < C; ++j1)
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2) xbuf[x2(m2 * C + j1, k1 + 32 * k2)] = v[j1 * A + k2];
    }
    __syncthreads();
    // ---- round 3
    {
      const int g = t % S3, j1 = t / S3;
#pragma unroll
      for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int m2 = 0; m2 < Bq; ++m2) v[q * Bq + m2] = xbuf[x2(m2 * C + j1, g + S3 * q)];
      static_for<0, Q>([&](auto QQ) { DFT<Bq, -1>::template run<32, 1, decltype(QQ)::value * Bq>(v); });
    }
  }

  // frequency layout -> real layout, unnormalised, exp(+2 pi i ...) kernel (no 1/W^2)
  static __device__ __forceinline__ void inverse(float2 (&v)[32], float2* xbuf,
                                                 const float2* tw1, const float2* tw2) {
    inverse_head(v, xbuf, tw1, tw2);
    inverse_tail(v, tw1);
  }

  // The register-only end of the inverse transform (round 1): callers that reuse xbuf may
  // run inverse_head (everything up to the last xbuf read), synchronise, refill xbuf
  // asynchronously, and then run inverse_tail while the copy is in flight.
  static __device__ __forceinline__ void inverse_tail(float2 (&v)[32], const float2* tw1) {
    (void)tw1;   // the conjugate x twiddle was applied in round 2 of inverse_head
    DFT<32, +1>::template run<32, 1, 0>(v);
  }

  // inverse() without its register-only tail: after it returns (and a barrier), xbuf is free.
  static __device__ __forceinline__ void inverse_head(float2 (&v)[32], float2* xbuf,
                                                      const float2* tw1, const float2* tw2) {
    const int t = threadIdx.x;
    {
      const int g = t % S3, j1 = t / S3;
      static_for<0, Q>([&](auto QQ) { DFT<Bq, +1>::template run<32, 1, decltype(QQ)::value * Bq>(v); });
      __syncthreads();
#pragma unroll
      for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int m2 = 0; m2 < Bq; ++m2) xbuf[x2(m2 * C + j1, g + S3 * q)] = v[q * Bq + m2];
    }
    __syncthreads();
    {
      const int k1 = t % 32, m2 = t / 32;
#pragma unroll
      for (int j1 = 0; j1 < C; ++j1)
#pragma unroll
        for (int k2 = 0; k2 < A; ++k2) v[j1 * A + k2] = xbuf[x2(m2 * C + j1, k1 + 32 * k2)];
      if (m2 != 0) {
#pragma unroll
        for (int j1 = 1; j1 < C; ++j1) {
          float2 w = tw2[m2 * C + j1];
#pragma unroll
          for (int k2 = 0; k2 < A; ++k2) v[j1 * A + k2] = cmulc(v[j1 * A + k2], w);
        }
      }
      static_for<0, A>([&](auto K2) { DFT<C, +1>::template run<32, A, decltype(K2)::value>(v); });
      static_for<0, C>([&](auto M1) { DFT<A, +1>::template run<32, 1, decltype(M1)::value * A>(v); });
      {   // conjugate x twiddle w_W^(-k1*n2), this thread's k1 fixed
        float2 w[A];
#pragma unroll
        for (int n2 = 1; n2 < A; ++n2) w[n2] = tw1[n2 * 32 + (k1 ^ n2)];
#pragma unroll
        for (int m1 = 0; m1 < C; ++m1)
#pragma unroll
          for (int n2 = 1; n2 < A; ++n2) v[m1 * A + n2] = cmulc(v[m1 * A + n2], w[n2]);
      }
      __syncthreads();
#pragma unroll
      for (int m1 = 0; m1 < C; ++m1)
#pragma unroll
        for (int n2 = 0; n2 < A; ++n2) xbuf[x1((Bq * m1 + m2) * A + n2, k1)] = v[m1 * A + n2];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const float4 q = reinterpret_cast<const float4*>(xbuf)[x1(t, 2 * j) >> 1];
      v[2 * j] = make_float2(q.x, q.y);
      v[2 * j + 1] = make_float2(q.z, q.w);
    }
  }
};

// ------------------------------------------------------------------ native window layout
// Windows that live only inside the library are stored in the order the FFT threads own
// them: element i of thread t at float2 offset 2*((i/2)*T + t) + i%2. A thread's element
// pair (2j, 2j+1) is one 16-byte word and a warp touches 512 contiguous bytes per access.
// Elements i < 2j of every thread form one contiguous prefix (2j*T float2).
template <int W>
__device__ __forceinline__ int nidx(int i, int t) {
  return 2 * ((i >> 1) * Geo<W>::T + t) + (i & 1);
}

template <int W>
__device__ __forceinline__ void ld_native(const float2* base, float2 (&v)[32]) {
  const float4* p = reinterpret_cast<const float4*>(base);
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float4 q = p[j * Geo<W>::T + t];
    v[2 * j] = make_float2(q.x, q.y);
    v[2 * j + 1] = make_float2(q.z, q.w);
  }
}

template <int W>
__device__ __forceinline__ void st_native(float2* base, const float2 (&v)[32]) {
  float4* p = reinterpret_cast<float4*>(base);
  const int t = threadIdx.x;
#pragma unroll
  for (int j = 0; j < 16; ++j) p[j * Geo<W>::T + t] = make_float4(v[2 * j].x, v[2 * j].y, v[2 * j + 1].x, v[2 * j + 1].y);
}

// ------------------------------------------------------------------ bulk async copies
// One-dimensional TMA bulk copies global -> shared completed on an mbarrier, with bounded
// waits: a wait that runs out sets *err and returns instead of spinning forever.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// orders this thread's earlier generic-proxy shared-memory accesses before later
// async-proxy (TMA) accesses
__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// the same for global memory written with ordinary stores and read back by TMA
__device__ __forceinline__ void fence_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

constexpr int kMbarWaitLimit = 1 << 20;   // try_wait rounds before a wait is declared failed

__device__ __forceinline__ void mbar_wait(uint64_t* bar, uint32_t& parity, int* err) {
  for (int it = 0; !mbar_try_wait(bar, parity); ++it) {
    if (it >= kMbarWaitLimit) {
      if (err) *err = 1;
      break;
    }
  }
  parity ^= 1u;
}

// Asynchronous copies global -> shared through the load path (cp.async: any global address,
// device memory or mapped pinned host memory), 16 or 4 bytes per copy with both addresses
// aligned to the size; a thread's copies are complete after its cp_async_wait_all().
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Issue (one thread) an L2 prefetch of `bytes` at `src` (16-byte aligned, a multiple of 16
// bytes) in chunks of at most 64 KiB; nothing waits on it.
__device__ __forceinline__ void prefetch_l2(const void* src, uint32_t bytes) {
  constexpr uint32_t kChunk = 64u * 1024u;
  for (uint32_t o = 0; o < bytes; o += kChunk) {
    const uint32_t n = bytes - o < kChunk ? bytes - o : kChunk;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(static_cast<const char*>(src) + o), "r"(n)
                 : "memory");
  }
}

// Issue (one thread) a copy of `bytes` from global `src` into shared `dst` in chunks of at
// most 64 KiB, all completing on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  mbar_expect_tx(bar, bytes);
  constexpr uint32_t kChunk = 64u * 1024u;
  for (uint32_t o = 0; o < bytes; o += kChunk) {
    const uint32_t n = bytes - o < kChunk ? bytes - o : kChunk;
    bulk_copy_g2s(static_cast<char*>(dst) + o, static_cast<const char*>(src) + o, n, bar);
  }
}

// Issue (one thread) a copy of `bytes` from shared `src` to global `dst` in chunks of at most
// 64 KiB as one bulk group. The writer threads of `src` have run fence_async_shared() and a
// block barrier before this; `src` may be overwritten after bulk_wait_read() in this thread.
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes) {
  constexpr uint32_t kChunk = 64u * 1024u;
  for (uint32_t o = 0; o < bytes; o += kChunk) {
    const uint32_t n = bytes - o < kChunk ? bytes - o : kChunk;
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(static_cast<char*>(dst) + o),
                 "r"(smem_u32(src) + o), "r"(n)
                 : "memory");
  }
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// every bulk store of this thread has finished reading its shared-memory source
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// every bulk store of this thread has completed its writes to global memory
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Entry i of the twiddle tables in global memory (see load_twiddles).
template <int W>
__device__ __forceinline__ float2 twiddle_entry(int i) {
  using G = Geo<W>;
  int e;
  if (i < G::TW1) {
    int n2 = i / 32, k1 = (i % 32) ^ n2;
    e = (k1 * n2) % W;
  } else {
    int j = i - G::TW1, m2 = j / G::C, j1 = j % G::C;
    e = (j1 * m2) % W;
  }
  float s, c;
  sincospif(2.0f * (float)e / (float)W, &s, &c);   // exact argument: e/W is a dyadic rational
  return make_float2(c, -s);
}

// Builder of the twiddle tables in global memory.
template <int W>
__global__ void build_twiddles_kernel(float2* g_tw) {
  using G = Geo<W>;
  for (int i = threadIdx.x + blockIdx.x * blockDim.x; i < G::TW1 + G::TW2; i += blockDim.x * gridDim.x)
    g_tw[i] = twiddle_entry<W>(i);
}

}  // namespace pty

// Device side of pypty's optimizer step around loss_and_direction:
//   * the full-array band limit `fourier_clean` (pypty/utils.py:102-150), applied to the
//     object, its gradient, the search direction and the probe every line-search trial
//     (pypty/iterative.py:497-514, 541-548, 674-681, 741-748, 790-797);
//   * the vector algebra of the L-BFGS update and Wolfe line search of `bfgs_update`
//     (pypty/iterative.py:562-571, 583-731, 811-817, 849-916): two-loop recursion, step
//     normalisation, directional derivatives, history pairs, Barzilai-Borwein gammas;
//   * Gram-Schmidt orthogonalisation of probe modes (pypty/objective.py:1119-1141).
//
// fourier_clean of an (Ny, Nx, K) complex64 array (K = slices x modes, innermost) takes
// three passes over HBM, each a batch of strided 1D FFTs computed in shared memory:
//   pass X  : FFT along x of every (y, k) line           (of a + step * b when b is given)
//   pass Y  : FFT along y of every (x, k) line, times the band-limit mask, inverse FFT along y
//   pass X' : inverse FFT along x, scaled by 1 / (Ny Nx)
// The fftshift before the mask and the ifftshift after it cancel: the mask is tabulated in
// unshifted frequency order.
//
// Inner products accumulate in FP64 over a fixed grid in a fixed order, so every scalar of
// the recursion is deterministic run to run. The recursion's scalars (alpha, beta, rho,
// gamma, step normalisation) are computed on the device by one-warp kernels between the
// vector passes: the host reads back only the two directional derivatives it needs for
// the Wolfe decisions.
#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"

namespace pty {
namespace oc {

// ------------------------------------------------------------------ strided batched FFT
constexpr int TILE = 8192;          // complex elements per tile: N points x KB lines
constexpr int TPB = 512;
constexpr int EPT = TILE / TPB;     // elements held per thread
constexpr int SMEM_F2 = TILE + TILE / 16;
__host__ __device__ constexpr int pad(int a) { return a + (a >> 4); }   // 1 float2 every 16: bank spread

constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }

// radix schedule of an N-point transform: ceil(log2 N / 4) passes of radix <= 16, balanced
template <int N>
struct Sched {
  static constexpr int P2 = ilog2c(N);
  static constexpr int NP = (P2 + 3) / 4;
  static constexpr int lr(int i) { return P2 / NP + (i < P2 % NP ? 1 : 0); }
  static constexpr int ns(int i) {
    int s = 1;
    for (int k = 0; k < i; ++k) s <<= lr(k);
    return s;
  }
};

// line g of a batch starts at element (g / V) * U + g % V and has element stride E
struct Lines {
  long long U, V, E, count;
};

struct PassArgs {
  const float2* a;      // pass X: input (nullptr: read `out` in place)
  const float2* b;      // pass X: optional, the input is a + step * b
  float step;
  float2* out;
  const float2* tw;     // exp(-2 pi i m / N), m < N
  const float* mask;    // pass Y: band limit [ky * nx + kx], unshifted frequency order
  int nx;
  long long k;          // pass Y: the mask column of line g is g / k
  float scale;          // pass X': output scale
  Lines L;
};

// One Stockham radix-R pass (the formulation of Govindaraju et al., SC 2008):
//   for j < N/R:  v_r = in[j + r N/R] * w_{NS R}^{r (j mod NS)},  V = DFT_R(v),
//                 out[(j / NS) NS R + (j mod NS) + q NS] = V_q.
// Every thread owns one line (s = thread mod KB) and EPT / R butterflies of it.
template <int N, int R, int NS, int SIGN, class Src>
__device__ __forceinline__ void gather(float2 (&v)[EPT], const Src& src, const float2* __restrict__ tw) {
  constexpr int KB = TILE / N;
  static_for<0, EPT / R>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const int j = (threadIdx.x + TPB * i) / KB;
#pragma unroll
    for (int r = 0; r < R; ++r) v[i * R + r] = src(j + r * (N / R));
    if constexpr (NS > 1) {
      const int jm = j % NS;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const float2 w = __ldg(tw + r * jm * (N / (NS * R)));
        v[i * R + r] = SIGN < 0 ? cmul(v[i * R + r], w) : cmulc(v[i * R + r], w);
      }
    }
    DFT<R, SIGN>::template run<EPT, 1, i * R>(v);
  });
}

template <int N, int R, int NS, class Dst>
__device__ __forceinline__ void scatter(const float2 (&v)[EPT], const Dst& dst) {
  constexpr int KB = TILE / N;
  static_for<0, EPT / R>([&](auto I) {
    constexpr int i = decltype(I)::value;
    const int j = (threadIdx.x + TPB * i) / KB;
    const int d = (j / NS) * NS * R + j % NS;
#pragma unroll
    for (int q = 0; q < R; ++q) dst(d + q * NS, v[i * R + q]);
  });
}

// Full N-point transform of the tile: the first pass reads `src`, the last writes `dst`,
// the passes between go through shared memory (a barrier after every shared read and write).
template <int N, int SIGN, bool SRC_SMEM, bool DST_SMEM, class Src, class Dst>
__device__ __forceinline__ void transform(float2 (&v)[EPT], float2* sm, const Src& src, const Dst& dst,
                                          const float2* __restrict__ tw) {
  constexpr int KB = TILE / N;
  using S = Sched<N>;
  const int s = threadIdx.x % KB;
  auto sm_src = [&](int n) { return sm[pad(n * KB + s)]; };
  auto sm_dst = [&](int n, float2 x) { sm[pad(n * KB + s)] = x; };
  static_for<0, S::NP>([&](auto P) {
    constexpr int p = decltype(P)::value;
    constexpr int R = 1 << S::lr(p);
    constexpr int NS = S::ns(p);
    if constexpr (p == 0) {
      gather<N, R, NS, SIGN>(v, src, tw);
      if constexpr (SRC_SMEM) __syncthreads();
    } else {
      gather<N, R, NS, SIGN>(v, sm_src, tw);
      __syncthreads();
    }
    if constexpr (p == S::NP - 1) {
      scatter<N, R, NS>(v, dst);
      if constexpr (DST_SMEM) __syncthreads();
    } else {
      scatter<N, R, NS>(v, sm_dst);
      __syncthreads();
    }
  });
}

// MODE 0: pass X (forward, optional a + step b); 1: pass Y (forward, mask, inverse);
// 2: pass X' (inverse, scaled).
template <int N, int MODE>
__global__ void __launch_bounds__(TPB, MODE == 1 ? 1 : 2) clean_pass_kernel(PassArgs A) {
  extern __shared__ float2 sm[];
  constexpr int KB = TILE / N;
  const int s = threadIdx.x % KB;
  const long long g = (long long)blockIdx.x * KB + s;
  const bool valid = g < A.L.count;
  const long long base = valid ? (g / A.L.V) * A.L.U + g % A.L.V : 0;
  const long long E = A.L.E;
  float2 v[EPT];
  auto gload = [&](const float2* p, int n) {
    return valid ? p[base + (long long)n * E] : make_float2(0.f, 0.f);
  };
  auto gstore = [&](int n, float2 x) {
    if (valid) A.out[base + (long long)n * E] = x;
  };
  if constexpr (MODE == 0) {
    const float2* a = A.a ? A.a : A.out;
    if (A.b) {
      const float st = A.step;
      auto src = [&](int n) {
        const float2 x = gload(a, n), d = gload(A.b, n);
        return make_float2(__fadd_rn(x.x, __fmul_rn(st, d.x)), __fadd_rn(x.y, __fmul_rn(st, d.y)));
      };
      transform<N, -1, false, false>(v, sm, src, gstore, A.tw);
    } else {
      auto src = [&](int n) { return gload(a, n); };
      transform<N, -1, false, false>(v, sm, src, gstore, A.tw);
    }
  } else if constexpr (MODE == 1) {
    auto src = [&](int n) { return gload(A.out, n); };
    auto to_sm = [&](int n, float2 x) { sm[pad(n * KB + s)] = x; };
    transform<N, -1, false, true>(v, sm, src, to_sm, A.tw);
    const float* mcol = A.mask + (valid ? g / A.k : 0);
    const int nx = A.nx;
    auto masked = [&](int n) { return cscale(sm[pad(n * KB + s)], __ldg(mcol + (long long)n * nx)); };
    transform<N, 1, true, false>(v, sm, masked, gstore, A.tw);
  } else {
    const float sc = A.scale;
    auto src = [&](int n) { return gload(A.out, n); };
    auto dst = [&](int n, float2 x) { gstore(n, cscale(x, sc)); };
    transform<N, 1, false, false>(v, sm, src, dst, A.tw);
  }
}

__global__ void twiddle_kernel(float2* tw, int n) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  double sn, cs;
  sincospi(2.0 * (double)m / (double)n, &sn, &cs);   // exact dyadic argument
  tw[m] = make_float2((float)cs, (float)-sn);
}

// Band limit of utils.fourier_clean (pypty/utils.py:128-138), in unshifted order:
//   r = fx^2 + fy^2 (float64), max_r = 0.5 cutoff, mask = r <= max_r^2 (float32 cutoff
//   arithmetic promoted to float64 for the comparison), and with a roll-off the cosine taper
//   0.5 (1 + cos(3.141592654 (r - r0) / (max_r^2 - r0))) for r > r0 = (0.5 (cutoff - rolloff))^2.
// A caller-given mask (fftshifted order, as utils.fourier_clean(mask=...) receives it) is
// copied into unshifted order instead.
__global__ void mask_kernel(float* mask, int ny, int nx, double inv_ny, double inv_nx, float cutoff, float rolloff,
                            const float* given) {
  const int kx = blockIdx.x * blockDim.x + threadIdx.x;
  const int ky = blockIdx.y;
  if (kx >= nx) return;
  const long long idx = (long long)ky * nx + kx;
  if (given) {
    mask[idx] = given[(long long)((ky + ny / 2) % ny) * nx + (kx + nx / 2) % nx];
    return;
  }
  // numpy.fft.fftfreq(n)[k] = k_signed * (1.0 / n)
  const double fy = (double)(ky < (ny + 1) / 2 ? ky : ky - ny) * inv_ny;
  const double fx = (double)(kx < (nx + 1) / 2 ? kx : kx - nx) * inv_nx;
  const double r = fx * fx + fy * fy;
  const float max_r = __fmul_rn(0.5f, cutoff);
  const float thr = __fmul_rn(max_r, max_r);
  float m = r <= (double)thr ? 1.0f : 0.0f;
  if (rolloff != 0.0f) {
    const float h = __fmul_rn(0.5f, __fsub_rn(cutoff, rolloff));
    const float r0 = __fmul_rn(h, h);
    if (r > (double)r0) {
      const double t = 0.5 * (1.0 + cos(3.141592654 * (r - (double)r0) / (double)__fsub_rn(thr, r0)));
      m = (float)((double)m * t);
    }
  }
  mask[idx] = m;
}

template <int N, int MODE>
cudaError_t launch_pass(const PassArgs& A, cudaStream_t st) {
  constexpr int KB = TILE / N;
  const long long tiles = (A.L.count + KB - 1) / KB;
  if (tiles <= 0) return cudaSuccess;
  if (tiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  auto k = clean_pass_kernel<N, MODE>;
  const int smem = SMEM_F2 * (int)sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k<<<(unsigned)tiles, TPB, smem, st>>>(A);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t dispatch_pass(int n, const PassArgs& A, cudaStream_t st) {
  switch (n) {
    case 64: return launch_pass<64, MODE>(A, st);
    case 128: return launch_pass<128, MODE>(A, st);
    case 256: return launch_pass<256, MODE>(A, st);
    case 512: return launch_pass<512, MODE>(A, st);
    case 1024: return launch_pass<1024, MODE>(A, st);
    case 2048: return launch_pass<2048, MODE>(A, st);
    case 4096: return launch_pass<4096, MODE>(A, st);
    case 8192: return launch_pass<8192, MODE>(A, st);
    default: return cudaErrorInvalidValue;
  }
}

bool pow2_in_range(long long n) { return n >= 64 && n <= 8192 && (n & (n - 1)) == 0; }

struct CleanWs {
  size_t o_twx, o_twy, o_mask, total;
};
CleanWs clean_ws(int ny, int nx) {
  CleanWs w;
  w.o_twx = 0;
  w.o_twy = align_up(w.o_twx + (size_t)nx * sizeof(float2));
  w.o_mask = align_up(w.o_twy + (size_t)ny * sizeof(float2));
  w.total = align_up(w.o_mask + (size_t)ny * nx * sizeof(float));
  return w;
}

// ------------------------------------------------------------------ vector algebra
constexpr int VB = 608;    // fixed reduction grid: 4 blocks per SM of a 152-SM GB300
constexpr int VT = 256;
constexpr int HMAX = 64;   // history slots
constexpr int NSEG = PTY_VSPACE_MAX_SEG;   // object, probe, positions, tilts, static background,
                                           // aberrations, beam current

struct OptState {
  double w[NSEG];              // inner-product weight of each segment
  double coef[2 * NSEG];       // a-coefficients, b-coefficients of the next vector pass
  double dot[NSEG];            // last reduced inner products, per segment (unweighted)
  double dot2[NSEG];           // second reduced product (accept: y.s)
  double gamma[NSEG];          // Barzilai-Borwein scaling per segment
  double dval, dval_new;       // directional derivatives at the start point and at the trial
  double rho[HMAX], alpha[HMAX];
  double part[2][NSEG][VB];    // per-block partial sums of the last reduction
};

struct VSeg {
  float* out;
  const float* a;
  const float* b;
  const float* dx;
  const float* dy;
  long long n;
};

struct VecArgs {
  VSeg seg[NSEG];
  int nseg;
  const double* coef;   // device coefficients [a_0 .. a_NSEG-1, b_0 .. b_NSEG-1], or nullptr: use hc
  double hc[2 * NSEG];
  int dot_out;          // 1: the inner product's left operand is the value just written
  double* part;         // [NSEG][VB] partial sums (a dot is taken where seg.dy != nullptr)
};

__device__ __forceinline__ float lin(float ca, float a, float cb, const float* b, long long i, bool hb) {
  const float t = __fmul_rn(ca, a);
  return hb ? __fadd_rn(t, __fmul_rn(cb, b[i])) : t;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < VT / 32; ++i) t += red[i];
  return t;
}

__device__ __forceinline__ bool al16(const void* p) { return p == nullptr || ((uintptr_t)p & 15) == 0; }

// out = ca * a + cb * b per segment (float32 roundings as the reference's NumPy
// expressions), and the per-block partial sums of <x, dy> with x = out or dx.
__global__ void __launch_bounds__(VT) vec_kernel(VecArgs A) {
  __shared__ double red[VT / 32];
  for (int sg = 0; sg < A.nseg; ++sg) {
    const VSeg S = A.seg[sg];
    const float ca = (float)(A.coef ? A.coef[sg] : A.hc[sg]);
    const float cb = (float)(A.coef ? A.coef[NSEG + sg] : A.hc[NSEG + sg]);
    const bool hb = S.b != nullptr, dot = S.dy != nullptr, wr = S.out != nullptr;
    double acc = 0.0;
    const bool v4 = (S.n % 4 == 0) && al16(S.out) && al16(S.a) && al16(S.b) && al16(S.dx) && al16(S.dy);
    const long long stride = (long long)VB * VT;
    if (v4) {
      const long long n4 = S.n / 4;
      for (long long i = (long long)blockIdx.x * VT + threadIdx.x; i < n4; i += stride) {
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        if (wr) {
          const float4 a = reinterpret_cast<const float4*>(S.a)[i];
          const float4 b = hb ? reinterpret_cast<const float4*>(S.b)[i] : make_float4(0.f, 0.f, 0.f, 0.f);
          o.x = hb ? __fadd_rn(__fmul_rn(ca, a.x), __fmul_rn(cb, b.x)) : __fmul_rn(ca, a.x);
          o.y = hb ? __fadd_rn(__fmul_rn(ca, a.y), __fmul_rn(cb, b.y)) : __fmul_rn(ca, a.y);
          o.z = hb ? __fadd_rn(__fmul_rn(ca, a.z), __fmul_rn(cb, b.z)) : __fmul_rn(ca, a.z);
          o.w = hb ? __fadd_rn(__fmul_rn(ca, a.w), __fmul_rn(cb, b.w)) : __fmul_rn(ca, a.w);
          reinterpret_cast<float4*>(S.out)[i] = o;
        }
        if (dot) {
          const float4 x = A.dot_out ? o : reinterpret_cast<const float4*>(S.dx)[i];
          const float4 y = reinterpret_cast<const float4*>(S.dy)[i];
          float p = x.x * y.x;
          p = fmaf(x.y, y.y, p);
          p = fmaf(x.z, y.z, p);
          p = fmaf(x.w, y.w, p);
          acc += (double)p;
        }
      }
    } else {
      for (long long i = (long long)blockIdx.x * VT + threadIdx.x; i < S.n; i += stride) {
        float o = 0.f;
        if (wr) {
          o = lin(ca, S.a[i], cb, S.b, i, hb);
          S.out[i] = o;
        }
        if (dot) acc += (double)((A.dot_out ? o : S.dx[i]) * S.dy[i]);
      }
    }
    if (dot) {
      const double t = block_sum(acc, red);
      if (threadIdx.x == 0) A.part[sg * VB + blockIdx.x] = t;
    }
  }
}

// History pair of an accepted step: s = step * q, y = new_g - g, and the partial sums of
// <y, y> (buffer 0) and <y, s> (buffer 1) per segment (pypty/iterative.py:849-856, 869-916).
struct AcceptArgs {
  const float* q[NSEG];
  const float* g[NSEG];
  const float* ng[NSEG];
  float* s[NSEG];
  float* y[NSEG];
  long long n[NSEG];
  int nseg;
  float step;
  double* part;   // [2][NSEG][VB]
};

__global__ void __launch_bounds__(VT) accept_kernel(AcceptArgs A) {
  __shared__ double red[VT / 32];
  for (int sg = 0; sg < A.nseg; ++sg) {
    double ayy = 0.0, ays = 0.0;
    const long long stride = (long long)VB * VT;
    for (long long i = (long long)blockIdx.x * VT + threadIdx.x; i < A.n[sg]; i += stride) {
      const float sv = __fmul_rn(A.step, A.q[sg][i]);
      const float yv = __fsub_rn(A.ng[sg][i], A.g[sg][i]);
      A.s[sg][i] = sv;
      A.y[sg][i] = yv;
      ayy += (double)(yv * yv);
      ays += (double)(yv * sv);
    }
    const double tyy = block_sum(ayy, red);
    if (threadIdx.x == 0) A.part[(0 * NSEG + sg) * VB + blockIdx.x] = tyy;
    const double tys = block_sum(ays, red);
    if (threadIdx.x == 0) A.part[(1 * NSEG + sg) * VB + blockIdx.x] = tys;
  }
}

enum ScalarOp {
  OP_DOT = 0,        // reduce only
  OP_FIRST = 1,      // empty-history direction scaling (iterative.py:562-571)
  OP_STEEPEST = 2,   // steepest-descent fallback (iterative.py:691-724)
  OP_ALPHA = 3,      // alpha_i = rho_i <s_i, q>; next pass q -= alpha_i y_i (iterative.py:583-618)
  OP_GAMMA = 4,      // q *= gamma where gamma != 0 and not NaN (iterative.py:620-640)
  OP_BETA = 5,       // beta = alpha_i - rho_i <y_i, r>; next pass r += beta s_i (iterative.py:641-672)
  OP_DVAL = 6,       // d_value (iterative.py:684-690)
  OP_DVAL_NEW = 7,   // new_d_value (iterative.py:811-817)
  OP_ACCEPT = 8,     // gamma per segment and rho of the new pair (iterative.py:869-916)
};

// One warp: reduce the partial sums in a fixed order (lane 0's result is used), then the
// scalar step of the recursion on lane 0.
__global__ void scalar_kernel(OptState* S, int op, int nseg, int obj_seg, int slot, int final_beta) {
  const int lane = threadIdx.x;
  const int nbuf = op == OP_ACCEPT ? 2 : 1;
  double d[2][NSEG] = {};
  if (op != OP_GAMMA && op != OP_STEEPEST) {
    for (int b = 0; b < nbuf; ++b)
      for (int sg = 0; sg < nseg; ++sg) {
        double a = 0.0;
        for (int i = lane; i < VB; i += 32) a += S->part[b][sg][i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        d[b][sg] = a;
      }
  }
  if (lane != 0) return;
  double wsum = 0.0;
  const bool reduced = op != OP_GAMMA && op != OP_STEEPEST;
  for (int sg = 0; sg < nseg; ++sg) {
    if (reduced) S->dot[sg] = d[0][sg];
    wsum += S->w[sg] * d[0][sg];
  }
  switch (op) {
    case OP_FIRST: {
      double dvo = obj_seg >= 0 ? S->w[obj_seg] * d[0][obj_seg] : 0.0;
      if (dvo == 0.0) dvo = 1.0;
      for (int sg = 0; sg < nseg; ++sg) {
        S->coef[sg] = sg == obj_seg ? -1.0 : -dvo / (S->w[sg] * d[0][sg]);
        S->coef[NSEG + sg] = 0.0;
      }
      break;
    }
    case OP_STEEPEST:
      for (int sg = 0; sg < nseg; ++sg) {
        const double gm = S->gamma[sg];
        S->coef[sg] = (gm > 0.0 && gm == gm) ? -gm : -1.0;
        S->coef[NSEG + sg] = 0.0;
      }
      break;
    case OP_ALPHA: {
      const double a = S->rho[slot] * wsum;
      S->alpha[slot] = a;
      for (int sg = 0; sg < nseg; ++sg) {
        S->coef[sg] = 1.0;
        S->coef[NSEG + sg] = -a;
      }
      break;
    }
    case OP_GAMMA:
      for (int sg = 0; sg < nseg; ++sg) {
        const double gm = S->gamma[sg];
        S->coef[sg] = (gm != 0.0 && gm == gm) ? gm : 1.0;
        S->coef[NSEG + sg] = 0.0;
      }
      break;
    case OP_BETA: {
      const double beta = S->alpha[slot] - S->rho[slot] * wsum;
      for (int sg = 0; sg < nseg; ++sg) {
        S->coef[sg] = final_beta ? -1.0 : 1.0;
        S->coef[NSEG + sg] = final_beta ? -beta : beta;
      }
      break;
    }
    case OP_DVAL: S->dval = wsum; break;
    case OP_DVAL_NEW: S->dval_new = wsum; break;
    case OP_ACCEPT: {
      double tot = 0.0;
      for (int sg = 0; sg < nseg; ++sg) {
        const double ys = S->w[sg] * d[1][sg];
        S->dot2[sg] = d[1][sg];
        S->gamma[sg] = ys / d[0][sg];
        tot += ys;
      }
      S->rho[slot] = 1.0 / tot;
      break;
    }
    default: break;
  }
}

struct SegWeights {
  double w[NSEG];
};

__global__ void reset_kernel(OptState* S, SegWeights W) {
  if (threadIdx.x != 0) return;
  for (int i = 0; i < NSEG; ++i) {
    S->w[i] = W.w[i];
    S->gamma[i] = 1.0;
    S->dot[i] = S->dot2[i] = 0.0;
  }
  for (int i = 0; i < 2 * NSEG; ++i) S->coef[i] = 0.0;
  S->dval = S->dval_new = 0.0;
  for (int i = 0; i < HMAX; ++i) S->rho[i] = S->alpha[i] = 0.0;
}

// Gram-Schmidt over probe modes (pypty/objective.py:1133-1141): for each mode i and each
// earlier mode j, p_i -= p_j <p_j, p_i> / (1e-10 + |p_j|^2). One block; FP64 sums.
__global__ void __launch_bounds__(1024) orthogonalize_kernel(float2* p, long long npix, int mp) {
  __shared__ double red[2][32];
  __shared__ float2 coef;
  for (int i = 1; i < mp; ++i) {
    for (int j = 0; j < i; ++j) {
      double dr = 0.0, di = 0.0, nn = 0.0;
      for (long long x = threadIdx.x; x < npix; x += blockDim.x) {
        const float2 a = p[x * mp + j], b = p[x * mp + i];
        dr += (double)a.x * b.x + (double)a.y * b.y;   // conj(a) b
        di += (double)a.x * b.y - (double)a.y * b.x;
        nn += (double)a.x * a.x + (double)a.y * a.y;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dr += __shfl_down_sync(0xffffffffu, dr, o);
        di += __shfl_down_sync(0xffffffffu, di, o);
        nn += __shfl_down_sync(0xffffffffu, nn, o);
      }
      const int w = threadIdx.x / 32, l = threadIdx.x % 32;
      if (l == 0) {
        red[0][w] = dr;
        red[1][w] = di;
      }
      __shared__ double rn[32];
      if (l == 0) rn[w] = nn;
      __syncthreads();
      if (threadIdx.x == 0) {
        double sr = 0, si = 0, sn = 0;
        for (int k = 0; k < (int)(blockDim.x / 32); ++k) {
          sr += red[0][k];
          si += red[1][k];
          sn += rn[k];
        }
        const double den = 1e-10 + sn;
        coef = make_float2((float)(sr / den), (float)(si / den));
      }
      __syncthreads();
      const float2 c = coef;
      for (long long x = threadIdx.x; x < npix; x += blockDim.x) {
        const float2 a = p[x * mp + j];
        float2 b = p[x * mp + i];
        const float2 t = cmul(a, c);
        b.x = __fsub_rn(b.x, t.x);
        b.y = __fsub_rn(b.y, t.y);
        p[x * mp + i] = b;
      }
      __syncthreads();
    }
  }
}

// ------------------------------------------------------------------ host helpers
int check_vspace(const pty_vspace_t* vs) {
  if (!vs || vs->n_seg < 1 || vs->n_seg > NSEG) return PTY_ERR_INVALID;
  if (vs->obj_seg < -1 || vs->obj_seg >= vs->n_seg) return PTY_ERR_INVALID;
  for (int i = 0; i < vs->n_seg; ++i)
    if (vs->n[i] <= 0) return PTY_ERR_INVALID;
  return PTY_OK;
}

int run_vec(const pty_vspace_t* vs, float* const* out, float* const* a, float* const* b, float* const* dx,
            float* const* dy, int dot_out, const double* coef, const double* hc, OptState* S, cudaStream_t st) {
  VecArgs A{};
  A.nseg = vs->n_seg;
  for (int i = 0; i < vs->n_seg; ++i) {
    A.seg[i].out = out ? out[i] : nullptr;
    A.seg[i].a = a ? a[i] : nullptr;
    A.seg[i].b = b ? b[i] : nullptr;
    A.seg[i].dx = dx ? dx[i] : nullptr;
    A.seg[i].dy = dy ? dy[i] : nullptr;
    A.seg[i].n = vs->n[i];
    if (A.seg[i].out && !A.seg[i].a) return PTY_ERR_INVALID;
    if (A.seg[i].dy && !dot_out && !A.seg[i].dx) return PTY_ERR_INVALID;
  }
  A.coef = coef;
  for (int i = 0; i < 2 * NSEG; ++i) A.hc[i] = hc ? hc[i] : 0.0;
  A.dot_out = dot_out;
  A.part = &S->part[0][0][0];
  prof_mark(st, KID_VEC);
  vec_kernel<<<VB, VT, 0, st>>>(A);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

int run_scalar(OptState* S, int op, const pty_vspace_t* vs, int slot, int final_beta, cudaStream_t st) {
  prof_mark(st, KID_SCALAR);
  scalar_kernel<<<1, 32, 0, st>>>(S, op, vs->n_seg, vs->obj_seg, slot, final_beta);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

}  // namespace oc
}  // namespace pty

using namespace pty;
using namespace pty::oc;

extern "C" {

int pty_fourier_clean_workspace_bytes(int32_t ny, int32_t nx, size_t* bytes) {
  if (!bytes) return PTY_ERR_INVALID;
  if (ny <= 0 || nx <= 0) return PTY_ERR_INVALID;
  if (!pow2_in_range(ny) || !pow2_in_range(nx)) return PTY_ERR_UNSUPPORTED;
  *bytes = clean_ws(ny, nx).total;
  return PTY_OK;
}

int pty_fourier_clean_prepare(int32_t ny, int32_t nx, float cutoff, float rolloff, const float* mask_shifted,
                              void* workspace, size_t workspace_bytes, void* stream) {
  if (!workspace || ny <= 0 || nx <= 0) return PTY_ERR_INVALID;
  if (!pow2_in_range(ny) || !pow2_in_range(nx)) return PTY_ERR_UNSUPPORTED;
  const CleanWs w = clean_ws(ny, nx);
  if (workspace_bytes < w.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_CLEAN_TABLES);
  twiddle_kernel<<<(nx + 255) / 256, 256, 0, st>>>(at<float2>(workspace, w.o_twx), nx);
  prof_mark(st, KID_CLEAN_TABLES);
  twiddle_kernel<<<(ny + 255) / 256, 256, 0, st>>>(at<float2>(workspace, w.o_twy), ny);
  prof_mark(st, KID_CLEAN_TABLES);
  mask_kernel<<<dim3((nx + 255) / 256, ny), 256, 0, st>>>(at<float>(workspace, w.o_mask), ny, nx, 1.0 / (double)ny,
                                                          1.0 / (double)nx, cutoff, rolloff, mask_shifted);
  prof_mark(st, -1);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

int pty_fourier_clean_apply(const void* x, const void* dx, double step, void* out, int32_t ny, int32_t nx, int64_t k,
                            const void* workspace, size_t workspace_bytes, void* stream) {
  if (!out || !workspace || ny <= 0 || nx <= 0 || k <= 0) return PTY_ERR_INVALID;
  if (!pow2_in_range(ny) || !pow2_in_range(nx)) return PTY_ERR_UNSUPPORTED;
  const CleanWs w = clean_ws(ny, nx);
  if (workspace_bytes < w.total) return PTY_ERR_WORKSPACE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void* ws = const_cast<void*>(workspace);
  const float2* twx = at<float2>(ws, w.o_twx);
  const float2* twy = at<float2>(ws, w.o_twy);
  const float* mask = at<float>(ws, w.o_mask);
  const long long npix = (long long)ny * nx;
  PassArgs A{};
  A.out = static_cast<float2*>(out);
  // pass X: lines (y, k), element stride K
  A.a = static_cast<const float2*>(x ? x : out);
  A.b = static_cast<const float2*>(dx);
  A.step = (float)step;
  A.tw = twx;
  A.L = Lines{(long long)nx * k, k, k, (long long)ny * k};
  prof_mark(st, KID_CLEAN_X);
  if (dispatch_pass<0>(nx, A, st) != cudaSuccess) return PTY_ERR_CUDA;
  // pass Y: lines (x, k) = the contiguous index x * K + k, element stride Nx K
  A.a = nullptr;
  A.b = nullptr;
  A.tw = twy;
  A.mask = mask;
  A.nx = nx;
  A.k = k;
  A.L = Lines{0, (long long)nx * k, (long long)nx * k, (long long)nx * k};
  prof_mark(st, KID_CLEAN_Y);
  if (dispatch_pass<1>(ny, A, st) != cudaSuccess) return PTY_ERR_CUDA;
  // pass X': inverse along x, 1 / (Ny Nx) (a power of two: exact)
  A.tw = twx;
  A.mask = nullptr;
  A.scale = (float)(1.0 / (double)npix);
  A.L = Lines{(long long)nx * k, k, k, (long long)ny * k};
  prof_mark(st, KID_CLEAN_XI);
  if (dispatch_pass<2>(nx, A, st) != cudaSuccess) return PTY_ERR_CUDA;
  prof_mark(st, -1);
  return PTY_OK;
}

int pty_fourier_clean(const void* x, const void* dx, double step, void* out, int32_t ny, int32_t nx, int64_t k,
                      float cutoff, float rolloff, const float* mask_shifted, void* workspace,
                      size_t workspace_bytes, void* stream) {
  if (!out || k <= 0) return PTY_ERR_INVALID;
  int rc = pty_fourier_clean_prepare(ny, nx, cutoff, rolloff, mask_shifted, workspace, workspace_bytes, stream);
  if (rc) return rc;
  return pty_fourier_clean_apply(x, dx, step, out, ny, nx, k, workspace, workspace_bytes, stream);
}

int pty_lbfgs_state_bytes(size_t* bytes) {
  if (!bytes) return PTY_ERR_INVALID;
  *bytes = align_up(sizeof(OptState));
  return PTY_OK;
}

int pty_lbfgs_reset(const pty_vspace_t* vs, void* state, void* stream) {
  int rc = check_vspace(vs);
  if (rc) return rc;
  if (!state) return PTY_ERR_INVALID;
  SegWeights sw{};
  for (int i = 0; i < vs->n_seg; ++i) sw.w[i] = vs->weight[i];
  reset_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<OptState*>(state), sw);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

int pty_lbfgs_first_direction(const pty_vspace_t* vs, float* const* grad, float* const* dir, void* state,
                              void* stream) {
  int rc = check_vspace(vs);
  if (rc) return rc;
  if (!grad || !dir || !state) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  OptState* S = static_cast<OptState*>(state);
  // |g|^2 per segment, then q = c g and d_value = <q, g>
  if ((rc = run_vec(vs, nullptr, nullptr, nullptr, grad, grad, 0, nullptr, nullptr, S, st))) return rc;
  if ((rc = run_scalar(S, OP_FIRST, vs, 0, 0, st))) return rc;
  if ((rc = run_vec(vs, dir, grad, nullptr, nullptr, grad, 1, S->coef, nullptr, S, st))) return rc;
  rc = run_scalar(S, OP_DVAL, vs, 0, 0, st);
  prof_mark(st, -1);
  return rc;
}

int pty_lbfgs_steepest(const pty_vspace_t* vs, float* const* grad, float* const* dir, void* state, void* stream) {
  int rc = check_vspace(vs);
  if (rc) return rc;
  if (!grad || !dir || !state) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  OptState* S = static_cast<OptState*>(state);
  if ((rc = run_scalar(S, OP_STEEPEST, vs, 0, 0, st))) return rc;
  if ((rc = run_vec(vs, dir, grad, nullptr, nullptr, grad, 1, S->coef, nullptr, S, st))) return rc;
  rc = run_scalar(S, OP_DVAL, vs, 0, 0, st);
  prof_mark(st, -1);
  return rc;
}

int pty_lbfgs_two_loop(const pty_vspace_t* vs, float* const* grad, float* const* dir, int32_t m,
                       float* const* s_hist, float* const* y_hist, const int32_t* slots, void* state, void* stream) {
  int rc = check_vspace(vs);
  if (rc) return rc;
  if (!grad || !dir || !state || m < 1 || !s_hist || !y_hist || !slots) return PTY_ERR_INVALID;
  for (int i = 0; i < m; ++i)
    if (slots[i] < 0 || slots[i] >= HMAX) return PTY_ERR_UNSUPPORTED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  OptState* S = static_cast<OptState*>(state);
  const int ns = vs->n_seg;
  auto Sv = [&](int i) { return s_hist + (size_t)i * ns; };
  auto Yv = [&](int i) { return y_hist + (size_t)i * ns; };
  double copy[2 * NSEG] = {};   // a = 1, b = 0: q = g
  for (int i = 0; i < NSEG; ++i) copy[i] = 1.0;
  // q = g; alpha_{m-1}
  if ((rc = run_vec(vs, dir, grad, nullptr, nullptr, Sv(m - 1), 1, nullptr, copy, S, st))) return rc;
  if ((rc = run_scalar(S, OP_ALPHA, vs, slots[m - 1], 0, st))) return rc;
  for (int i = m - 1; i >= 1; --i) {   // q -= alpha_i y_i; alpha_{i-1}
    if ((rc = run_vec(vs, dir, dir, Yv(i), nullptr, Sv(i - 1), 1, S->coef, nullptr, S, st))) return rc;
    if ((rc = run_scalar(S, OP_ALPHA, vs, slots[i - 1], 0, st))) return rc;
  }
  if ((rc = run_vec(vs, dir, dir, Yv(0), nullptr, nullptr, 0, S->coef, nullptr, S, st))) return rc;
  // gamma scaling, then the second loop; the last pass negates
  if ((rc = run_scalar(S, OP_GAMMA, vs, 0, 0, st))) return rc;
  if ((rc = run_vec(vs, dir, dir, nullptr, nullptr, Yv(0), 1, S->coef, nullptr, S, st))) return rc;
  if ((rc = run_scalar(S, OP_BETA, vs, slots[0], m == 1, st))) return rc;
  for (int i = 0; i + 1 < m; ++i) {
    if ((rc = run_vec(vs, dir, dir, Sv(i), nullptr, Yv(i + 1), 1, S->coef, nullptr, S, st))) return rc;
    if ((rc = run_scalar(S, OP_BETA, vs, slots[i + 1], i + 2 == m, st))) return rc;
  }
  rc = run_vec(vs, dir, dir, Sv(m - 1), nullptr, nullptr, 0, S->coef, nullptr, S, st);
  prof_mark(st, -1);
  return rc;
}

int pty_lbfgs_dot(const pty_vspace_t* vs, float* const* x, float* const* y, int32_t target, void* state,
                  void* stream) {
  int rc = check_vspace(vs);
  if (rc) return rc;
  if (!x || !y || !state || target < 0 || target > 1) return PTY_ERR_INVALID;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  OptState* S = static_cast<OptState*>(state);
  if ((rc = run_vec(vs, nullptr, nullptr, nullptr, x, y, 0, nullptr, nullptr, S, st))) return rc;
  rc = run_scalar(S, target == 0 ? OP_DVAL : OP_DVAL_NEW, vs, 0, 0, st);
  prof_mark(st, -1);
  return rc;
}

int pty_lbfgs_axpy(const pty_vspace_t* vs, float* const* out, float* const* a, float* const* b, double step,
                   void* stream) {
  int rc = check_vspace(vs);
  if (rc) return rc;
  if (!out || !a || !b) return PTY_ERR_INVALID;
  // out = a + step * b (no inner product: the partial-sum buffer is not touched)
  VecArgs A{};
  A.nseg = vs->n_seg;
  for (int i = 0; i < vs->n_seg; ++i) {
    if (!out[i] || !a[i] || !b[i]) return PTY_ERR_INVALID;
    A.seg[i] = VSeg{out[i], a[i], b[i], nullptr, nullptr, vs->n[i]};
    A.hc[i] = 1.0;
    A.hc[NSEG + i] = step;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_VEC);
  vec_kernel<<<VB, VT, 0, st>>>(A);
  prof_mark(st, -1);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

int pty_lbfgs_accept(const pty_vspace_t* vs, double step, float* const* dir, float* const* grad,
                     float* const* new_grad, float* const* s_out, float* const* y_out, int32_t slot, void* state,
                     void* stream) {
  int rc = check_vspace(vs);
  if (rc) return rc;
  if (!dir || !grad || !new_grad || !s_out || !y_out || !state) return PTY_ERR_INVALID;
  if (slot < 0 || slot >= HMAX) return PTY_ERR_UNSUPPORTED;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  OptState* S = static_cast<OptState*>(state);
  AcceptArgs A{};
  A.nseg = vs->n_seg;
  for (int i = 0; i < vs->n_seg; ++i) {
    A.q[i] = dir[i];
    A.g[i] = grad[i];
    A.ng[i] = new_grad[i];
    A.s[i] = s_out[i];
    A.y[i] = y_out[i];
    A.n[i] = vs->n[i];
  }
  A.step = (float)step;
  A.part = &S->part[0][0][0];
  prof_mark(st, KID_ACCEPT);
  accept_kernel<<<VB, VT, 0, st>>>(A);
  if (cudaGetLastError() != cudaSuccess) return PTY_ERR_CUDA;
  rc = run_scalar(S, OP_ACCEPT, vs, slot, 0, st);
  prof_mark(st, -1);
  return rc;
}

int pty_lbfgs_read(const void* state, double* out, void* stream) {
  if (!state || !out) return PTY_ERR_INVALID;
  const OptState* S = static_cast<const OptState*>(state);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // d_value, new_d_value, gamma[NSEG], dot[NSEG]
  if (cudaMemcpyAsync(out, &S->dval, 2 * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess) return PTY_ERR_CUDA;
  if (cudaMemcpyAsync(out + 2, &S->gamma[0], NSEG * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess)
    return PTY_ERR_CUDA;
  if (cudaMemcpyAsync(out + 2 + NSEG, &S->dot[0], NSEG * sizeof(double), cudaMemcpyDefault, st) != cudaSuccess)
    return PTY_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

int pty_orthogonalize_modes(void* probe, int64_t n_pixels, int32_t n_modes, void* stream) {
  if (!probe || n_pixels <= 0 || n_modes <= 0) return PTY_ERR_INVALID;
  if (n_modes == 1) return PTY_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  prof_mark(st, KID_ORTHO);
  orthogonalize_kernel<<<1, 1024, 0, st>>>(static_cast<float2*>(probe), n_pixels, n_modes);
  prof_mark(st, -1);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

}  // extern "C"

// Window DFTs as dense GEMMs on the tensor cores (tcgen05), in BF16x3 (or BF16x6) split
// precision with FP32 accumulation: the tensor-core counterpart of the FP32 register FFT for windows of
// 64, 128 and 256 px (the precision sweep of pypty.fft.fft2 / ifft2, pypty/fft.py:114-156).
//
// One pass transforms every row of every window and writes the result transposed:
//   out[b][k][r] = scale * sum_c in[b][r][c] * w^(c k),   w = exp(-+ 2 pi i / W),
// so two passes give the 2D DFT in natural (ky, kx) order. As a real GEMM the rows of all
// windows are the M dimension (M = windows * W), the interleaved real/imaginary parts of a
// row are K (= 2W) and of the output N (= 2W); the constant real matrix B^T (N x K) holds
// the 2x2 blocks [[Re w, -Im w], [Im w, Re w]]. Split precision: every FP32 value x is a sum
// of S BF16 terms t0 = bf16(x), t1 = bf16(x - t0), ...; D = sum over products of terms
// (i, j) with i + j < S accumulates in FP32 in tensor memory. S = 2 (BF16x3: 3 products,
// ~2^-17 relative error per product) or S = 3 (BF16x6: 6 products, FP32-level error).
//
// Per CTA: a 128-row x BN-column tile of D (BN = min(2W, 256 / 128)), K in blocks of 64 through a
// two-stage shared-memory ring. B blocks are pre-split and pre-swizzled images in global
// memory (L2-resident, shared by all CTAs) moved by one-dimensional bulk copies; A blocks
// are loaded as FP32, split in registers and stored in the 128B-swizzled K-major layout by
// all threads. One thread issues the MMAs of a stage (products x 4 K-steps of 16) into one of
// two TMEM accumulators (ping-pong by K block) and commits them to the stage's "empty" and the
// buffer's "drain" mbarriers. The tensor core's FP32 accumulation is biased (its error grows
// linearly with the number of accumulated MMAs, ~2^-24 each), so every K block's partial
// product is drained into registers with 32-lane TMEM loads (warp w: lanes 32 (w % 4), column
// part w / 4 of four) and added there with round-to-nearest FP32 adds, while the tensor core works on
// the next block. Every wait is bounded; a wait that runs out sets the error word instead of
// spinning. The epilogue stores the transposed window with 256-byte coalesced warp stores.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"
#include "umma.cuh"

namespace pty {
namespace dg {

constexpr int BM = 128, BK = 64, THREADS = 512, STAGES = 2;
constexpr int NPART = THREADS / 128;   // warps per TMEM lane quadrant: each drains BN / NPART columns

// S = number of BF16 slices per FP32 operand of A:
//   S = 2 (BF16x3): floating split a = hi + lo (hi = bf16(a), lo = bf16(a - hi)), the same for
//         B; products hh, hl, lh in one accumulator (~2^-17 relative per product).
//   S = 3 (BF16x6, exact accumulation): fixed-point integer slices. Every row of A is scaled per
//         64-wide K block by 2^(7 - E) (2^E just above the block's largest magnitude) and cut
//         into integers s0, s1, s2 in [-128, 128] with a 2^(7-E) = s0 + s1 2^-8 + s2 2^-16 (+ <=
//         2^-17); B = 2^-7 (u0 + u1 2^-8 + u2 2^-16) likewise with a fixed scale (|B| <= 1).
//         Integers of 8 bits are exact in BF16 and their products exact in FP32, so the main
//         product s0 u0, summed over a 64-wide K block (< 2^20), is exact however the tensor
//         core accumulates; the five correction products (s0 u1, s1 u0 at 2^-8; s0 u2, s1 u1,
//         s2 u0 at 2^-16, pre-scaled by 2^-8 in the slices: s2 in A, u2 and a copy of u1 in B)
//         share a second accumulator whose truncation, scaled 2^-8 below the main one, stays
//         under FP32 rounding. The only roundings left are the round-to-nearest drains, so the
//         error does not pile up with a bias over chained transforms.
// B carries TB slices: 2 for S = 2, 4 (u0, u1, u2 2^-8, u1 2^-8) for S = 3. BN shrinks to 128
// for S = 3 so that two stages fit in shared memory.
template <int W, int S>
struct Cfg {
  static constexpr bool EXACT = S == 3;
  static constexpr int TB = EXACT ? 4 : S;
  static constexpr int NTOT = 2 * W;
  static constexpr int BNMAX = S == 2 ? 256 : 128;
  static constexpr int BN = NTOT < BNMAX ? NTOT : BNMAX;
  static constexpr int NT = NTOT / BN;
  static constexpr int KC = (2 * W) / BK;
  static constexpr int A_BYTES = BM * BK * 2;          // one slice
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE = S * A_BYTES + TB * B_BYTES;
  static constexpr int SMEM = STAGES * STAGE + 1024;   // + slack for 1024-byte alignment
  static constexpr size_t IMG_BYTES = (size_t)TB * NT * KC * B_BYTES;   // every slice's image, one direction
  // TMEM: two K-block buffers (ping-pong); with S = 3 each holds the main product s0 u0 and,
  // separately, the correction products
  static constexpr int ACCS = S == 3 ? 2 : 1;
  static constexpr int TMEM_COLS = 2 * ACCS * BN;
  static_assert(TMEM_COLS <= 512, "TMEM holds 512 columns");
};

// ring of per-row scale exponents of the exact variant: block kc's are written in iteration kc
// and read by the drain in iteration kc + 1; iteration kc + 4 rewrites the slot, after two
// block barriers that every drain of kc precedes
constexpr int EXP_RING = 4;

// Pre-split, pre-swizzled images of B^T for one direction: [term][nt][kc][BN x 64 block].
template <int W, int S>
__global__ void dft_matrix_kernel(uint8_t* img, int inverse) {
  using C = Cfg<W, S>;
  const long long total = (long long)C::NT * C::KC * C::BN * BK;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % BK);
    const int r = (int)((i / BK) % C::BN);
    const int kc = (int)((i / ((long long)BK * C::BN)) % C::KC);
    const int nt = (int)(i / ((long long)BK * C::BN * C::KC));
    const int n = nt * C::BN + r, kk = kc * BK + k;
    const int c = kk >> 1, kout = n >> 1;
    const int m = (c * kout) % W;
    double sn, cs;
    sincospi(2.0 * (double)m / (double)W, &sn, &cs);
    const double wr = cs, wi = inverse ? sn : -sn;   // w^(c k) = exp(-+ 2 pi i c k / W)
    const int so = n & 1, si = kk & 1;
    const double v = so == 0 ? (si == 0 ? wr : -wi) : (si == 0 ? wi : wr);
    const size_t blk = ((size_t)nt * C::KC + kc) * C::B_BYTES + umma::sw128_offset(r, k);
    auto put = [&](int term, double x) {   // x exactly representable in BF16 by construction
      *reinterpret_cast<__nv_bfloat16*>(img + (size_t)term * C::NT * C::KC * C::B_BYTES + blk) =
          __float2bfloat16_rn((float)x);
    };
    if constexpr (C::EXACT) {
      // 128 v = u0 + u1 2^-8 + u2 2^-16 + (|.| <= 2^-17), u_i integers in [-128, 128] (exact in double)
      const double x0 = 128.0 * v, u0 = rint(x0);
      const double x1 = (x0 - u0) * 256.0, u1 = rint(x1);
      const double u2 = rint((x1 - u1) * 256.0);
      put(0, u0);
      put(1, u1);
      put(2, u2 * 0.00390625);   // 2^-16 products, pre-scaled into the 2^-8 accumulator
      put(3, u1 * 0.00390625);   // for s1 u1
    } else {
      double rest = v;
#pragma unroll
      for (int term = 0; term < S; ++term) {
        const __nv_bfloat16 t = __float2bfloat16_rn((float)rest);
        rest -= (double)__bfloat162float(t);
        put(term, (double)__bfloat162float(t));
      }
    }
  }
}

template <int W, int S>
__global__ void __launch_bounds__(THREADS, 1)
    dft_pass_kernel(const float2* __restrict__ in, float2* __restrict__ out, const uint8_t* __restrict__ img,
                    long long n_rows, float scale, int* err) {
  using C = Cfg<W, S>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full_bar[STAGES], empty_bar[STAGES], drain_bar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort;   // a bounded wait ran out somewhere in the CTA: issue nothing more
  __shared__ int16_t rowexp[C::EXACT ? EXP_RING : 1][BM];   // exact variant: per-row scale exponents
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // the N tiles of one row tile are adjacent in the grid: the second read of A hits L2
  const long long row0 = (long long)blockIdx.y * BM;
  const int nt = blockIdx.x;
  int e = 0;
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&drain_bar[0], 1);
    mbar_init(&drain_bar[1], 1);
    s_abort = 0;
    fence_async_shared();
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, C::TMEM_COLS);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint8_t* img_nt = img + (size_t)nt * C::KC * C::B_BYTES;
  constexpr size_t TERM = (size_t)C::NT * C::KC * C::B_BYTES;
  constexpr uint32_t idesc = umma::idesc_bf16_f32(BM, C::BN);
  uint32_t full_par[STAGES] = {0, 0}, empty_par[STAGES] = {0, 0}, drain_par[2] = {0, 0};
  // this thread's accumulator slice: TMEM lanes 32 (w % 4) + lane (tile rows), column part w / 4
  const int q = warp & 3, h = warp >> 2;
  constexpr int HALF = C::BN / NPART;   // columns this warp drains
  float acc[HALF];
#pragma unroll
  for (int j = 0; j < HALF; ++j) acc[j] = 0.0f;
  // add the partial product of K block kc (TMEM buffer kc & 1) to the registers: FP32 adds with
  // round-to-nearest, so the tensor core's accumulation runs over one K block only
  int drained = -1;   // last K block drained
  auto drain = [&](int kc) {
    const int buf = kc & 1;
    drained = kc;
    mbar_wait(&drain_bar[buf], drain_par[buf], &e);
    umma::fence_after_sync();
    // exact variant: this thread's row (TMEM lane 32 q + lane) carries scale 2^(E - 7) from A and
    // 2^-7 from B
    float rs = 1.0f;
    if constexpr (C::EXACT) rs = ldexpf(1.0f, (int)rowexp[kc % EXP_RING][32 * q + lane] - 14);
#pragma unroll
    for (int c0 = 0; c0 < HALF; c0 += 32) {
      const uint32_t col = (uint32_t)(buf * C::ACCS * C::BN + h * HALF + c0);
      float v[32];
      umma::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + col, v);
      if constexpr (C::EXACT) {
        float w[32];
        umma::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + col + C::BN, w);
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[c0 + j] = fmaf(fmaf(w[j], 0.00390625f, v[j]), rs, acc[c0 + j]);
      } else {
        if constexpr (C::ACCS == 2) {
          float w[32];
          umma::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + col + C::BN, w);
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] += w[j];
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[c0 + j] += v[j];
      }
    }
    umma::fence_before_sync();
  };

  // A blocks: rows row0 .. row0+127, real columns kc*64 .. kc*64+63 (16 float4 per row); the next
  // block's FP32 values are loaded into registers while the current block's MMAs run
  constexpr int APT = (BM * BK / 4) / THREADS;   // float4 per thread per block
  float4 pre[APT];
  auto load_a = [&](int kc) {
#pragma unroll
    for (int i = 0; i < APT; ++i) {
      const int qq = tid + THREADS * i;
      const int r = qq >> 4, c4 = qq & 15;
      const long long row = row0 + r;
      pre[i] = row < n_rows ? reinterpret_cast<const float4*>(in + row * W)[kc * 16 + c4] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };
  load_a(0);

  // Failure handling: every wait is bounded; a thread whose wait ran out sets s_abort, which the
  // whole CTA reads after the next barrier (uniformly) and then stops issuing copies and MMAs.
  // Thread 0 tracks what it has in flight (bulk copies not yet waited for, MMAs of the previous
  // K block not yet drained) and waits for those, again bounded, before TMEM is freed.
  bool copy_pending[STAGES] = {false, false};   // thread 0 only
  int committed = -1;                           // thread 0: last K block whose MMAs were committed
  bool aborted = false;
  for (int kc = 0; kc < C::KC; ++kc) {
    const int s = kc % STAGES;
    uint8_t* sA = base + s * C::STAGE;            // S terms of A, then S terms of B
    uint8_t* sB = sA + S * C::A_BYTES;
    if (kc >= STAGES) mbar_wait(&empty_bar[s], empty_par[s], &e);   // the MMAs of kc - STAGES are done
    if (tid == 0 && !e) {
      mbar_expect_tx(&full_bar[s], C::TB * C::B_BYTES);
#pragma unroll
      for (int term = 0; term < C::TB; ++term)
        bulk_copy_g2s(sB + term * C::B_BYTES, img_nt + term * TERM + (size_t)kc * C::B_BYTES, C::B_BYTES,
                      &full_bar[s]);
      copy_pending[s] = true;
    }
#pragma unroll
    for (int i = 0; i < APT; ++i) {
      const int qq = tid + THREADS * i;
      const int r = qq >> 4, c4 = qq & 15;
      const uint32_t off = umma::sw128_offset(r, 4 * c4);
      float4 rest = pre[i];
      if constexpr (C::EXACT) {
        // the row's 64 values of this K block sit in 16 consecutive lanes (c4 = 0..15): their
        // largest magnitude m = f 2^E (f in [0.5, 1)) sets the scale 2^(7 - E), |a 2^(7-E)| < 128
        float m = fmaxf(fmaxf(fabsf(rest.x), fabsf(rest.y)), fmaxf(fabsf(rest.z), fabsf(rest.w)));
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        int E = 0;
        frexpf(m, &E);
        E = max(E, -100);   // a (near-)zero block: keep the scale finite
        if (c4 == 0) rowexp[kc % EXP_RING][r] = (int16_t)E;
        const float up = ldexpf(1.0f, 7 - E);
        float x[4] = {rest.x * up, rest.y * up, rest.z * up, rest.w * up};
        uint16_t t[3][4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          // x = s0 + s1 2^-8 + s2 2^-16 (+ <= 2^-17); every subtraction below is exact
          const float s0 = rintf(x[c]);
          const float x1 = (x[c] - s0) * 256.0f, s1 = rintf(x1);
          const float s2 = rintf((x1 - s1) * 256.0f);
          t[0][c] = umma::bf16_bits(s0);
          t[1][c] = umma::bf16_bits(s1);
          t[2][c] = umma::bf16_bits(s2 * 0.00390625f);   // pre-scaled into the 2^-8 accumulator
        }
#pragma unroll
        for (int term = 0; term < 3; ++term)
          *reinterpret_cast<uint2*>(sA + term * C::A_BYTES + off) =
              make_uint2(t[term][0] | ((uint32_t)t[term][1] << 16), t[term][2] | ((uint32_t)t[term][3] << 16));
      } else {
#pragma unroll
      for (int term = 0; term < S; ++term) {
        // successive BF16 terms; every residual x - bf16(x) is exact in FP32
        const uint16_t t0 = umma::bf16_bits(rest.x), t1 = umma::bf16_bits(rest.y);
        const uint16_t t2 = umma::bf16_bits(rest.z), t3 = umma::bf16_bits(rest.w);
        *reinterpret_cast<uint2*>(sA + term * C::A_BYTES + off) =
            make_uint2(t0 | ((uint32_t)t1 << 16), t2 | ((uint32_t)t3 << 16));
        if (term + 1 < S) {
          rest.x -= umma::bf16_value(t0);
          rest.y -= umma::bf16_value(t1);
          rest.z -= umma::bf16_value(t2);
          rest.w -= umma::bf16_value(t3);
        }
      }
      }
    }
    if (kc + 1 < C::KC) load_a(kc + 1);
    if (e) s_abort = 1;
    fence_async_shared();
    umma::fence_before_sync();
    __syncthreads();   // A is written; every thread has drained TMEM buffer kc & 1 (block kc - 2)
    if (s_abort) {     // uniform: every write of s_abort precedes this barrier
      aborted = true;
      break;
    }
    if (tid == 0) {
      mbar_wait(&full_bar[s], full_par[s], &e);
      if (e) {
        s_abort = 1;   // the copy may still be in flight: waited for below; no MMA of this block
      } else {
        copy_pending[s] = false;
      }
    }
    if (tid == 0 && !e) {
      umma::fence_after_sync();
      const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
      const uint32_t d = tmem + (uint32_t)((kc & 1) * C::ACCS * C::BN);
      const uint32_t dc = d + (C::ACCS == 2 ? (uint32_t)C::BN : 0u);   // accumulator of the correction products
#pragma unroll
      for (int k = 0; k < BK / 16; ++k) {
        const uint32_t o = 32u * k;
        if constexpr (C::EXACT) {
          // (A slice, B slice, accumulator): s0 u0 -> main; s0 u1, s1 u0, s0 (u2 2^-8),
          // s1 (u1 2^-8), (s2 2^-8) u0 -> corrections
          constexpr int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 3, 0};
#pragma unroll
          for (int j = 0; j < 6; ++j)
            umma::mma_bf16(j == 0 ? d : dc, umma::desc_sw128(a0 + pa[j] * C::A_BYTES + o),
                           umma::desc_sw128(b0 + pb[j] * C::B_BYTES + o), idesc,
                           k > 0 || j > 1 ? 1u : 0u);
        } else {
        // every product of terms (i, j) with i + j < S, largest first
#pragma unroll
        for (int sum = 0; sum < S; ++sum)
#pragma unroll
          for (int i = 0; i <= sum; ++i) {
            const bool main = sum == 0 || C::ACCS == 1;
            const bool first = C::ACCS == 1 ? (k | sum) == 0 : (k == 0 && i == 0 && sum <= 1);
            umma::mma_bf16(main ? d : dc, umma::desc_sw128(a0 + i * C::A_BYTES + o),
                           umma::desc_sw128(b0 + (sum - i) * C::B_BYTES + o), idesc, !first);
          }
        }
      }
      umma::mma_commit(&empty_bar[s]);
      umma::mma_commit(&drain_bar[kc & 1]);
      committed = kc;
    }
    // block kc - 1's MMAs were committed: thread 0's wait of iteration kc - 1 succeeded, or the
    // CTA would have stopped at this iteration's barrier
    if (kc > 0) drain(kc - 1);   // overlaps the MMAs of block kc
  }
  if (!aborted) {
    if (e) s_abort = 1;
    __syncthreads();
    aborted = s_abort != 0;   // thread 0 may have failed in the last iteration
    if (!aborted) drain(C::KC - 1);
  }
  if (aborted && tid == 0) {
    // let this CTA's own copies and MMAs finish (bounded) before TMEM and shared memory go
    int e2 = 0;
    for (int st = 0; st < STAGES; ++st)
      if (copy_pending[st]) mbar_wait(&full_bar[st], full_par[st], &e2);
    if (committed > drained) mbar_wait(&drain_bar[committed & 1], drain_par[committed & 1], &e2);
  }
  // epilogue: out[window][k][row in window] = scale * acc (transposed, coalesced over rows); NaN
  // when the CTA stopped early, so that a failed transform cannot pass for a result
  const long long row = row0 + 32 * q + lane;
  const long long win = row / W;
  const int r = (int)(row % W);
  if (row < n_rows) {
    float2* o = out + win * (long long)W * W + r;
    const int k0 = (nt * C::BN + h * HALF) >> 1;
    const float nan = __int_as_float(0x7fc00000);
#pragma unroll
    for (int j = 0; j < HALF / 2; ++j)
      o[(long long)(k0 + j) * W] = aborted ? make_float2(nan, nan)
                                           : make_float2(acc[2 * j] * scale, acc[2 * j + 1] * scale);
  }
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, C::TMEM_COLS);
  if (aborted && tid == 0 && err) atomicExch(err, 1);
}

struct Ws {
  size_t o_fwd, o_inv, o_tmp, o_err, total;
};

template <int W, int S>
Ws make_ws(long long batch) {
  Ws w;
  w.o_fwd = 0;
  w.o_inv = align_up(w.o_fwd + Cfg<W, S>::IMG_BYTES);
  w.o_err = align_up(w.o_inv + Cfg<W, S>::IMG_BYTES);
  w.o_tmp = align_up(w.o_err + 256);
  w.total = align_up(w.o_tmp + (size_t)batch * W * W * sizeof(float2));
  return w;
}

// clear_err: reset the error word first (a top-level call); a caller running many transforms
// in one call (the layered path) clears it once and reads it at its end.
template <int W, int S>
int run_fft2(const float2* in, float2* out, long long batch, int inverse, void* ws, size_t ws_bytes, cudaStream_t st,
             bool clear_err) {
  using C = Cfg<W, S>;
  const Ws w = make_ws<W, S>(batch);
  if (ws_bytes < w.total) return PTY_ERR_WORKSPACE;
  uint8_t* img = at<uint8_t>(ws, inverse ? w.o_inv : w.o_fwd);
  int* err = at<int>(ws, w.o_err);
  float2* tmp = at<float2>(ws, w.o_tmp);
  prof_mark(st, KID_DFT_TABLES);
  dft_matrix_kernel<W, S><<<256, 256, 0, st>>>(img, inverse);
  if (clear_err && cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return PTY_ERR_CUDA;
  auto k = dft_pass_kernel<W, S>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM) != cudaSuccess) return PTY_ERR_CUDA;
  const float sc = inverse ? 1.0f / (float)W : 1.0f;   // 1/W per pass: exact
  // at most 32768 row tiles per launch (grid.y <= 65535)
  const long long max_win = 32768LL * BM / W;
  for (long long b0 = 0; b0 < batch; b0 += max_win) {
    const long long nb = batch - b0 < max_win ? batch - b0 : max_win;
    const long long rows = nb * W;
    const dim3 grid(C::NT, (unsigned)((rows + BM - 1) / BM));
    const size_t off = (size_t)b0 * W * W;
    prof_mark(st, KID_DFT_GEMM);
    k<<<grid, THREADS, C::SMEM, st>>>(in + off, tmp + off, img, rows, sc, err);
    prof_mark(st, KID_DFT_GEMM);
    k<<<grid, THREADS, C::SMEM, st>>>(tmp + off, out + off, img, rows, sc, err);
  }
  prof_mark(st, -1);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

}  // namespace dg

// The layered path's entry: one transform of a call that clears the error word itself once.
int tc_fft2(const float2* in, float2* out, long long batch, int window, int inverse, int terms, void* ws,
            size_t ws_bytes, cudaStream_t st) {
  if (!in || !out || !ws || batch <= 0 || in == out) return PTY_ERR_INVALID;
  switch (window * 10 + terms) {
    case 642: return dg::run_fft2<64, 2>(in, out, batch, inverse, ws, ws_bytes, st, false);
    case 1282: return dg::run_fft2<128, 2>(in, out, batch, inverse, ws, ws_bytes, st, false);
    case 2562: return dg::run_fft2<256, 2>(in, out, batch, inverse, ws, ws_bytes, st, false);
    case 643: return dg::run_fft2<64, 3>(in, out, batch, inverse, ws, ws_bytes, st, false);
    case 1283: return dg::run_fft2<128, 3>(in, out, batch, inverse, ws, ws_bytes, st, false);
    case 2563: return dg::run_fft2<256, 3>(in, out, batch, inverse, ws, ws_bytes, st, false);
    default: return PTY_ERR_UNSUPPORTED;
  }
}

// The error word inside a tensor-core DFT workspace (its offset does not depend on the batch).
int* tc_err_word(void* ws, int window, int terms) {
  switch (window * 10 + terms) {
    case 642: return at<int>(ws, dg::make_ws<64, 2>(1).o_err);
    case 1282: return at<int>(ws, dg::make_ws<128, 2>(1).o_err);
    case 2562: return at<int>(ws, dg::make_ws<256, 2>(1).o_err);
    case 643: return at<int>(ws, dg::make_ws<64, 3>(1).o_err);
    case 1283: return at<int>(ws, dg::make_ws<128, 3>(1).o_err);
    case 2563: return at<int>(ws, dg::make_ws<256, 3>(1).o_err);
    default: return nullptr;
  }
}
}  // namespace pty

using namespace pty;

extern "C" {

static int ws_bytes_for(int32_t batch, int32_t window, int terms, size_t* bytes) {
  if (!bytes || batch <= 0) return PTY_ERR_INVALID;
  const int key = window * 10 + terms;
  switch (key) {
    case 642: *bytes = dg::make_ws<64, 2>(batch).total; return PTY_OK;
    case 1282: *bytes = dg::make_ws<128, 2>(batch).total; return PTY_OK;
    case 2562: *bytes = dg::make_ws<256, 2>(batch).total; return PTY_OK;
    case 643: *bytes = dg::make_ws<64, 3>(batch).total; return PTY_OK;
    case 1283: *bytes = dg::make_ws<128, 3>(batch).total; return PTY_OK;
    case 2563: *bytes = dg::make_ws<256, 3>(batch).total; return PTY_OK;
    default: return PTY_ERR_UNSUPPORTED;
  }
}

static int fft2_tc(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse, int terms,
                   void* workspace, size_t workspace_bytes, void* stream) {
  if (!in || !out || !workspace || batch <= 0) return PTY_ERR_INVALID;
  if (in == out) return PTY_ERR_INVALID;
  const float2* i = static_cast<const float2*>(in);
  float2* o = static_cast<float2*>(out);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (window * 10 + terms) {
    case 642: return dg::run_fft2<64, 2>(i, o, batch, inverse, workspace, workspace_bytes, st, true);
    case 1282: return dg::run_fft2<128, 2>(i, o, batch, inverse, workspace, workspace_bytes, st, true);
    case 2562: return dg::run_fft2<256, 2>(i, o, batch, inverse, workspace, workspace_bytes, st, true);
    case 643: return dg::run_fft2<64, 3>(i, o, batch, inverse, workspace, workspace_bytes, st, true);
    case 1283: return dg::run_fft2<128, 3>(i, o, batch, inverse, workspace, workspace_bytes, st, true);
    case 2563: return dg::run_fft2<256, 3>(i, o, batch, inverse, workspace, workspace_bytes, st, true);
    default: return PTY_ERR_UNSUPPORTED;
  }
}

int pty_fft2_bf16x3_workspace_bytes(int32_t batch, int32_t window, size_t* bytes) {
  return ws_bytes_for(batch, window, 2, bytes);
}

int pty_fft2_bf16x3(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse, void* workspace,
                    size_t workspace_bytes, void* stream) {
  return fft2_tc(in, out, batch, window, inverse, 2, workspace, workspace_bytes, stream);
}

int pty_fft2_bf16x6_workspace_bytes(int32_t batch, int32_t window, size_t* bytes) {
  return ws_bytes_for(batch, window, 3, bytes);
}

int pty_fft2_bf16x6(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse, void* workspace,
                    size_t workspace_bytes, void* stream) {
  return fft2_tc(in, out, batch, window, inverse, 3, workspace, workspace_bytes, stream);
}

}  // extern "C"

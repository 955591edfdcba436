// Window DFTs as dense GEMMs on the tensor cores (tcgen05), in BF16x3 split precision with
// FP32 accumulation: the tensor-core counterpart of the FP32 register FFT for windows of
// 64, 128 and 256 px (the precision sweep of pypty.fft.fft2 / ifft2, pypty/fft.py:114-156).
//
// One pass transforms every row of every window and writes the result transposed:
//   out[b][k][r] = scale * sum_c in[b][r][c] * w^(c k),   w = exp(-+ 2 pi i / W),
// so two passes give the 2D DFT in natural (ky, kx) order. As a real GEMM the rows of all
// windows are the M dimension (M = windows * W), the interleaved real/imaginary parts of a
// row are K (= 2W) and of the output N (= 2W); the constant real matrix B^T (N x K) holds
// the 2x2 blocks [[Re w, -Im w], [Im w, Re w]]. Split precision: every FP32 value x is
// hi + lo with hi = bf16(x), lo = bf16(x - hi), and D = A_hi B_hi + A_hi B_lo + A_lo B_hi
// (the lo*lo term, ~2^-18 relative, is dropped) accumulates in FP32 in tensor memory.
//
// Per CTA: a 128-row x BN-column tile of D (BN = min(2W, 256)), K in blocks of 64 through a
// two-stage shared-memory ring. B blocks are pre-split and pre-swizzled images in global
// memory (L2-resident, shared by all CTAs) moved by one-dimensional bulk copies; A blocks
// are loaded as FP32, split in registers and stored in the 128B-swizzled K-major layout by
// all threads. One thread issues the 12 MMAs (3 products x 4 K-steps of 16) of a stage and
// commits them to the stage's "empty" mbarrier; every wait is bounded and a wait that runs
// out sets the error word instead of spinning. The epilogue reads the accumulator with
// 32-lane TMEM loads (warp w: lanes 32 (w % 4), column half w / 4) and stores the transposed
// window with 256-byte coalesced warp stores.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"
#include "umma.cuh"

namespace pty {
namespace dg {

constexpr int BM = 128, BK = 64, THREADS = 256, STAGES = 2;

template <int W>
struct Cfg {
  static constexpr int NTOT = 2 * W;
  static constexpr int BN = NTOT < 256 ? NTOT : 256;
  static constexpr int NT = NTOT / BN;
  static constexpr int KC = (2 * W) / BK;
  static constexpr int A_BYTES = BM * BK * 2;          // one of hi / lo
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int SMEM = STAGES * STAGE + 1024;   // + slack for 1024-byte alignment
  static constexpr size_t IMG_BYTES = (size_t)2 * NT * KC * B_BYTES;   // hi and lo images of one direction
};

// Pre-split, pre-swizzled images of B^T for one direction: [hl][nt][kc][BN x 64 block].
template <int W>
__global__ void dft_matrix_kernel(uint8_t* img, int inverse) {
  using C = Cfg<W>;
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
    const __nv_bfloat16 hi = __float2bfloat16_rn((float)v);
    const __nv_bfloat16 lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
    const size_t blk = ((size_t)nt * C::KC + kc) * C::B_BYTES + umma::sw128_offset(r, k);
    *reinterpret_cast<__nv_bfloat16*>(img + blk) = hi;
    *reinterpret_cast<__nv_bfloat16*>(img + (size_t)C::NT * C::KC * C::B_BYTES + blk) = lo;
  }
}

template <int W>
__global__ void __launch_bounds__(THREADS, 1)
    dft_pass_kernel(const float2* __restrict__ in, float2* __restrict__ out, const uint8_t* __restrict__ img,
                    long long n_rows, float scale, int* err) {
  using C = Cfg<W>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full_bar[STAGES], empty_bar[STAGES], done_bar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long row0 = (long long)blockIdx.x * BM;
  const int nt = blockIdx.y;
  int e = 0;
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    fence_async_shared();
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, C::BN);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint8_t* img_hi = img + (size_t)nt * C::KC * C::B_BYTES;
  const uint8_t* img_lo = img + (size_t)C::NT * C::KC * C::B_BYTES + (size_t)nt * C::KC * C::B_BYTES;
  constexpr uint32_t idesc = umma::idesc_bf16_f32(BM, C::BN);
  uint32_t full_par[STAGES] = {0, 0}, empty_par[STAGES] = {0, 0};

  for (int kc = 0; kc < C::KC; ++kc) {
    const int s = kc % STAGES;
    uint8_t* sAh = base + s * C::STAGE;
    uint8_t* sAl = sAh + C::A_BYTES;
    uint8_t* sBh = sAl + C::A_BYTES;
    uint8_t* sBl = sBh + C::B_BYTES;
    if (kc >= STAGES) mbar_wait(&empty_bar[s], empty_par[s], &e);   // the MMAs of kc - STAGES are done
    if (tid == 0) {
      mbar_expect_tx(&full_bar[s], 2 * C::B_BYTES);
      bulk_copy_g2s(sBh, img_hi + (size_t)kc * C::B_BYTES, C::B_BYTES, &full_bar[s]);
      bulk_copy_g2s(sBl, img_lo + (size_t)kc * C::B_BYTES, C::B_BYTES, &full_bar[s]);
    }
    // A block: rows row0 .. row0+127, real columns kc*64 .. kc*64+63 (16 float4 per row)
#pragma unroll
    for (int i = 0; i < (BM * BK / 4) / THREADS; ++i) {
      const int q = tid + THREADS * i;
      const int r = q >> 4, c4 = q & 15;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      const long long row = row0 + r;
      if (row < n_rows) v = reinterpret_cast<const float4*>(in + row * W)[kc * 16 + c4];
      uint16_t h0, l0, h1, l1, h2, l2, h3, l3;
      umma::split_bf16(v.x, h0, l0);
      umma::split_bf16(v.y, h1, l1);
      umma::split_bf16(v.z, h2, l2);
      umma::split_bf16(v.w, h3, l3);
      const uint32_t off = umma::sw128_offset(r, 4 * c4);
      *reinterpret_cast<uint2*>(sAh + off) = make_uint2(h0 | ((uint32_t)h1 << 16), h2 | ((uint32_t)h3 << 16));
      *reinterpret_cast<uint2*>(sAl + off) = make_uint2(l0 | ((uint32_t)l1 << 16), l2 | ((uint32_t)l3 << 16));
    }
    fence_async_shared();
    umma::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      mbar_wait(&full_bar[s], full_par[s], &e);
      umma::fence_after_sync();
      const uint32_t ah = smem_u32(sAh), al = smem_u32(sAl), bh = smem_u32(sBh), bl = smem_u32(sBl);
#pragma unroll
      for (int k = 0; k < BK / 16; ++k) {
        const uint32_t o = 32u * k;
        umma::mma_bf16(tmem, umma::desc_sw128(ah + o), umma::desc_sw128(bh + o), idesc, (kc | k) != 0);
        umma::mma_bf16(tmem, umma::desc_sw128(ah + o), umma::desc_sw128(bl + o), idesc, 1);
        umma::mma_bf16(tmem, umma::desc_sw128(al + o), umma::desc_sw128(bh + o), idesc, 1);
      }
      umma::mma_commit(&empty_bar[s]);
    }
  }
  if (tid == 0) umma::mma_commit(&done_bar);
  uint32_t done_par = 0;
  mbar_wait(&done_bar, done_par, &e);
  umma::fence_after_sync();
  // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (tile rows), column half w / 4
  const int q = warp & 3, h = warp >> 2;
  const long long row = row0 + 32 * q + lane;
  const long long win = row / W;
  const int r = (int)(row % W);
  constexpr int HALF = C::BN / 2;
#pragma unroll 1
  for (int c0 = 0; c0 < HALF; c0 += 32) {
    float v[32];
    umma::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(h * HALF + c0), v);
    if (row < n_rows) {
      const int k0 = (nt * C::BN + h * HALF + c0) >> 1;
      float2* o = out + win * (long long)W * W + r;
#pragma unroll
      for (int j = 0; j < 16; ++j) o[(long long)(k0 + j) * W] = make_float2(v[2 * j] * scale, v[2 * j + 1] * scale);
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(tmem, C::BN);
  if (e && lane == 0 && err) atomicExch(err, 1);
}

template <int W>
size_t img_bytes() {
  return Cfg<W>::IMG_BYTES;
}

struct Ws {
  size_t o_fwd, o_inv, o_tmp, o_err, total;
};

template <int W>
Ws make_ws(long long batch) {
  Ws w;
  w.o_fwd = 0;
  w.o_inv = align_up(w.o_fwd + Cfg<W>::IMG_BYTES);
  w.o_err = align_up(w.o_inv + Cfg<W>::IMG_BYTES);
  w.o_tmp = align_up(w.o_err + 256);
  w.total = align_up(w.o_tmp + (size_t)batch * W * W * sizeof(float2));
  return w;
}

template <int W>
int run_fft2(const float2* in, float2* out, long long batch, int inverse, void* ws, size_t ws_bytes, cudaStream_t st) {
  using C = Cfg<W>;
  const Ws w = make_ws<W>(batch);
  if (ws_bytes < w.total) return PTY_ERR_WORKSPACE;
  uint8_t* img = at<uint8_t>(ws, inverse ? w.o_inv : w.o_fwd);
  int* err = at<int>(ws, w.o_err);
  float2* tmp = at<float2>(ws, w.o_tmp);
  prof_mark(st, KID_DFT_TABLES);
  dft_matrix_kernel<W><<<256, 256, 0, st>>>(img, inverse);
  if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return PTY_ERR_CUDA;
  auto k = dft_pass_kernel<W>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM) != cudaSuccess) return PTY_ERR_CUDA;
  const long long rows = batch * W;
  const dim3 grid((unsigned)((rows + BM - 1) / BM), C::NT);
  const float sc = inverse ? 1.0f / (float)W : 1.0f;   // 1/W per pass: exact
  prof_mark(st, KID_DFT_GEMM);
  k<<<grid, THREADS, C::SMEM, st>>>(in, tmp, img, rows, sc, err);
  prof_mark(st, KID_DFT_GEMM);
  k<<<grid, THREADS, C::SMEM, st>>>(tmp, out, img, rows, sc, err);
  prof_mark(st, -1);
  return cudaGetLastError() == cudaSuccess ? PTY_OK : PTY_ERR_CUDA;
}

}  // namespace dg
}  // namespace pty

using namespace pty;

extern "C" {

int pty_fft2_bf16x3_workspace_bytes(int32_t batch, int32_t window, size_t* bytes) {
  if (!bytes || batch <= 0) return PTY_ERR_INVALID;
  switch (window) {
    case 64: *bytes = dg::make_ws<64>(batch).total; return PTY_OK;
    case 128: *bytes = dg::make_ws<128>(batch).total; return PTY_OK;
    case 256: *bytes = dg::make_ws<256>(batch).total; return PTY_OK;
    default: return PTY_ERR_UNSUPPORTED;
  }
}

int pty_fft2_bf16x3(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse, void* workspace,
                    size_t workspace_bytes, void* stream) {
  if (!in || !out || !workspace || batch <= 0) return PTY_ERR_INVALID;
  if (in == out) return PTY_ERR_INVALID;
  const float2* i = static_cast<const float2*>(in);
  float2* o = static_cast<float2*>(out);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  switch (window) {
    case 64: return dg::run_fft2<64>(i, o, batch, inverse, workspace, workspace_bytes, st);
    case 128: return dg::run_fft2<128>(i, o, batch, inverse, workspace, workspace_bytes, st);
    case 256: return dg::run_fft2<256>(i, o, batch, inverse, workspace, workspace_bytes, st);
    default: return PTY_ERR_UNSUPPORTED;
  }
}

}  // extern "C"

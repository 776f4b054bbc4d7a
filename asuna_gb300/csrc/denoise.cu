// denoise.cu — BF16 tensor-core kernels of the learned denoiser (training and
// inference): a U-Net over the radiance / albedo / normal images, standing in
// for the reference's OptiX AOV denoiser (src/tracer/denoiser.cpp:143-224).
//
// Tensors are NHWC bf16 with channel counts padded to multiples of 16; all
// products accumulate in fp32.  The 3x3 convolution is an implicit GEMM
// (M = pixels, N = output channels, K = 9 taps x input channels) on
// mma.sync.m16n8k16 bf16 tensor-core instructions, fed by a 3-stage cp.async
// pipeline (zero-fill for the halo) and ldmatrix fragment loads; bias, ReLU
// and the ReLU mask of the backward pass are fused into the epilogue.  The
// input gradient is the same kernel on flipped, transposed weights; the
// weight gradient is a split-K GEMM over pixels (ldmatrix.trans fragments,
// fp32 atomics into the weight-gradient buffer).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <new>
#include <vector>

#include "../../include/asuna_denoise.h"
#include "common.h"
#include "handles.h"

namespace asuna {
namespace nn {
namespace {

constexpr int kBM = 128, kBN = 64, kBK = 16, kStages = 3;
constexpr int kLds = 24;  // smem row stride in halves (48 B): ldmatrix without bank conflicts

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cpAsync16(void* smem, const void* gmem, bool valid) {
  const int n = valid ? 16 : 0;  // src-size 0: fill the 16 bytes with zeros
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smemAddr(smem)), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cpAsyncWait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
__device__ __forceinline__ void ldmatrixX4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smemAddr(p)));
}
__device__ __forceinline__ void ldmatrixX4T(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(smemAddr(p)));
}
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct ConvArgs {
  const __nv_bfloat16* in;  // [P][Cin]
  const __nv_bfloat16* w;   // [Cout][9][Cin]
  const float* bias;        // [Cout] or null
  const __nv_bfloat16* mask;  // [P][Cout] or null: out *= (mask > 0)
  void* out;                // [P][Cout] bf16, or fp32 when outF32
  int N, H, W, Cin, Cout;
  int relu, outF32;
};

// Forward 3x3 convolution, stride 1, zero padding 1.
__global__ void __launch_bounds__(256) k_conv3x3(ConvArgs a) {
  __shared__ __align__(16) __nv_bfloat16 sA[kStages][kBM * kLds];
  __shared__ __align__(16) __nv_bfloat16 sB[kStages][kBN * kLds];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;  // 4 x 2 warps of 32 x 32
  const int P = a.N * a.H * a.W;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const int cChunks = a.Cin / kBK;
  const int kSteps = 9 * cChunks;
  // this thread's A row (pixel) and B row (output channel) for the loads
  const int ar = tid >> 1, ah = (tid & 1) * 8;
  const int ap = m0 + ar;
  int an = 0, ay = 0, ax = 0;
  if (ap < P) {
    an = ap / (a.H * a.W);
    const int rem = ap - an * a.H * a.W;
    ay = rem / a.W;
    ax = rem - ay * a.W;
  }
  const int br = tid >> 1, bh = (tid & 1) * 8;
  const int bco = n0 + br;

  auto load = [&](int stage, int k) {
    const int tap = k / cChunks, c0 = (k - tap * cChunks) * kBK;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int ys = ay + dy, xs = ax + dx;
    const bool va = ap < P && ys >= 0 && ys < a.H && xs >= 0 && xs < a.W;
    const __nv_bfloat16* srcA =
        va ? a.in + ((size_t(an) * a.H + ys) * a.W + xs) * a.Cin + c0 + ah : a.in;
    cpAsync16(&sA[stage][ar * kLds + ah], srcA, va);
    if (tid < 2 * kBN) {
      const bool vb = bco < a.Cout;
      const __nv_bfloat16* srcB = vb ? a.w + (size_t(bco) * 9 + tap) * a.Cin + c0 + bh : a.w;
      cpAsync16(&sB[stage][br * kLds + bh], srcB, vb);
    }
  };

  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.0f;

#pragma unroll
  for (int s = 0; s < kStages - 1; ++s) {
    if (s < kSteps) load(s, s);
    cpAsyncCommit();
  }
  for (int k = 0; k < kSteps; ++k) {
    cpAsyncWait<kStages - 2>();
    __syncthreads();
    const int st = k % kStages;
    uint32_t af[2][4], bf[4][2];
#pragma unroll
    for (int mi = 0; mi < 2; ++mi) {
      const __nv_bfloat16* p = &sA[st][(wm * 32 + mi * 16 + (lane & 15)) * kLds + (lane >> 4) * 8];
      ldmatrixX4(af[mi][0], af[mi][1], af[mi][2], af[mi][3], p);
    }
#pragma unroll
    for (int nj = 0; nj < 2; ++nj) {
      const int nrow = wn * 32 + nj * 16 + (lane & 7) + ((lane >> 4) << 3);
      const __nv_bfloat16* p = &sB[st][nrow * kLds + ((lane >> 3) & 1) * 8];
      ldmatrixX4(bf[2 * nj][0], bf[2 * nj][1], bf[2 * nj + 1][0], bf[2 * nj + 1][1], p);
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) mma16816(acc[mi][ni], af[mi], bf[ni]);
    const int kn = k + kStages - 1;
    if (kn < kSteps) load(kn % kStages, kn);
    cpAsyncCommit();
  }
  cpAsyncWait<0>();
  // epilogue: bias, ReLU, mask, store
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int p = m0 + wm * 32 + mi * 16 + (lane >> 2) + half * 8;
      if (p >= P) continue;
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        const int co = n0 + wn * 32 + ni * 8 + 2 * (lane & 3);
        if (co >= a.Cout) continue;
        float v0 = acc[mi][ni][2 * half], v1 = acc[mi][ni][2 * half + 1];
        if (a.bias) {
          v0 += a.bias[co];
          v1 += a.bias[co + 1];
        }
        if (a.relu) {
          v0 = fmaxf(v0, 0.0f);
          v1 = fmaxf(v1, 0.0f);
        }
        if (a.mask) {
          const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162*>(a.mask + size_t(p) * a.Cout + co);
          if (!(__bfloat162float(m.x) > 0.0f)) v0 = 0.0f;
          if (!(__bfloat162float(m.y) > 0.0f)) v1 = 0.0f;
        }
        if (a.outF32) {
          float2* o = reinterpret_cast<float2*>(static_cast<float*>(a.out) + size_t(p) * a.Cout + co);
          *o = make_float2(v0, v1);
        } else {
          __nv_bfloat162* o =
              reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(a.out) + size_t(p) * a.Cout + co);
          *o = __floats2bfloat162_rn(v0, v1);
        }
      }
    }
}

struct WgradArgs {
  const __nv_bfloat16* dz;  // [P][Cout]
  const __nv_bfloat16* x;   // [P][Cin]
  float* dw;                // [Cout][9][Cin], accumulated
  int N, H, W, Cin, Cout;
  int pixelsPerBlock;
};

constexpr int kWBK = 32;  // pixels per K step
constexpr int kWLds = 72;  // smem row stride in halves for 64-wide rows (144 B)

// dW[co][tap][ci] += sum_p dz[p][co] * x[p + off(tap)][ci]
__global__ void __launch_bounds__(256) k_conv3x3_wgrad(WgradArgs a) {
  __shared__ __align__(16) __nv_bfloat16 sA[2][kWBK * kWLds];  // [k = pixel][m = co]
  __shared__ __align__(16) __nv_bfloat16 sB[2][kWBK * kWLds];  // [k = pixel][n = ci]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 1, wn = warp >> 1;  // 2 x 4 warps of 32 x 16
  const int P = a.N * a.H * a.W;
  const int co0 = blockIdx.x * 64;
  const int tap = blockIdx.y % 9, ci0 = (blockIdx.y / 9) * 64;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int pBegin = blockIdx.z * a.pixelsPerBlock;
  const int pEnd = min(P, pBegin + a.pixelsPerBlock);
  // loads: 32 pixel rows x 64 channels = 256 x 16 B for each operand
  const int lr = tid >> 3, lc = (tid & 7) * 8;
  auto load = [&](int buf, int p0) {
    const int p = p0 + lr;
    // A: dz row
    const bool vaRow = p < pEnd && co0 + lc < a.Cout;
    cpAsync16(&sA[buf][lr * kWLds + lc], vaRow ? a.dz + size_t(p) * a.Cout + co0 + lc : a.dz, vaRow);
    // B: shifted x row
    bool vb = p < pEnd && ci0 + lc < a.Cin;
    const __nv_bfloat16* src = a.x;
    if (vb) {
      const int n = p / (a.H * a.W), rem = p - n * a.H * a.W;
      const int y = rem / a.W + dy, xx = rem % a.W + dx;
      vb = y >= 0 && y < a.H && xx >= 0 && xx < a.W;
      if (vb) src = a.x + ((size_t(n) * a.H + y) * a.W + xx) * a.Cin + ci0 + lc;
    }
    cpAsync16(&sB[buf][lr * kWLds + lc], src, vb);
  };
  float acc[2][2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.0f;
  int buf = 0;
  if (pBegin < pEnd) load(0, pBegin);
  cpAsyncCommit();
  for (int p0 = pBegin; p0 < pEnd; p0 += kWBK) {
    if (p0 + kWBK < pEnd) load(buf ^ 1, p0 + kWBK);
    cpAsyncCommit();
    cpAsyncWait<1>();
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kWBK; ks += 16) {
      uint32_t af[2][4], bf[2][2];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
        const int krow = ks + (lane & 7) + ((lane >> 4) << 3);
        const int mcol = wm * 32 + mi * 16 + ((lane >> 3) & 1) * 8;
        ldmatrixX4T(af[mi][0], af[mi][1], af[mi][2], af[mi][3], &sA[buf][krow * kWLds + mcol]);
      }
      {
        const int krow = ks + (lane & 7) + (((lane >> 3) & 1) << 3);
        const int ncol = wn * 16 + (lane >> 4) * 8;
        ldmatrixX4T(bf[0][0], bf[0][1], bf[1][0], bf[1][1], &sB[buf][krow * kWLds + ncol]);
      }
#pragma unroll
      for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 2; ++ni) mma16816(acc[mi][ni], af[mi], bf[ni]);
    }
    __syncthreads();
    buf ^= 1;
  }
  cpAsyncWait<0>();
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int co = co0 + wm * 32 + mi * 16 + (lane >> 2) + half * 8;
      if (co >= a.Cout) continue;
#pragma unroll
      for (int ni = 0; ni < 2; ++ni) {
        const int ci = ci0 + wn * 16 + ni * 8 + 2 * (lane & 3);
        if (ci >= a.Cin) continue;
        float* d = a.dw + (size_t(co) * 9 + tap) * a.Cin + ci;
        atomicAdd(d, acc[mi][ni][2 * half]);
        atomicAdd(d + 1, acc[mi][ni][2 * half + 1]);
      }
    }
}

// db[c] += sum_p dz[p][c]
__global__ void k_bias_grad(const __nv_bfloat16* dz, float* db, int P, int C) {
  const int c = threadIdx.x;  // blockDim.x == C (<= 256)
  float s = 0.0f;
  for (int p = blockIdx.x; p < P; p += gridDim.x) s += __bfloat162float(dz[size_t(p) * C + c]);
  atomicAdd(&db[c], s);
}

// W'[ci][8 - tap][co] = W[co][tap][ci]  (weights of the input-gradient convolution)
__global__ void k_flip_weights(const __nv_bfloat16* w, __nv_bfloat16* wt, int Cout, int Cin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Cout * 9 * Cin) return;
  const int ci = i % Cin, tap = (i / Cin) % 9, co = i / (9 * Cin);
  wt[(size_t(ci) * 9 + (8 - tap)) * Cout + co] = w[i];
}

__global__ void k_avgpool2(const __nv_bfloat16* in, __nv_bfloat16* out, int N, int H, int W, int C) {
  const int Ho = H / 2, Wo = W / 2;
  const size_t total = size_t(N) * Ho * Wo * C;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int c = int(i % C);
    size_t q = i / C;
    const int x = int(q % Wo), y = int((q / Wo) % Ho), n = int(q / (size_t(Wo) * Ho));
    const __nv_bfloat16* b = in + ((size_t(n) * H + 2 * y) * W + 2 * x) * C + c;
    const float s = __bfloat162float(b[0]) + __bfloat162float(b[C]) + __bfloat162float(b[size_t(W) * C]) +
                    __bfloat162float(b[size_t(W) * C + C]);
    out[i] = __float2bfloat16(0.25f * s);
  }
}

// din (+)= 0.25 * dout broadcast to the 2x2 window (accumulate: add to din)
__global__ void k_avgpool2_bwd(const __nv_bfloat16* dout, __nv_bfloat16* din, int N, int H, int W, int C,
                               int accumulate) {
  const size_t total = size_t(N) * H * W * C;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int c = int(i % C);
    size_t q = i / C;
    const int x = int(q % W), y = int((q / W) % H), n = int(q / (size_t(W) * H));
    const float g = 0.25f * __bfloat162float(dout[((size_t(n) * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c]);
    din[i] = __float2bfloat16(accumulate ? __bfloat162float(din[i]) + g : g);
  }
}

// out[..][cOff + c] = in[y/2][x/2][c]  (nearest x2 into a wider channel buffer)
__global__ void k_upsample2(const __nv_bfloat16* in, __nv_bfloat16* out, int N, int H, int W, int C, int Ctot,
                            int cOff) {
  const size_t total = size_t(N) * H * W * C;  // H, W of the output
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int c = int(i % C);
    size_t q = i / C;
    const int x = int(q % W), y = int((q / W) % H), n = int(q / (size_t(W) * H));
    out[q * Ctot + cOff + c] = in[((size_t(n) * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c];
  }
}

// din[y][x][c] = sum over the 2x2 children of dout[..][cOff + c]
__global__ void k_upsample2_bwd(const __nv_bfloat16* dout, __nv_bfloat16* din, int N, int H, int W, int C, int Ctot,
                                int cOff) {
  const size_t total = size_t(N) * H * W * C;  // H, W of the (small) input
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int c = int(i % C);
    size_t q = i / C;
    const int x = int(q % W), y = int((q / W) % H), n = int(q / (size_t(W) * H));
    const size_t W2 = size_t(2 * W);
    const __nv_bfloat16* b = dout + ((size_t(n) * 2 * H + 2 * y) * W2 + 2 * x) * Ctot + cOff + c;
    const float s = __bfloat162float(b[0]) + __bfloat162float(b[Ctot]) + __bfloat162float(b[W2 * Ctot]) +
                    __bfloat162float(b[W2 * Ctot + Ctot]);
    din[i] = __float2bfloat16(s);
  }
}

// dst[p][dOff + c] (+)= src[p][sOff + c] for c < C
__global__ void k_copy_channels(const __nv_bfloat16* src, int Csrc, int sOff, __nv_bfloat16* dst, int Cdst, int dOff,
                                int C, size_t P, int accumulate) {
  const size_t total = P * C;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const size_t p = i / C;
    const int c = int(i % C);
    const float v = __bfloat162float(src[p * Csrc + sOff + c]);
    __nv_bfloat16& d = dst[p * Cdst + dOff + c];
    d = __float2bfloat16(accumulate ? __bfloat162float(d) + v : v);
  }
}

// The same five layout operations on 8-channel (16-byte) chunks, for
// channel counts and offsets that are multiples of 8 and 16-byte aligned
// buffers; I is the index type (32-bit when every buffer has fewer than 2^32
// chunks).  Per element they compute what the scalar kernels above do, in
// the same order, with no contraction into fused multiply-adds.
struct Bf8 {
  float v[8];
};
__device__ __forceinline__ Bf8 unpack8(uint4 u) {
  Bf8 r;
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float2 f = __bfloat1622float2(h[i]);
    r.v[2 * i] = f.x;
    r.v[2 * i + 1] = f.y;
  }
  return r;
}
__device__ __forceinline__ uint4 pack8(const Bf8& r) {
  uint4 u;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(r.v[2 * i], r.v[2 * i + 1]);
  return u;
}

template <typename I>
__global__ void k_avgpool2_v(const uint4* in, uint4* out, I N, I H, I W, I C8) {
  const I Ho = H / 2, Wo = W / 2, total = N * Ho * Wo * C8;
  for (I i = I(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += I(gridDim.x) * blockDim.x) {
    const I c = i % C8, q = i / C8, x = q % Wo, t = q / Wo, y = t % Ho, n = t / Ho;
    const uint4* b = in + ((n * H + 2 * y) * W + 2 * x) * C8 + c;
    const Bf8 a0 = unpack8(__ldg(b)), a1 = unpack8(__ldg(b + C8)), a2 = unpack8(__ldg(b + W * C8)),
              a3 = unpack8(__ldg(b + W * C8 + C8));
    Bf8 r;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.v[k] = __fmul_rn(0.25f, __fadd_rn(__fadd_rn(__fadd_rn(a0.v[k], a1.v[k]), a2.v[k]), a3.v[k]));
    out[i] = pack8(r);
  }
}

template <typename I>
__global__ void k_avgpool2_bwd_v(const uint4* dout, uint4* din, I N, I H, I W, I C8, int accumulate) {
  const I total = N * H * W * C8;
  for (I i = I(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += I(gridDim.x) * blockDim.x) {
    const I c = i % C8, q = i / C8, x = q % W, t = q / W, y = t % H, n = t / H;
    const Bf8 g = unpack8(__ldg(&dout[((n * (H / 2) + y / 2) * (W / 2) + x / 2) * C8 + c]));
    Bf8 r;
    if (accumulate) {
      const Bf8 o = unpack8(din[i]);
#pragma unroll
      for (int k = 0; k < 8; ++k) r.v[k] = __fadd_rn(o.v[k], __fmul_rn(0.25f, g.v[k]));
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) r.v[k] = __fmul_rn(0.25f, g.v[k]);
    }
    din[i] = pack8(r);
  }
}

template <typename I>
__global__ void k_upsample2_v(const uint4* in, uint4* out, I N, I H, I W, I C8, I Ct8, I cOff8) {
  const I total = N * H * W * C8;  // H, W of the output
  for (I i = I(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += I(gridDim.x) * blockDim.x) {
    const I c = i % C8, q = i / C8, x = q % W, t = q / W, y = t % H, n = t / H;
    out[q * Ct8 + cOff8 + c] = __ldg(&in[((n * (H / 2) + y / 2) * (W / 2) + x / 2) * C8 + c]);
  }
}

template <typename I>
__global__ void k_upsample2_bwd_v(const uint4* dout, uint4* din, I N, I H, I W, I C8, I Ct8, I cOff8) {
  const I total = N * H * W * C8;  // H, W of the (small) input
  for (I i = I(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += I(gridDim.x) * blockDim.x) {
    const I c = i % C8, q = i / C8, x = q % W, t = q / W, y = t % H, n = t / H;
    const I W2 = 2 * W;
    const uint4* b = dout + ((n * 2 * H + 2 * y) * W2 + 2 * x) * Ct8 + cOff8 + c;
    const Bf8 a0 = unpack8(__ldg(b)), a1 = unpack8(__ldg(b + Ct8)), a2 = unpack8(__ldg(b + W2 * Ct8)),
              a3 = unpack8(__ldg(b + W2 * Ct8 + Ct8));
    Bf8 r;
#pragma unroll
    for (int k = 0; k < 8; ++k) r.v[k] = __fadd_rn(__fadd_rn(__fadd_rn(a0.v[k], a1.v[k]), a2.v[k]), a3.v[k]);
    din[i] = pack8(r);
  }
}

template <typename I>
__global__ void k_copy_channels_v(const uint4* src, I Cs8, I sOff8, uint4* dst, I Cd8, I dOff8, I C8, I P,
                                  int accumulate) {
  const I total = P * C8;
  for (I i = I(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += I(gridDim.x) * blockDim.x) {
    const I p = i / C8, c = i % C8;
    const uint4 v = __ldg(&src[p * Cs8 + sOff8 + c]);
    uint4& d = dst[p * Cd8 + dOff8 + c];
    if (accumulate) {
      const Bf8 a = unpack8(d), b = unpack8(v);
      Bf8 r;
#pragma unroll
      for (int k = 0; k < 8; ++k) r.v[k] = __fadd_rn(a.v[k], b.v[k]);
      d = pack8(r);
    } else {
      d = v;
    }
  }
}

// decoder input in one pass: out[p] = (up2(low)[p] channels 0..Cu, skip[p]
// channels 0..Cs); every chunk of out written once, in order
template <typename I>
__global__ void k_upsample_concat_v(const uint4* low, const uint4* skip, uint4* out, I N, I H, I W, I Cu8, I Cs8) {
  const I Ct8 = Cu8 + Cs8, total = N * H * W * Ct8;
  for (I i = I(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += I(gridDim.x) * blockDim.x) {
    const I c = i % Ct8, q = i / Ct8;
    uint4 v;
    if (c < Cu8) {
      const I x = q % W, t = q / W, y = t % H, n = t / H;
      v = __ldg(&low[((n * (H / 2) + y / 2) * (W / 2) + x / 2) * Cu8 + c]);
    } else {
      v = __ldg(&skip[q * Cs8 + (c - Cu8)]);
    }
    out[i] = v;
  }
}

// Network input: log1p(radiance), albedo, normal, log2(1 + filter-weight
// sum) / 16 (the sample count: how much noise there is to remove), the
// per-pixel noise as log1p of the mean over rgb of the input radiance's
// standard-deviation estimate, and a flag that the noise is known (1) or
// not (0, no estimate given); zeros up to C; pixels outside the h x w image
// (padding up to hp x wp) are zero.
__global__ void k_prep_input(const float4* rad, const float4* alb, const float4* nrm, const float4* wsum,
                             const float4* noise, __nv_bfloat16* out, int n, int h, int w, int hp, int wp, int C) {
  const size_t P = size_t(n) * hp * wp;
  for (size_t q = blockIdx.x * size_t(blockDim.x) + threadIdx.x; q < P; q += size_t(gridDim.x) * blockDim.x) {
    const int x = int(q % wp), y = int((q / wp) % hp), b = int(q / (size_t(wp) * hp));
    float v[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (y < h && x < w) {
      const size_t p = (size_t(b) * h + y) * w + x;
      const float4 r = rad[p];
      v[0] = log1pf(fmaxf(r.x, 0.0f));
      v[1] = log1pf(fmaxf(r.y, 0.0f));
      v[2] = log1pf(fmaxf(r.z, 0.0f));
      if (alb) {
        const float4 a = alb[p];
        v[3] = a.x;
        v[4] = a.y;
        v[5] = a.z;
      }
      if (nrm) {
        const float4 m = nrm[p];
        v[6] = m.x;
        v[7] = m.y;
        v[8] = m.z;
      }
      if (wsum) v[9] = log2f(1.0f + fmaxf(wsum[p].x, 0.0f)) * 0.0625f;
      if (noise) {
        const float4 e = noise[p];
        v[10] = log1pf(fmaxf((e.x + e.y + e.z) * (1.0f / 3.0f), 0.0f));
        v[11] = 1.0f;
      }
    }
    __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(out + q * C);
    for (int c = 0; c < C; c += 2)
      o[c / 2] = __floats2bfloat162_rn(c < 12 ? v[c] : 0.0f, c + 1 < 12 ? v[c + 1] : 0.0f);
  }
}

// Noise estimates from two independent half renders a, b of one shot:
// per channel |a - b| / sqrt(2) for either half alone and |a - b| / 2 for
// their average (the standard deviation of a difference of two equal-noise
// estimates is sqrt(2) times either's).
__global__ void k_half_noise(const float4* a, const float4* b, float4* half, float4* all, size_t P) {
  for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < P; p += size_t(gridDim.x) * blockDim.x) {
    const float4 x = a[p], y = b[p];
    const float d[3] = {fabsf(x.x - y.x), fabsf(x.y - y.y), fabsf(x.z - y.z)};
    if (half) half[p] = make_float4(d[0] * 0.70710678f, d[1] * 0.70710678f, d[2] * 0.70710678f, 0.0f);
    if (all) all[p] = make_float4(d[0] * 0.5f, d[1] * 0.5f, d[2] * 0.5f, 0.0f);
  }
}

// L1 loss on log radiance with the residual connection:
//   y_c = head_c + log1p(rad_c),  loss += |y_c - log1p(target_c)|  (c < 3)
// and its gradient with respect to head (sign / count; zero elsewhere).
__global__ void k_l1_loss(const float* head, int C, const float4* rad, const float4* target, __nv_bfloat16* grad,
                          int n, int h, int w, int hp, int wp, float invCount, float* loss) {
  const size_t P = size_t(n) * hp * wp;
  float s = 0.0f;
  for (size_t q = blockIdx.x * size_t(blockDim.x) + threadIdx.x; q < P; q += size_t(gridDim.x) * blockDim.x) {
    const int x = int(q % wp), y = int((q / wp) % hp), b = int(q / (size_t(wp) * hp));
    float g[3] = {0.0f, 0.0f, 0.0f};
    if (y < h && x < w) {
      const size_t p = (size_t(b) * h + y) * w + x;
      const float4 r = rad[p], t = target[p];
      const float rr[3] = {r.x, r.y, r.z}, tt[3] = {t.x, t.y, t.z};
      for (int c = 0; c < 3; ++c) {
        const float d = head[q * C + c] + log1pf(fmaxf(rr[c], 0.0f)) - log1pf(fmaxf(tt[c], 0.0f));
        s += fabsf(d);
        g[c] = d > 0.0f ? invCount : (d < 0.0f ? -invCount : 0.0f);
      }
    }
    __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(grad + q * C);
    o[0] = __floats2bfloat162_rn(g[0], g[1]);
    o[1] = __floats2bfloat162_rn(g[2], 0.0f);
    for (int c = 4; c < C; c += 2) o[c / 2] = __floats2bfloat162_rn(0.0f, 0.0f);
  }
  for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

// Relative squared error on radiance with the denominator held fixed (the
// "relMSE" of Lehtinen et al., Noise2Noise, ICML 2018, section 3.4):
// L = mean (o - t)^2 / (sg(o) + 0.01)^2, o = max(expm1(head + log1p(r)), 0).
// Its minimiser is the target's mean, so noisy targets add no bias (an L1
// loss converges to the median, which sits below the mean of right-skewed
// radiance noise).  dL/dhead = 2 (o - t) (o + 1) / (o + 0.01)^2 where o > 0.
__global__ void k_relmse_loss(const float* head, int C, const float4* rad, const float4* target,
                              __nv_bfloat16* grad, int n, int h, int w, int hp, int wp, float invCount, float* loss) {
  const size_t P = size_t(n) * hp * wp;
  float s = 0.0f;
  for (size_t q = blockIdx.x * size_t(blockDim.x) + threadIdx.x; q < P; q += size_t(gridDim.x) * blockDim.x) {
    const int x = int(q % wp), y = int((q / wp) % hp), b = int(q / (size_t(wp) * hp));
    float g[3] = {0.0f, 0.0f, 0.0f};
    if (y < h && x < w) {
      const size_t p = (size_t(b) * h + y) * w + x;
      const float4 r = rad[p], t = target[p];
      const float rr[3] = {r.x, r.y, r.z}, tt[3] = {t.x, t.y, t.z};
      for (int c = 0; c < 3; ++c) {
        const float e = expm1f(head[q * C + c] + log1pf(fmaxf(rr[c], 0.0f)));
        const float o = fmaxf(e, 0.0f);
        const float den = 1.0f / ((o + 0.01f) * (o + 0.01f));
        const float d = o - fmaxf(tt[c], 0.0f);
        s += d * d * den;
        g[c] = e > 0.0f ? 2.0f * d * (e + 1.0f) * den * invCount : 0.0f;
      }
    }
    __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(grad + q * C);
    o[0] = __floats2bfloat162_rn(g[0], g[1]);
    o[1] = __floats2bfloat162_rn(g[2], 0.0f);
    for (int c = 4; c < C; c += 2) o[c / 2] = __floats2bfloat162_rn(0.0f, 0.0f);
  }
  for (int off = 16; off; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

// radiance = max(expm1(head + log1p(rad)), 0), alpha 1
__global__ void k_output(const float* head, int C, const float4* rad, float4* out, int n, int h, int w, int hp,
                         int wp) {
  const size_t P = size_t(n) * h * w;
  for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < P; p += size_t(gridDim.x) * blockDim.x) {
    const int x = int(p % w), y = int((p / w) % h), b = int(p / (size_t(w) * h));
    const size_t q = (size_t(b) * hp + y) * wp + x;
    const float4 r = rad[p];
    out[p] = make_float4(fmaxf(expm1f(head[q * C] + log1pf(fmaxf(r.x, 0.0f))), 0.0f),
                         fmaxf(expm1f(head[q * C + 1] + log1pf(fmaxf(r.y, 0.0f))), 0.0f),
                         fmaxf(expm1f(head[q * C + 2] + log1pf(fmaxf(r.z, 0.0f))), 0.0f), 1.0f);
  }
}

// grad *= (y > 0)
__global__ void k_relu_mask(__nv_bfloat16* g, const __nv_bfloat16* y, size_t count) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < count; i += size_t(gridDim.x) * blockDim.x)
    if (!(__bfloat162float(y[i]) > 0.0f)) g[i] = __float2bfloat16(0.0f);
}

// sums[0] += sum (d - b)^2, sums[1] += sum (a - b)^2 over RGB
__global__ void k_err_sums(const float4* d, const float4* a, const float4* b, size_t P, double* sums) {
  float s0 = 0.0f, s1 = 0.0f;
  for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < P; p += size_t(gridDim.x) * blockDim.x) {
    const float4 dv = d[p], av = a[p], bv = b[p];
    s0 += (dv.x - bv.x) * (dv.x - bv.x) + (dv.y - bv.y) * (dv.y - bv.y) + (dv.z - bv.z) * (dv.z - bv.z);
    s1 += (av.x - bv.x) * (av.x - bv.x) + (av.y - bv.y) * (av.y - bv.y) + (av.z - bv.z) * (av.z - bv.z);
  }
  for (int off = 16; off; off >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, off);
    s1 += __shfl_down_sync(0xffffffffu, s1, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&sums[0], double(s0));
    atomicAdd(&sums[1], double(s1));
  }
}

// sums of |D_A - D_B|^2 (two denoised halves) and the combined input of
// both films: radiance (A + B) / 2, weight A + B
__global__ void k_combine(const float4* da, const float4* db, const float4* a, const float4* b, const float4* wa,
                          const float4* wb, float4* rad, float4* wsum, size_t P, double* sums) {
  float s0 = 0.0f;
  for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < P; p += size_t(gridDim.x) * blockDim.x) {
    const float4 x = da[p], y = db[p], av = a[p], bv = b[p], w0 = wa[p], w1 = wb[p];
    s0 += (x.x - y.x) * (x.x - y.x) + (x.y - y.y) * (x.y - y.y) + (x.z - y.z) * (x.z - y.z);
    rad[p] = make_float4(0.5f * (av.x + bv.x), 0.5f * (av.y + bv.y), 0.5f * (av.z + bv.z), 1.0f);
    wsum[p] = make_float4(w0.x + w1.x, w0.y + w1.y, w0.z + w1.z, w0.w + w1.w);
  }
  for (int off = 16; off; off >>= 1) s0 += __shfl_down_sync(0xffffffffu, s0, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(&sums[2], double(s0));
}

// Sums for the blend of the denoised and plain images (rgb, over pixels):
// with da, db the denoised halves and a, b the halves' radiance,
//   [3] (da - b)^2   [4] (da - b)(a - b)   [5] (a - b)^2
//   [6] (da - db)^2  [7] (da - db)(a - b)
// and the input of the all-sample denoise: radiance (a + b) / 2, weight a + b.
__global__ void k_blend_sums(const float4* da, const float4* db, const float4* a, const float4* b, const float4* wa,
                             const float4* wb, float4* rad, float4* wsum, size_t P, double* sums) {
  float s[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < P; p += size_t(gridDim.x) * blockDim.x) {
    const float4 x = da[p], y = db[p], av = a[p], bv = b[p], w0 = wa[p], w1 = wb[p];
    const float xb[3] = {x.x - bv.x, x.y - bv.y, x.z - bv.z}, ab[3] = {av.x - bv.x, av.y - bv.y, av.z - bv.z};
    const float xy[3] = {x.x - y.x, x.y - y.y, x.z - y.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      s[0] += xb[c] * xb[c];
      s[1] += xb[c] * ab[c];
      s[2] += ab[c] * ab[c];
      s[3] += xy[c] * xy[c];
      s[4] += xy[c] * ab[c];
    }
    rad[p] = make_float4(0.5f * (av.x + bv.x), 0.5f * (av.y + bv.y), 0.5f * (av.z + bv.z), 1.0f);
    wsum[p] = make_float4(w0.x + w1.x, w0.y + w1.y, w0.z + w1.z, w0.w + w1.w);
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    float v = s[k];
    for (int off = 16; off; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(&sums[3 + k], double(v));
  }
}

// out = w out + (1 - w) (a + b) / 2 on rgb; alpha 1
__global__ void k_blend(float4* out, const float4* a, const float4* b, float w, size_t P) {
  for (size_t p = blockIdx.x * size_t(blockDim.x) + threadIdx.x; p < P; p += size_t(gridDim.x) * blockDim.x) {
    const float4 o = out[p], av = a[p], bv = b[p];
    const float v = 1.0f - w;
    out[p] = make_float4(w * o.x + v * (0.5f * (av.x + bv.x)), w * o.y + v * (0.5f * (av.y + bv.y)),
                         w * o.z + v * (0.5f * (av.z + bv.z)), 1.0f);
  }
}

// Adam on fp32 master weights; writes the bf16 copy used by the kernels.
__global__ void k_adam(float* w, float* m, float* v, const float* g, __nv_bfloat16* wb, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16(wi);
  }
}

__global__ void k_f32_to_bf16(const float* a, __nv_bfloat16* b, size_t n) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    b[i] = __float2bfloat16(a[i]);
}

int grid1d(size_t n, int block = 256) {
  size_t g = (n + block - 1) / block;
  return int(g > 65535 * 4 ? 65535 * 4 : (g < 1 ? 1 : g));
}

}  // namespace
}  // namespace nn
}  // namespace asuna

using namespace asuna;
using namespace asuna::nn;

#define NN_CHECK_LAUNCH()                                                                          \
  do {                                                                                             \
    cudaError_t e_ = cudaGetLastError();                                                           \
    if (e_ != cudaSuccess) return fail(ASUNA_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
    return ASUNA_OK;                                                                               \
  } while (0)

namespace {
bool al16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
// the chunked kernels: channel counts and offsets multiples of 8, 16-byte
// bases; chunks = the largest buffer's 16-byte count (32-bit indexing below 2^32)
bool vec8(std::initializer_list<int> chans, std::initializer_list<const void*> ptrs) {
  for (int c : chans)
    if (c % 8) return false;
  for (const void* p : ptrs)
    if (!al16(p)) return false;
  return true;
}
bool small32(size_t chunks) { return chunks < (size_t(1) << 32); }
#define NN_LAUNCH_V(KERNEL, COUNT, CHUNKS, ...)                                                              \
  do {                                                                                                      \
    if (small32(CHUNKS))                                                                                    \
      KERNEL<uint32_t><<<grid1d(COUNT), 256, 0, static_cast<cudaStream_t>(stream)>>>(__VA_ARGS__);         \
    else                                                                                                    \
      KERNEL<size_t><<<grid1d(COUNT), 256, 0, static_cast<cudaStream_t>(stream)>>>(__VA_ARGS__);           \
  } while (0)
}  // namespace

extern "C" {

int asuna_nn_conv3x3(void* stream, const void* in, int n, int h, int w, int cin, const void* weight, const float* bias,
                     int cout, int relu, const void* mask, void* out, int out_f32) {
  clearError();
  if (!in || !weight || !out || n <= 0 || h <= 0 || w <= 0 || cin <= 0 || cout <= 0)
    return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3: bad argument");
  if (cin % 16 || cout % 8) return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3: cin %% 16 and cout %% 8 must be 0");
  ConvArgs a{static_cast<const __nv_bfloat16*>(in), static_cast<const __nv_bfloat16*>(weight), bias,
             static_cast<const __nv_bfloat16*>(mask), out, n, h, w, cin, cout, relu, out_f32};
  const int P = n * h * w;
  dim3 g((P + kBM - 1) / kBM, (cout + kBN - 1) / kBN);
  k_conv3x3<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  NN_CHECK_LAUNCH();
}

int asuna_nn_conv3x3_wgrad(void* stream, const void* dz, const void* x, int n, int h, int w, int cin, int cout,
                           float* dweight) {
  clearError();
  if (!dz || !x || !dweight || cin % 16 || cout % 8) return fail(ASUNA_ERR_INVALID, "asuna_nn_conv3x3_wgrad: bad argument");
  const int P = n * h * w;
  const int chunk = 2048;
  WgradArgs a{static_cast<const __nv_bfloat16*>(dz), static_cast<const __nv_bfloat16*>(x), dweight, n, h, w, cin, cout,
              chunk};
  dim3 g((cout + 63) / 64, 9 * ((cin + 63) / 64), (P + chunk - 1) / chunk);
  k_conv3x3_wgrad<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(a);
  NN_CHECK_LAUNCH();
}

int asuna_nn_bias_grad(void* stream, const void* dz, int pixels, int c, float* dbias) {
  if (!dz || !dbias || c > 256) return fail(ASUNA_ERR_INVALID, "asuna_nn_bias_grad: bad argument");
  k_bias_grad<<<std::min(pixels, 2048), c, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(dz), dbias, pixels, c);
  NN_CHECK_LAUNCH();
}

int asuna_nn_flip_weights(void* stream, const void* w, void* wt, int cout, int cin) {
  k_flip_weights<<<grid1d(size_t(cout) * 9 * cin), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(w), static_cast<__nv_bfloat16*>(wt), cout, cin);
  NN_CHECK_LAUNCH();
}


int asuna_nn_avgpool2(void* stream, const void* in, void* out, int n, int h, int w, int c) {
  if (vec8({c}, {in, out})) {
    const size_t chunks = size_t(n) * h * w * (c / 8);
    NN_LAUNCH_V(k_avgpool2_v, chunks / 4, chunks, static_cast<const uint4*>(in), static_cast<uint4*>(out), n, h, w,
                c / 8);
    NN_CHECK_LAUNCH();
  }
  k_avgpool2<<<grid1d(size_t(n) * h * w * c / 4), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(in), static_cast<__nv_bfloat16*>(out), n, h, w, c);
  NN_CHECK_LAUNCH();
}

int asuna_nn_avgpool2_bwd(void* stream, const void* dout, void* din, int n, int h, int w, int c, int accumulate) {
  if (vec8({c}, {dout, din})) {
    const size_t chunks = size_t(n) * h * w * (c / 8);
    NN_LAUNCH_V(k_avgpool2_bwd_v, chunks, chunks, static_cast<const uint4*>(dout), static_cast<uint4*>(din), n, h,
                w, c / 8, accumulate);
    NN_CHECK_LAUNCH();
  }
  k_avgpool2_bwd<<<grid1d(size_t(n) * h * w * c), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(dout), static_cast<__nv_bfloat16*>(din), n, h, w, c, accumulate);
  NN_CHECK_LAUNCH();
}

int asuna_nn_upsample2(void* stream, const void* in, void* out, int n, int h, int w, int c, int ctot, int coff) {
  if (vec8({c, ctot, coff}, {in, out})) {
    const size_t chunks = size_t(n) * h * w * (ctot / 8);
    NN_LAUNCH_V(k_upsample2_v, size_t(n) * h * w * (c / 8), chunks, static_cast<const uint4*>(in),
                static_cast<uint4*>(out), n, h, w, c / 8, ctot / 8, coff / 8);
    NN_CHECK_LAUNCH();
  }
  k_upsample2<<<grid1d(size_t(n) * h * w * c), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(in), static_cast<__nv_bfloat16*>(out), n, h, w, c, ctot, coff);
  NN_CHECK_LAUNCH();
}

int asuna_nn_upsample2_bwd(void* stream, const void* dout, void* din, int n, int h, int w, int c, int ctot, int coff) {
  if (vec8({c, ctot, coff}, {dout, din})) {
    const size_t chunks = size_t(n) * 4 * h * w * (ctot / 8);
    NN_LAUNCH_V(k_upsample2_bwd_v, size_t(n) * h * w * (c / 8), chunks, static_cast<const uint4*>(dout),
                static_cast<uint4*>(din), n, h, w, c / 8, ctot / 8, coff / 8);
    NN_CHECK_LAUNCH();
  }
  k_upsample2_bwd<<<grid1d(size_t(n) * h * w * c), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(dout), static_cast<__nv_bfloat16*>(din), n, h, w, c, ctot, coff);
  NN_CHECK_LAUNCH();
}

int asuna_nn_copy_channels(void* stream, const void* src, int csrc, int soff, void* dst, int cdst, int doff, int c,
                           uint64_t pixels, int accumulate) {
  if (vec8({csrc, soff, cdst, doff, c}, {src, dst})) {
    const size_t chunks = size_t(pixels) * (std::max(csrc, cdst) / 8);
    NN_LAUNCH_V(k_copy_channels_v, size_t(pixels) * (c / 8), chunks, static_cast<const uint4*>(src), csrc / 8,
                soff / 8, static_cast<uint4*>(dst), cdst / 8, doff / 8, c / 8, pixels, accumulate);
    NN_CHECK_LAUNCH();
  }
  k_copy_channels<<<grid1d(pixels * c), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(src), csrc, soff, static_cast<__nv_bfloat16*>(dst), cdst, doff, c, pixels,
      accumulate);
  NN_CHECK_LAUNCH();
}

int asuna_nn_relu_mask(void* stream, void* grad, const void* y, uint64_t count) {
  k_relu_mask<<<grid1d(count), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<__nv_bfloat16*>(grad), static_cast<const __nv_bfloat16*>(y), count);
  NN_CHECK_LAUNCH();
}

int asuna_nn_f32_to_bf16(void* stream, const float* a, void* b, uint64_t n) {
  k_f32_to_bf16<<<grid1d(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(a, static_cast<__nv_bfloat16*>(b), n);
  NN_CHECK_LAUNCH();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The network object: parameters, Adam state and activation workspace on the
// device; forward, loss + backward and Adam as sequences of the kernels above.

namespace {

struct ConvLayer {
  int cin = 0, cout = 0;
  size_t wOff = 0, bOff = 0;  // offsets (floats) in the parameter arrays
  size_t wtOff = 0;           // offset (halves) of the flipped weights
};

struct LevelBufs {
  __nv_bfloat16 *X = nullptr, *A = nullptr, *S = nullptr, *U = nullptr, *B = nullptr, *D = nullptr;
  __nv_bfloat16 *gX = nullptr, *gA = nullptr, *gS = nullptr, *gU = nullptr, *gB = nullptr, *gD = nullptr;
};

// splitmix64 + Box-Muller: the same initial weights on every host
struct InitRng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double normal() {
    const double u1 = uniform(), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

}  // namespace

struct asuna_denoiser {
  asuna_ctx* ctx = nullptr;  // the stream it runs on; not touched by destroy
  int device = 0;
  int L = 0;
  int ch[ASUNA_DENOISER_MAX_LEVELS] = {};
  bool training = false;
  uint32_t loss = ASUNA_DENOISER_LOSS_L1_LOG;
  uint64_t maxPixels = 0;
  std::vector<ConvLayer> layers;
  size_t nParams = 0, nFlip = 0;
  float *p32 = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *pbf = nullptr, *wt = nullptr;
  bool useTc = false;                                // convolutions on tcgen05
  __nv_bfloat16 *wtc = nullptr, *wtcT = nullptr;     // their weight layouts (forward, input gradient)
  float* dLoss = nullptr;
  double* dSums = nullptr;
  float* head = nullptr;
  __nv_bfloat16* gHead = nullptr;
  LevelBufs lv[ASUNA_DENOISER_MAX_LEVELS];
  std::vector<void*> allocs;
  int step = 0;
  bool flipped = false;

  int enc(int l, int k) const { return 2 * l + k; }
  int dec(int l, int k) const { return 2 * L + 2 * (L - 2 - l) + k; }
  int headIdx() const { return 4 * L - 2; }
  cudaStream_t stream() const { return ctx->stream; }
  ~asuna_denoiser() {
    for (void* p : allocs) cudaFree(p);
  }
};

namespace {

constexpr int kInC = 16, kHeadC = 16;

template <class T>
int dalloc(asuna_denoiser* d, T** p, size_t count) {
  void* q = nullptr;
  if (cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) {
    cudaGetLastError();
    return fail(ASUNA_ERR_OOM, "denoiser: device allocation of %zu bytes failed", count * sizeof(T));
  }
  d->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return ASUNA_OK;
}

#define NN_TRY(x)                  \
  do {                             \
    const int rc_ = (x);           \
    if (rc_ != ASUNA_OK) return rc_; \
  } while (0)

int convFwd(asuna_denoiser* d, int li, const __nv_bfloat16* in, int n, int h, int w, bool relu, void* out, bool f32) {
  const ConvLayer& c = d->layers[li];
  if (d->useTc)
    return asuna_nn_conv3x3_tc(d->stream(), in, n, h, w, c.cin, d->wtc + c.wtOff, d->p32 + c.bOff, c.cout,
                               relu ? 1 : 0, nullptr, out, f32 ? 1 : 0);
  return asuna_nn_conv3x3(d->stream(), in, n, h, w, c.cin, d->pbf + c.wOff, d->p32 + c.bOff, c.cout, relu ? 1 : 0,
                          nullptr, out, f32 ? 1 : 0);
}

// dX of layer li from dz; `mask` (the layer input's own ReLU output) fused
int convDx(asuna_denoiser* d, int li, const __nv_bfloat16* dz, int n, int h, int w, const __nv_bfloat16* mask,
           __nv_bfloat16* dx) {
  const ConvLayer& c = d->layers[li];
  if (d->useTc)
    return asuna_nn_conv3x3_tc(d->stream(), dz, n, h, w, c.cout, d->wtcT + c.wtOff, nullptr, c.cin, 0, mask, dx, 0);
  return asuna_nn_conv3x3(d->stream(), dz, n, h, w, c.cout, d->wt + c.wtOff, nullptr, c.cin, 0, mask, dx, 0);
}

int convDw(asuna_denoiser* d, int li, const __nv_bfloat16* dz, const __nv_bfloat16* x, int n, int h, int w) {
  const ConvLayer& c = d->layers[li];
  NN_TRY(asuna_nn_conv3x3_wgrad(d->stream(), dz, x, n, h, w, c.cin, c.cout, d->grad + c.wOff));
  return asuna_nn_bias_grad(d->stream(), dz, n * h * w, c.cout, d->grad + c.bOff);
}

// weights derived from the bf16 copy: flipped (input gradient) and, for the
// tcgen05 kernels, both in their operand layout
int flipAll(asuna_denoiser* d) {
  if (d->flipped) return ASUNA_OK;
  for (const ConvLayer& c : d->layers) {
    NN_TRY(asuna_nn_flip_weights(d->stream(), d->pbf + c.wOff, d->wt + c.wtOff, c.cout, c.cin));
    if (d->useTc) {
      NN_TRY(asuna_nn_weights_tc(d->stream(), d->pbf + c.wOff, d->wtc + c.wtOff, c.cout, c.cin));
      NN_TRY(asuna_nn_weights_tc(d->stream(), d->wt + c.wtOff, d->wtcT + c.wtOff, c.cin, c.cout));
    }
  }
  d->flipped = true;
  return ASUNA_OK;
}

struct Dims {
  int n, h, w, hp, wp;
};

int dims(const asuna_denoiser* d, uint32_t n, uint32_t h, uint32_t w, Dims& o) {
  if (n == 0 || h == 0 || w == 0) return fail(ASUNA_ERR_INVALID, "denoiser: empty image");
  const uint32_t a = 1u << (d->L - 1);
  o.n = int(n);
  o.h = int(h);
  o.w = int(w);
  o.hp = int((h + a - 1) / a * a);
  o.wp = int((w + a - 1) / a * a);
  if (uint64_t(n) * o.hp * o.wp > d->maxPixels)
    return fail(ASUNA_ERR_INVALID, "denoiser: %u x %d x %d padded pixels exceed max_pixels %llu", n, o.hp, o.wp,
                (unsigned long long)d->maxPixels);
  return ASUNA_OK;
}

// decoder input: the upsampled lower level beside the skip connection
int upsampleConcat(cudaStream_t stream, const __nv_bfloat16* low, const __nv_bfloat16* skip, __nv_bfloat16* out, int n,
                   int h, int w, int cu, int cs, size_t P) {
  if (vec8({cu, cs}, {low, skip, out})) {
    const size_t chunks = P * ((cu + cs) / 8);
    NN_LAUNCH_V(k_upsample_concat_v, chunks, chunks, reinterpret_cast<const uint4*>(low),
                reinterpret_cast<const uint4*>(skip), reinterpret_cast<uint4*>(out), n, h, w, cu / 8, cs / 8);
    NN_CHECK_LAUNCH();
  }
  NN_TRY(asuna_nn_upsample2(stream, low, out, n, h, w, cu, cu + cs, 0));
  return asuna_nn_copy_channels(stream, skip, cs, 0, out, cu + cs, cu, cs, P, 0);
}

int forward(asuna_denoiser* d, const float* rad, const float* alb, const float* nrm, const float* wsum,
            const float* noise, const Dims& D) {
  const int L = d->L;
  cudaStream_t s = d->stream();
  if (d->useTc) NN_TRY(flipAll(d));
  const size_t P0 = size_t(D.n) * D.hp * D.wp;
  k_prep_input<<<grid1d(P0), 256, 0, s>>>(reinterpret_cast<const float4*>(rad), reinterpret_cast<const float4*>(alb),
                                          reinterpret_cast<const float4*>(nrm), reinterpret_cast<const float4*>(wsum),
                                          reinterpret_cast<const float4*>(noise), d->lv[0].X, D.n, D.h, D.w, D.hp,
                                          D.wp, kInC);
  ASUNA_CUDA_TRY(cudaGetLastError());
  for (int l = 0; l < L; ++l) {
    const int hl = D.hp >> l, wl = D.wp >> l;
    LevelBufs& b = d->lv[l];
    if (l > 0) NN_TRY(asuna_nn_avgpool2(s, d->lv[l - 1].S, b.X, D.n, hl * 2, wl * 2, d->ch[l - 1]));
    NN_TRY(convFwd(d, d->enc(l, 0), b.X, D.n, hl, wl, true, b.A, false));
    NN_TRY(convFwd(d, d->enc(l, 1), b.A, D.n, hl, wl, true, b.S, false));
  }
  for (int l = L - 2; l >= 0; --l) {
    const int hl = D.hp >> l, wl = D.wp >> l;
    const size_t Pl = size_t(D.n) * hl * wl;
    LevelBufs& b = d->lv[l];
    const __nv_bfloat16* src = (l == L - 2) ? d->lv[L - 1].S : d->lv[l + 1].D;
    const int cu = d->ch[l + 1], cs = d->ch[l], ct = cu + cs;
    NN_TRY(upsampleConcat(s, src, b.S, b.U, D.n, hl, wl, cu, cs, Pl));
    NN_TRY(convFwd(d, d->dec(l, 0), b.U, D.n, hl, wl, true, b.B, false));
    NN_TRY(convFwd(d, d->dec(l, 1), b.B, D.n, hl, wl, true, b.D, false));
  }
  return convFwd(d, d->headIdx(), d->lv[0].D, D.n, D.hp, D.wp, false, d->head, true);
}

int backward(asuna_denoiser* d, const Dims& D) {
  const int L = d->L;
  cudaStream_t s = d->stream();
  NN_TRY(flipAll(d));
  NN_TRY(convDw(d, d->headIdx(), d->gHead, d->lv[0].D, D.n, D.hp, D.wp));
  NN_TRY(convDx(d, d->headIdx(), d->gHead, D.n, D.hp, D.wp, d->lv[0].D, d->lv[0].gD));
  for (int l = 0; l <= L - 2; ++l) {
    const int hl = D.hp >> l, wl = D.wp >> l;
    const size_t Pl = size_t(D.n) * hl * wl;
    LevelBufs& b = d->lv[l];
    const int cu = d->ch[l + 1], cs = d->ch[l], ct = cu + cs;
    NN_TRY(convDw(d, d->dec(l, 1), b.gD, b.B, D.n, hl, wl));
    NN_TRY(convDx(d, d->dec(l, 1), b.gD, D.n, hl, wl, b.B, b.gB));
    NN_TRY(convDw(d, d->dec(l, 0), b.gB, b.U, D.n, hl, wl));
    NN_TRY(convDx(d, d->dec(l, 0), b.gB, D.n, hl, wl, nullptr, b.gU));
    NN_TRY(asuna_nn_copy_channels(s, b.gU, ct, cu, b.gS, cs, 0, cs, Pl, 0));
    __nv_bfloat16* dst = (l == L - 2) ? d->lv[L - 1].gS : d->lv[l + 1].gD;
    NN_TRY(asuna_nn_upsample2_bwd(s, b.gU, dst, D.n, hl / 2, wl / 2, cu, ct, 0));
    if (l < L - 2) NN_TRY(asuna_nn_relu_mask(s, dst, d->lv[l + 1].D, Pl / 4 * cu));
  }
  for (int l = L - 1; l >= 0; --l) {
    const int hl = D.hp >> l, wl = D.wp >> l;
    const size_t Pl = size_t(D.n) * hl * wl;
    LevelBufs& b = d->lv[l];
    NN_TRY(asuna_nn_relu_mask(s, b.gS, b.S, Pl * d->ch[l]));
    NN_TRY(convDw(d, d->enc(l, 1), b.gS, b.A, D.n, hl, wl));
    NN_TRY(convDx(d, d->enc(l, 1), b.gS, D.n, hl, wl, b.A, b.gA));
    NN_TRY(convDw(d, d->enc(l, 0), b.gA, b.X, D.n, hl, wl));
    if (l > 0) {
      NN_TRY(convDx(d, d->enc(l, 0), b.gA, D.n, hl, wl, nullptr, b.gX));
      NN_TRY(asuna_nn_avgpool2_bwd(s, b.gX, d->lv[l - 1].gS, D.n, hl * 2, wl * 2, d->ch[l - 1], 1));
    }
  }
  return ASUNA_OK;
}

const float* filmImage(const asuna_film* f, int image) {
  const size_t np = size_t(f->width) * f->height;
  if (image < 0) return nullptr;
  if (image == 0) return reinterpret_cast<const float*>(f->rad);
  if (image == 8) return reinterpret_cast<const float*>(f->w);
  return reinterpret_cast<const float*>(f->ch + size_t(image - 1) * np);
}

}  // namespace

extern "C" {

int asuna_denoiser_create(asuna_ctx* ctx, const asuna_denoiser_opts* o, asuna_denoiser** out) {
  clearError();
  if (!ctx || !o || !out) return fail(ASUNA_ERR_INVALID, "asuna_denoiser_create: null argument");
  *out = nullptr;
  const int L = int(o->levels);
  if (L < 2 || L > ASUNA_DENOISER_MAX_LEVELS) return fail(ASUNA_ERR_INVALID, "denoiser: levels %d not in 2..6", L);
  for (int l = 0; l < L; ++l)
    if (o->channels[l] == 0 || o->channels[l] % 16 || o->channels[l] > 256)
      return fail(ASUNA_ERR_INVALID, "denoiser: channels[%d] = %u must be a multiple of 16 in 16..256", l,
                  o->channels[l]);
  if (o->max_pixels == 0 || o->max_pixels > (1ull << 31))
    return fail(ASUNA_ERR_INVALID, "denoiser: max_pixels %llu out of range", (unsigned long long)o->max_pixels);
  if (o->loss != ASUNA_DENOISER_LOSS_L1_LOG && o->loss != ASUNA_DENOISER_LOSS_RELMSE)
    return fail(ASUNA_ERR_INVALID, "denoiser: unknown loss %u", o->loss);
  ASUNA_CUDA_TRY(cudaSetDevice(ctx->device));
  asuna_denoiser* d = new (std::nothrow) asuna_denoiser;
  if (!d) return fail(ASUNA_ERR_OOM, "host allocation failed");
  d->ctx = ctx;
  d->device = ctx->device;
  d->L = L;
  for (int l = 0; l < L; ++l) d->ch[l] = int(o->channels[l]);
  d->training = o->training != 0;
  d->useTc = o->tensor_memory != 0;
  d->loss = o->loss;
  d->maxPixels = o->max_pixels;
  // layers in parameter order
  auto add = [&](int cin, int cout) {
    ConvLayer c;
    c.cin = cin;
    c.cout = cout;
    c.wOff = d->nParams;
    d->nParams += size_t(cout) * 9 * cin;
    c.bOff = d->nParams;
    d->nParams += size_t(cout);
    c.wtOff = d->nFlip;
    d->nFlip += size_t(cout) * 9 * cin;
    d->layers.push_back(c);
  };
  for (int l = 0; l < L; ++l) {
    add(l == 0 ? kInC : d->ch[l - 1], d->ch[l]);
    add(d->ch[l], d->ch[l]);
  }
  for (int l = L - 2; l >= 0; --l) {
    add(d->ch[l + 1] + d->ch[l], d->ch[l]);
    add(d->ch[l], d->ch[l]);
  }
  add(d->ch[0], kHeadC);
  int rc = ASUNA_OK;
  auto A = [&](auto** p, size_t count) {
    if (rc == ASUNA_OK) rc = dalloc(d, p, count);
  };
  A(&d->p32, d->nParams);
  A(&d->pbf, d->nParams);
  A(&d->wt, d->nFlip);
  if (d->useTc) {
    A(&d->wtc, d->nFlip);
    A(&d->wtcT, d->nFlip);
  }
  A(&d->dLoss, 1);
  A(&d->dSums, 8);
  if (d->training) {
    A(&d->grad, d->nParams);
    A(&d->m, d->nParams);
    A(&d->v, d->nParams);
  }
  // activation workspace: level l holds max_pixels / 4^l pixels (rounded up)
  for (int l = 0; l < L; ++l) {
    const size_t Pl = size_t((o->max_pixels + (1ull << (2 * l)) - 1) >> (2 * l));
    LevelBufs& b = d->lv[l];
    const int cx = l == 0 ? kInC : d->ch[l - 1], c = d->ch[l];
    A(&b.X, Pl * cx);
    A(&b.A, Pl * c);
    A(&b.S, Pl * c);
    if (l <= L - 2) {
      A(&b.U, Pl * (d->ch[l + 1] + c));
      A(&b.B, Pl * c);
      A(&b.D, Pl * c);
    }
    if (d->training) {
      if (l > 0) A(&b.gX, Pl * cx);
      A(&b.gA, Pl * c);
      A(&b.gS, Pl * c);
      if (l <= L - 2) {
        A(&b.gU, Pl * (d->ch[l + 1] + c));
        A(&b.gB, Pl * c);
        A(&b.gD, Pl * c);
      }
    }
  }
  A(&d->head, size_t(o->max_pixels) * kHeadC);
  if (d->training) A(&d->gHead, size_t(o->max_pixels) * kHeadC);
  if (rc != ASUNA_OK) {
    delete d;
    return rc;
  }
  // He-normal weights (the head scaled by 0.1, so the first output is close
  // to the input), zero biases
  std::vector<float> host(d->nParams, 0.0f);
  InitRng rng{o->seed};
  for (size_t li = 0; li < d->layers.size(); ++li) {
    const ConvLayer& c = d->layers[li];
    const double sd = std::sqrt(2.0 / (9.0 * c.cin)) * (li + 1 == d->layers.size() ? 0.1 : 1.0);
    for (size_t i = 0; i < size_t(c.cout) * 9 * c.cin; ++i) host[c.wOff + i] = float(sd * rng.normal());
  }
  rc = asuna_denoiser_set_params(d, host.data(), host.size());
  if (rc != ASUNA_OK) {
    delete d;
    return rc;
  }
  *out = d;
  return ASUNA_OK;
}

// May run after the context is gone (garbage-collected handles): uses only
// the device ordinal; cudaFree waits for the device's work.
int asuna_denoiser_destroy(asuna_denoiser* d) {
  if (!d) return ASUNA_OK;
  cudaSetDevice(d->device);
  delete d;
  return ASUNA_OK;
}

uint64_t asuna_denoiser_num_params(const asuna_denoiser* d) { return d ? d->nParams : 0; }

int asuna_denoiser_set_params(asuna_denoiser* d, const float* host, uint64_t n) {
  if (!d || !host) return fail(ASUNA_ERR_INVALID, "asuna_denoiser_set_params: null argument");
  if (n != d->nParams) return fail(ASUNA_ERR_INVALID, "denoiser has %zu parameters, got %llu", d->nParams,
                                   (unsigned long long)n);
  ASUNA_CUDA_TRY(cudaSetDevice(d->ctx->device));
  cudaStream_t s = d->stream();
  ASUNA_CUDA_TRY(cudaMemcpyAsync(d->p32, host, n * sizeof(float), cudaMemcpyHostToDevice, s));
  NN_TRY(asuna_nn_f32_to_bf16(s, d->p32, d->pbf, n));
  if (d->training) {
    ASUNA_CUDA_TRY(cudaMemsetAsync(d->m, 0, n * sizeof(float), s));
    ASUNA_CUDA_TRY(cudaMemsetAsync(d->v, 0, n * sizeof(float), s));
    ASUNA_CUDA_TRY(cudaMemsetAsync(d->grad, 0, n * sizeof(float), s));
  }
  d->step = 0;
  d->flipped = false;
  ASUNA_CUDA_TRY(cudaStreamSynchronize(s));
  return ASUNA_OK;
}

int asuna_denoiser_get_params(asuna_denoiser* d, float* host, uint64_t n) {
  if (!d || !host || n != d->nParams) return fail(ASUNA_ERR_INVALID, "asuna_denoiser_get_params: bad argument");
  ASUNA_CUDA_TRY(cudaSetDevice(d->ctx->device));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(host, d->p32, n * sizeof(float), cudaMemcpyDeviceToHost, d->stream()));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(d->stream()));
  return ASUNA_OK;
}

int asuna_denoiser_get_grads(asuna_denoiser* d, float* host, uint64_t n) {
  if (!d || !host || n != d->nParams) return fail(ASUNA_ERR_INVALID, "asuna_denoiser_get_grads: bad argument");
  if (!d->training) return fail(ASUNA_ERR_INVALID, "denoiser was created without training state");
  ASUNA_CUDA_TRY(cudaSetDevice(d->ctx->device));
  ASUNA_CUDA_TRY(cudaMemcpyAsync(host, d->grad, n * sizeof(float), cudaMemcpyDeviceToHost, d->stream()));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(d->stream()));
  return ASUNA_OK;
}

int asuna_denoiser_forward(asuna_denoiser* d, const float* radiance, const float* albedo, const float* normal,
                           const float* weight, const float* noise, uint32_t n, uint32_t h, uint32_t w, float* out) {
  clearError();
  if (!d || !radiance || !out) return fail(ASUNA_ERR_INVALID, "asuna_denoiser_forward: null argument");
  Dims D;
  NN_TRY(dims(d, n, h, w, D));
  ASUNA_CUDA_TRY(cudaSetDevice(d->ctx->device));
  NN_TRY(forward(d, radiance, albedo, normal, weight, noise, D));
  k_output<<<grid1d(size_t(n) * h * w), 256, 0, d->stream()>>>(d->head, kHeadC,
                                                               reinterpret_cast<const float4*>(radiance),
                                                               reinterpret_cast<float4*>(out), D.n, D.h, D.w, D.hp,
                                                               D.wp);
  ASUNA_CUDA_TRY(cudaGetLastError());
  return ASUNA_OK;
}

int asuna_denoiser_loss_grad(asuna_denoiser* d, const float* radiance, const float* albedo, const float* normal,
                             const float* weight, const float* noise, const float* target, uint32_t n, uint32_t h,
                             uint32_t w, float* loss) {
  clearError();
  if (!d || !radiance || !target) return fail(ASUNA_ERR_INVALID, "asuna_denoiser_loss_grad: null argument");
  if (!d->training) return fail(ASUNA_ERR_INVALID, "denoiser was created without training state");
  Dims D;
  NN_TRY(dims(d, n, h, w, D));
  ASUNA_CUDA_TRY(cudaSetDevice(d->ctx->device));
  cudaStream_t s = d->stream();
  ASUNA_CUDA_TRY(cudaMemsetAsync(d->grad, 0, d->nParams * sizeof(float), s));
  ASUNA_CUDA_TRY(cudaMemsetAsync(d->dLoss, 0, sizeof(float), s));
  NN_TRY(forward(d, radiance, albedo, normal, weight, noise, D));
  const size_t P0 = size_t(D.n) * D.hp * D.wp;
  const float invCount = float(1.0 / (3.0 * double(n) * h * w));
  if (d->loss == ASUNA_DENOISER_LOSS_RELMSE)
    k_relmse_loss<<<grid1d(P0), 256, 0, s>>>(d->head, kHeadC, reinterpret_cast<const float4*>(radiance),
                                             reinterpret_cast<const float4*>(target), d->gHead, D.n, D.h, D.w, D.hp,
                                             D.wp, invCount, d->dLoss);
  else
    k_l1_loss<<<grid1d(P0), 256, 0, s>>>(d->head, kHeadC, reinterpret_cast<const float4*>(radiance),
                                         reinterpret_cast<const float4*>(target), d->gHead, D.n, D.h, D.w, D.hp, D.wp,
                                         invCount, d->dLoss);
  ASUNA_CUDA_TRY(cudaGetLastError());
  NN_TRY(backward(d, D));
  float l = 0.0f;
  ASUNA_CUDA_TRY(cudaMemcpyAsync(&l, d->dLoss, sizeof(float), cudaMemcpyDeviceToHost, s));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(s));
  if (loss) *loss = l / float(3.0 * double(n) * h * w);
  return ASUNA_OK;
}

int asuna_denoiser_adam(asuna_denoiser* d, float lr, float beta1, float beta2, float eps) {
  if (!d || !d->training) return fail(ASUNA_ERR_INVALID, "asuna_denoiser_adam: no training state");
  ASUNA_CUDA_TRY(cudaSetDevice(d->ctx->device));
  ++d->step;
  const float c1 = 1.0f - std::pow(beta1, float(d->step)), c2 = 1.0f - std::pow(beta2, float(d->step));
  k_adam<<<grid1d(d->nParams), 256, 0, d->stream()>>>(d->p32, d->m, d->v, d->grad, d->pbf, d->nParams, lr, beta1,
                                                      beta2, eps, c1, c2);
  ASUNA_CUDA_TRY(cudaGetLastError());
  d->flipped = false;
  return ASUNA_OK;
}

int asuna_denoise(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* film, int albedo_image, int normal_image,
                  float* out) {
  clearError();
  if (!ctx || !d || !film || !out) return fail(ASUNA_ERR_INVALID, "asuna_denoise: null argument");
  if (d->ctx != ctx) return fail(ASUNA_ERR_INVALID, "asuna_denoise: denoiser belongs to another context");
  if (albedo_image > 7 || normal_image > 7 || albedo_image == 0 || normal_image == 0)
    return fail(ASUNA_ERR_INVALID, "asuna_denoise: guide images must be channels 1..7 or -1");
  return asuna_denoiser_forward(d, filmImage(film, 0), filmImage(film, albedo_image), filmImage(film, normal_image),
                                filmImage(film, 8), nullptr, 1, film->height, film->width, out);
}

// A film's radiance denoised with a per-pixel noise estimate (device RGBA).
static int denoiseWithNoise(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* film, int albedo_image, int normal_image,
                            const float4* noise, float* out) {
  if (d->ctx != ctx) return fail(ASUNA_ERR_INVALID, "denoiser belongs to another context");
  if (albedo_image > 7 || normal_image > 7 || albedo_image == 0 || normal_image == 0)
    return fail(ASUNA_ERR_INVALID, "guide images must be channels 1..7 or -1");
  return asuna_denoiser_forward(d, filmImage(film, 0), filmImage(film, albedo_image), filmImage(film, normal_image),
                                filmImage(film, 8), reinterpret_cast<const float*>(noise), 1, film->height,
                                film->width, out);
}

int asuna_denoise_estimate(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* a, asuna_film* b, int albedo_image,
                           int normal_image, float* out, double* err_denoised, double* err_plain) {
  clearError();
  if (!a || !b) return fail(ASUNA_ERR_INVALID, "asuna_denoise_estimate: null film");
  if (a->width != b->width || a->height != b->height)
    return fail(ASUNA_ERR_INVALID, "asuna_denoise_estimate: films differ in size");
  if (!ctx || !d || !out) return fail(ASUNA_ERR_INVALID, "asuna_denoise_estimate: null argument");
  cudaStream_t s = ctx->stream;
  const size_t P = size_t(a->width) * a->height;
  float4* noise = nullptr;
  ASUNA_CUDA_TRY(cudaMallocAsync(&noise, P * sizeof(float4), s));
  struct Free {
    float4* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{noise, s};
  k_half_noise<<<grid1d(P), 256, 0, s>>>(a->rad, b->rad, noise, nullptr, P);
  ASUNA_CUDA_TRY(cudaGetLastError());
  NN_TRY(denoiseWithNoise(ctx, d, a, albedo_image, normal_image, noise, out));
  ASUNA_CUDA_TRY(cudaMemsetAsync(d->dSums, 0, 2 * sizeof(double), s));
  k_err_sums<<<grid1d(P), 256, 0, s>>>(reinterpret_cast<const float4*>(out), a->rad, b->rad, P, d->dSums);
  ASUNA_CUDA_TRY(cudaGetLastError());
  double h[2];
  ASUNA_CUDA_TRY(cudaMemcpyAsync(h, d->dSums, sizeof(h), cudaMemcpyDeviceToHost, s));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(s));
  const double mDB = h[0] / (3.0 * P), mAB = h[1] / (3.0 * P);
  if (err_denoised) *err_denoised = std::sqrt(std::max(0.0, mDB - 0.5 * mAB));
  if (err_plain) *err_plain = std::sqrt(0.25 * mAB);
  return ASUNA_OK;
}

int asuna_denoise_combined(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* a, asuna_film* b, int albedo_image,
                           int normal_image, float* out, double* err_denoised, double* err_plain) {
  clearError();
  if (!ctx || !d || !a || !b || !out) return fail(ASUNA_ERR_INVALID, "asuna_denoise_combined: null argument");
  if (a->width != b->width || a->height != b->height)
    return fail(ASUNA_ERR_INVALID, "asuna_denoise_combined: films differ in size");
  cudaStream_t s = ctx->stream;
  const size_t P = size_t(a->width) * a->height;
  float4 *db = nullptr, *rad = nullptr, *wsum = nullptr, *nHalf = nullptr, *nAll = nullptr;
  ASUNA_CUDA_TRY(cudaMallocAsync(&db, 5 * P * sizeof(float4), s));
  rad = db + P;
  wsum = rad + P;
  nHalf = wsum + P;
  nAll = nHalf + P;
  struct Free {
    float4* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{db, s};
  // D_A (into out) against film B, as asuna_denoise_estimate does
  double eA = 0.0, eP = 0.0;
  NN_TRY(asuna_denoise_estimate(ctx, d, a, b, albedo_image, normal_image, out, &eA, &eP));
  k_half_noise<<<grid1d(P), 256, 0, s>>>(a->rad, b->rad, nHalf, nAll, P);
  ASUNA_CUDA_TRY(cudaGetLastError());
  NN_TRY(denoiseWithNoise(ctx, d, b, albedo_image, normal_image, nHalf, reinterpret_cast<float*>(db)));
  ASUNA_CUDA_TRY(cudaMemsetAsync(d->dSums + 2, 0, sizeof(double), s));
  k_combine<<<grid1d(P), 256, 0, s>>>(reinterpret_cast<const float4*>(out), db, a->rad, b->rad, a->w, b->w, rad, wsum,
                                      P, d->dSums);
  ASUNA_CUDA_TRY(cudaGetLastError());
  double h = 0.0;
  ASUNA_CUDA_TRY(cudaMemcpyAsync(&h, d->dSums + 2, sizeof(double), cudaMemcpyDeviceToHost, s));
  NN_TRY(asuna_denoiser_forward(d, reinterpret_cast<const float*>(rad), filmImage(a, albedo_image),
                                filmImage(a, normal_image), reinterpret_cast<const float*>(wsum),
                                reinterpret_cast<const float*>(nAll), 1, a->height, a->width, out));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(s));
  // the halves' denoised outputs differ by twice the output variance of a
  // half; doubling the samples is taken to halve that variance and keep the
  // bias: err^2(all) = err^2(half) - var(half) / 2
  const double varHalf = 0.5 * h / (3.0 * P);
  if (err_denoised) *err_denoised = std::sqrt(std::max(0.0, eA * eA - 0.5 * varHalf));
  if (err_plain) *err_plain = eP;
  return ASUNA_OK;
}


int asuna_denoise_blended(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* a, asuna_film* b, int albedo_image,
                          int normal_image, float* out, double* err_out, double* err_plain, double* weight) {
  clearError();
  if (!ctx || !d || !a || !b || !out) return fail(ASUNA_ERR_INVALID, "asuna_denoise_blended: null argument");
  if (a->width != b->width || a->height != b->height)
    return fail(ASUNA_ERR_INVALID, "asuna_denoise_blended: films differ in size");
  cudaStream_t s = ctx->stream;
  const size_t P = size_t(a->width) * a->height;
  float4* scratch = nullptr;
  ASUNA_CUDA_TRY(cudaMallocAsync(&scratch, 6 * P * sizeof(float4), s));
  struct Free {
    float4* p;
    cudaStream_t s;
    ~Free() { cudaFreeAsync(p, s); }
  } guard{scratch, s};
  float4 *da = scratch, *db = da + P, *rad = db + P, *wsum = rad + P, *nHalf = wsum + P, *nAll = nHalf + P;
  k_half_noise<<<grid1d(P), 256, 0, s>>>(a->rad, b->rad, nHalf, nAll, P);
  ASUNA_CUDA_TRY(cudaGetLastError());
  NN_TRY(denoiseWithNoise(ctx, d, a, albedo_image, normal_image, nHalf, reinterpret_cast<float*>(da)));
  NN_TRY(denoiseWithNoise(ctx, d, b, albedo_image, normal_image, nHalf, reinterpret_cast<float*>(db)));
  ASUNA_CUDA_TRY(cudaMemsetAsync(d->dSums + 3, 0, 5 * sizeof(double), s));
  k_blend_sums<<<grid1d(P), 256, 0, s>>>(da, db, a->rad, b->rad, a->w, b->w, rad, wsum, P, d->dSums);
  ASUNA_CUDA_TRY(cudaGetLastError());
  double h[5];
  ASUNA_CUDA_TRY(cudaMemcpyAsync(h, d->dSums + 3, sizeof(h), cudaMemcpyDeviceToHost, s));
  NN_TRY(asuna_denoiser_forward(d, reinterpret_cast<const float*>(rad), filmImage(a, albedo_image),
                                filmImage(a, normal_image), reinterpret_cast<const float*>(wsum),
                                reinterpret_cast<const float*>(nAll), 1, a->height, a->width, out));
  ASUNA_CUDA_TRY(cudaStreamSynchronize(s));
  // X_half = w D_a + (1 - w) a, judged by b: err^2 = mean((X_half - b)^2) -
  // mean((a - b)^2) / 2; all samples: minus a quarter of mean((X_a - X_b)^2).
  // Both quadratic in w: f(w) = alpha w^2 + 2 beta w + gamma.
  const double n = 3.0 * double(P);
  const double Sdd = h[0] / n, Sda = h[1] / n, Saa = h[2] / n, Qdd = h[3] / n, Qda = h[4] / n;
  const double alpha = (Sdd - 2.0 * Sda + Saa) - 0.25 * (Qdd - 2.0 * Qda + Saa);
  const double beta = (Sda - Saa) - 0.25 * (Qda - Saa);
  const double gamma = 0.25 * Saa;
  auto f = [&](double w) { return alpha * w * w + 2.0 * beta * w + gamma; };
  double w = f(1.0) < f(0.0) ? 1.0 : 0.0;
  if (alpha > 0.0) {
    const double ws = std::min(1.0, std::max(0.0, -beta / alpha));
    if (f(ws) < f(w)) w = ws;
  }
  k_blend<<<grid1d(P), 256, 0, s>>>(reinterpret_cast<float4*>(out), a->rad, b->rad, float(w), P);
  ASUNA_CUDA_TRY(cudaGetLastError());
  ASUNA_CUDA_TRY(cudaStreamSynchronize(s));
  if (err_out) *err_out = std::sqrt(std::max(0.0, f(w)));
  if (err_plain) *err_plain = std::sqrt(std::max(0.0, gamma));
  if (weight) *weight = w;
  return ASUNA_OK;
}

}  // extern "C"

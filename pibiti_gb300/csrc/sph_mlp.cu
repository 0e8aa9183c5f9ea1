// sph_mlp.cu -- the per-particle MLP corrector (16 -> 64 -> 64 -> 3, tanh)
// on the tensor cores: BF16 operands, FP32 accumulation.  Two forms of each
// pass: mma.sync m16n8k16 (one warp = 16 particles per tile: k_forward,
// k_train) and tcgen05 kernels with TMEM accumulators (k_forward_tc, which
// the learned step runs, bit-identical to k_forward; k_train_tc, which
// training runs, equal to k_train up to FP32 summation order).
//
// Parameters are kept in FP32 (training master copy) in one vector:
//   W1[16][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]   (5443 floats)
// and packed to a BF16 image for the kernels (sph_mlp_pack):
//   WT1[64][24]  W1 transposed (out-major), forward operand of layer 1
//   WT2[64][72]  W2 transposed, forward operand of layer 2
//   W2r[64][72]  W2 in-major, backward operand (dH1 = dZ2 W2^T)
//   WT3[8][72]   W3 transposed, 3 outputs padded to 8, forward operand
//   W3r[64][24]  W3 in-major, outputs padded, backward operand
//   b1[64] b2[64] b3[8]   FP32
// Row strides are padded (24, 72 halves) so the fragment loads of a warp
// fall in distinct shared-memory banks.
//
// Fragment layout of mma.m16n8k16 (g = lane / 4, t = lane % 4):
//   A 16x16: a0 (g, 2t..2t+1) a1 (g+8, 2t..) a2 (g, 2t+8..) a3 (g+8, 2t+8..)
//   B 16x8 : b0 (k 2t..2t+1, n g) b1 (k 2t+8.., n g)
//   C 16x8 : c0 (g, 2t) c1 (g, 2t+1) c2 (g+8, 2t) c3 (g+8, 2t+1)
// The C fragments of two adjacent n-tiles are exactly the A fragment of the
// next layer's k-tile, so activations stay in registers between layers.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "sph_internal.h"

namespace sph {
namespace mlp {

constexpr int IN = 16, HID = 64, OUT = 3, OUTP = 8;
constexpr int S1 = 24, S2 = 72, S3r = 24;  // padded row strides (halves)
// packed image offsets (halves)
constexpr int oWT1 = 0;
constexpr int oWT2 = oWT1 + HID * S1;
constexpr int oW2r = oWT2 + HID * S2;
constexpr int oWT3 = oW2r + HID * S2;
constexpr int oW3r = oWT3 + OUTP * S2;
constexpr int kHalves = oW3r + HID * S3r;                 // 12864
constexpr int kBiasFloats = HID + HID + OUTP;             // 136
constexpr int kPackedBytes = kHalves * 2 + kBiasFloats * 4;
// canonical FP32 parameter offsets
constexpr int pW1 = 0, pB1 = pW1 + IN * HID, pW2 = pB1 + HID, pB2 = pW2 + HID * HID,
              pW3 = pB2 + HID, pB3 = pW3 + HID * OUT, kParams = pB3 + OUT;  // 5443

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float lo_of(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float hi_of(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }
__device__ __forceinline__ float bf(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }

__device__ __forceinline__ void mma(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const uint16_t* p) { return *reinterpret_cast<const uint32_t*>(p); }

// The hardware tanh (one instruction, accurate to about 2^-11): its result
// is rounded to BF16 (steps of 2^-9 relative) right after, so the
// approximation changes an activation by at most one BF16 step.
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ uint32_t tanh_pack2(float lo, float hi) {
  return pack2(tanh_hw(lo), tanh_hw(hi));
}

// Packs the FP32 parameters into the BF16 kernel image.
__global__ void k_pack(const float* __restrict__ prm, uint16_t* __restrict__ img) {
  uint16_t* w = img;
  float* bias = reinterpret_cast<float*>(img + kHalves);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kHalves + kBiasFloats;
       e += gridDim.x * blockDim.x) {
    if (e >= kHalves) {
      const int b = e - kHalves;
      float v = 0.f;
      if (b < HID) v = prm[pB1 + b];
      else if (b < 2 * HID) v = prm[pB2 + b - HID];
      else if (b - 2 * HID < OUT) v = prm[pB3 + b - 2 * HID];
      bias[b] = v;
      continue;
    }
    float v = 0.f;
    if (e < oWT2) {  // WT1[o][i] = W1[i][o]
      const int o = (e - oWT1) / S1, i = (e - oWT1) % S1;
      if (i < IN) v = prm[pW1 + i * HID + o];
    } else if (e < oW2r) {  // WT2[o][i] = W2[i][o]
      const int o = (e - oWT2) / S2, i = (e - oWT2) % S2;
      if (i < HID) v = prm[pW2 + i * HID + o];
    } else if (e < oWT3) {  // W2r[i][o] = W2[i][o]
      const int i = (e - oW2r) / S2, o = (e - oW2r) % S2;
      if (o < HID) v = prm[pW2 + i * HID + o];
    } else if (e < oW3r) {  // WT3[o][i] = W3[i][o]
      const int o = (e - oWT3) / S2, i = (e - oWT3) % S2;
      if (o < OUT && i < HID) v = prm[pW3 + i * OUT + o];
    } else {  // W3r[i][o] = W3[i][o]
      const int i = (e - oW3r) / S3r, o = (e - oW3r) % S3r;
      if (o < OUT) v = prm[pW3 + i * OUT + o];
    }
    w[e] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
  }
}

__device__ __forceinline__ void load_image(const uint16_t* __restrict__ img, uint16_t* sw) {
  const uint4* src = reinterpret_cast<const uint4*>(img);
  uint4* dst = reinterpret_cast<uint4*>(sw);
  for (int k = threadIdx.x; k < kPackedBytes / 16; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
}

// Forward pass of one 16-row tile; x is BF16 [rows][16].  Returns the
// output C fragment and leaves the hidden activations (BF16 A fragments).
struct Fwd {
  uint32_t h1[4][4];  // A fragments of layer 2 (k-tiles 0..3)
  uint32_t h2[4][4];  // A fragments of layer 3
  float y[4];         // C fragment of the output (cols 2t, 2t+1; rows g, g+8)
};

__device__ __forceinline__ void forward_tile(const uint16_t* sw, const float* sb,
                                             const uint16_t* __restrict__ x, uint32_t row0,
                                             uint32_t n, Fwd& f) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t r0 = row0 + g, r1 = row0 + g + 8;
  uint32_t a[4];
  a[0] = r0 < n ? ld32(x + (size_t)r0 * IN + 2 * t) : 0u;
  a[1] = r1 < n ? ld32(x + (size_t)r1 * IN + 2 * t) : 0u;
  a[2] = r0 < n ? ld32(x + (size_t)r0 * IN + 2 * t + 8) : 0u;
  a[3] = r1 < n ? ld32(x + (size_t)r1 * IN + 2 * t + 8) : 0u;
  // layer 1: [16 x 16] x [16 x 64]
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const float b0 = sb[8 * nt + 2 * t], b1 = sb[8 * nt + 2 * t + 1];
    float c[4] = {b0, b1, b0, b1};
    const uint16_t* w = sw + oWT1 + (8 * nt + g) * S1 + 2 * t;
    mma(c, a, ld32(w), ld32(w + 8));
    const int kt = nt >> 1;
    if ((nt & 1) == 0) {
      f.h1[kt][0] = tanh_pack2(c[0], c[1]);
      f.h1[kt][1] = tanh_pack2(c[2], c[3]);
    } else {
      f.h1[kt][2] = tanh_pack2(c[0], c[1]);
      f.h1[kt][3] = tanh_pack2(c[2], c[3]);
    }
  }
  // layer 2: [16 x 64] x [64 x 64]
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const float b0 = sb[HID + 8 * nt + 2 * t], b1 = sb[HID + 8 * nt + 2 * t + 1];
    float c[4] = {b0, b1, b0, b1};
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const uint16_t* w = sw + oWT2 + (8 * nt + g) * S2 + 16 * kt + 2 * t;
      mma(c, f.h1[kt], ld32(w), ld32(w + 8));
    }
    const int kt = nt >> 1;
    if ((nt & 1) == 0) {
      f.h2[kt][0] = tanh_pack2(c[0], c[1]);
      f.h2[kt][1] = tanh_pack2(c[2], c[3]);
    } else {
      f.h2[kt][2] = tanh_pack2(c[0], c[1]);
      f.h2[kt][3] = tanh_pack2(c[2], c[3]);
    }
  }
  // layer 3: [16 x 64] x [64 x 8]
  {
    const float b0 = sb[2 * HID + 2 * t], b1 = sb[2 * HID + 2 * t + 1];
    f.y[0] = b0;
    f.y[1] = b1;
    f.y[2] = b0;
    f.y[3] = b1;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const uint16_t* w = sw + oWT3 + g * S2 + 16 * kt + 2 * t;
      mma(f.y, f.h2[kt], ld32(w), ld32(w + 8));
    }
  }
}

// y[n][3] = MLP(x[n][16]).
__global__ void __launch_bounds__(128) k_forward(const uint16_t* __restrict__ img,
                                                 const uint16_t* __restrict__ x, uint32_t n,
                                                 float* __restrict__ y) {
  extern __shared__ __align__(16) uint16_t smem[];
  load_image(img, smem);
  const float* sb = reinterpret_cast<const float*>(smem + kHalves);
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n;
       tile += warps) {
    Fwd f;
    forward_tile(smem, sb, x, tile * 16, n, f);
    const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
    const int c0 = 2 * t;
    if (c0 < OUT) {
      if (r0 < n) y[(size_t)r0 * OUT + c0] = f.y[0];
      if (r1 < n) y[(size_t)r1 * OUT + c0] = f.y[2];
    }
    if (c0 + 1 < OUT) {
      if (r0 < n) y[(size_t)r0 * OUT + c0 + 1] = f.y[1];
      if (r1 < n) y[(size_t)r1 * OUT + c0 + 1] = f.y[3];
    }
  }
}

// One training pass over n samples: loss = sum((y - target)^2) * inv_count,
// gradients of that loss added (FP32 atomics) into grad[kParams], loss into
// *loss.  Per block: 4 warps x 16 samples per tile; forward and backward in
// registers, activations and their gradients staged in shared memory
// (BF16) for the weight-gradient products, which each warp accumulates for
// its quarter of every weight matrix over all tiles of the block.
constexpr int kTrainThreads = 128, kTileRows = 64;
constexpr int SA = 72;  // staging row stride (halves) for 64-wide rows
constexpr int SX = 24;  // staging row stride for 16-wide / 8-wide rows
constexpr int kStageHalves = kTileRows * (SX + SA + SA + SA + SA + SX);

__global__ void __launch_bounds__(kTrainThreads) k_train(const uint16_t* __restrict__ img,
                                                         const uint16_t* __restrict__ x,
                                                         const float* __restrict__ target,
                                                         uint32_t n, float inv_count,
                                                         float* __restrict__ grad,
                                                         float* __restrict__ loss) {
  extern __shared__ __align__(16) uint16_t smem[];
  load_image(img, smem);
  const float* sb = reinterpret_cast<const float*>(smem + kHalves);
  uint16_t* sX = smem + kHalves + 2 * kBiasFloats;
  uint16_t* sH1 = sX + kTileRows * SX;
  uint16_t* sH2 = sH1 + kTileRows * SA;
  uint16_t* sZ1 = sH2 + kTileRows * SA;
  uint16_t* sZ2 = sZ1 + kTileRows * SA;
  uint16_t* sY = sZ2 + kTileRows * SA;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  float aW2[8][4] = {}, aW1[2][4] = {}, aW3[4] = {};
  float bsum = 0.f, lsum = 0.f;  // bias gradient of column threadIdx.x (see below), loss
  const uint32_t tiles = (n + kTileRows - 1) / kTileRows;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t row0 = tile * kTileRows + 16 * w;
    Fwd f;
    forward_tile(smem, sb, x, row0, n, f);
    const uint32_t r0 = row0 + g, r1 = row0 + g + 8;
    // dL/dy for the 3 valid columns
    float dy[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t r = q < 2 ? r0 : r1;
      const int c = 2 * t + (q & 1);
      float d = 0.f;
      if (r < n && c < OUT) {
        const float e = f.y[q] - target[(size_t)r * OUT + c];
        lsum = fmaf(e, e, lsum);
        d = 2.f * e * inv_count;
      }
      dy[q] = d;
    }
    uint32_t ady[4] = {pack2(dy[0], dy[1]), pack2(dy[2], dy[3]), 0u, 0u};
    // dH2 = dY W3^T, dZ2 = dH2 (1 - h2^2)
    uint32_t az2[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      const uint16_t* wp = smem + oW3r + (8 * nt + g) * S3r + 2 * t;
      mma(c, ady, ld32(wp), ld32(wp + 8));
      const int kt = nt >> 1, hi = nt & 1;
      const uint32_t h01 = f.h2[kt][hi ? 2 : 0], h23 = f.h2[kt][hi ? 3 : 1];
      const float z0 = c[0] * (1.f - lo_of(h01) * lo_of(h01));
      const float z1 = c[1] * (1.f - hi_of(h01) * hi_of(h01));
      const float z2 = c[2] * (1.f - lo_of(h23) * lo_of(h23));
      const float z3 = c[3] * (1.f - hi_of(h23) * hi_of(h23));
      az2[kt][hi ? 2 : 0] = pack2(z0, z1);
      az2[kt][hi ? 3 : 1] = pack2(z2, z3);
    }
    // dH1 = dZ2 W2^T, dZ1 = dH1 (1 - h1^2)
    uint32_t az1[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        const uint16_t* wp = smem + oW2r + (8 * nt + g) * S2 + 16 * kt + 2 * t;
        mma(c, az2[kt], ld32(wp), ld32(wp + 8));
      }
      const int kt = nt >> 1, hi = nt & 1;
      const uint32_t h01 = f.h1[kt][hi ? 2 : 0], h23 = f.h1[kt][hi ? 3 : 1];
      const float z0 = c[0] * (1.f - lo_of(h01) * lo_of(h01));
      const float z1 = c[1] * (1.f - hi_of(h01) * hi_of(h01));
      const float z2 = c[2] * (1.f - lo_of(h23) * lo_of(h23));
      const float z3 = c[3] * (1.f - hi_of(h23) * hi_of(h23));
      az1[kt][hi ? 2 : 0] = pack2(z0, z1);
      az1[kt][hi ? 3 : 1] = pack2(z2, z3);
    }
    // stage this warp's 16 rows: X, H1, H2, dZ1, dZ2, dY (BF16)
    {
      const int lr0 = 16 * w + g, lr1 = lr0 + 8;
      auto st = [&](uint16_t* base, int stride, int row, int col, uint32_t v) {
        *reinterpret_cast<uint32_t*>(base + row * stride + col) = v;
      };
      st(sX, SX, lr0, 2 * t, r0 < n ? ld32(x + (size_t)r0 * IN + 2 * t) : 0u);
      st(sX, SX, lr1, 2 * t, r1 < n ? ld32(x + (size_t)r1 * IN + 2 * t) : 0u);
      st(sX, SX, lr0, 2 * t + 8, r0 < n ? ld32(x + (size_t)r0 * IN + 2 * t + 8) : 0u);
      st(sX, SX, lr1, 2 * t + 8, r1 < n ? ld32(x + (size_t)r1 * IN + 2 * t + 8) : 0u);
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        const int c0 = 16 * kt + 2 * t, c1 = c0 + 8;
        st(sH1, SA, lr0, c0, f.h1[kt][0]); st(sH1, SA, lr1, c0, f.h1[kt][1]);
        st(sH1, SA, lr0, c1, f.h1[kt][2]); st(sH1, SA, lr1, c1, f.h1[kt][3]);
        st(sH2, SA, lr0, c0, f.h2[kt][0]); st(sH2, SA, lr1, c0, f.h2[kt][1]);
        st(sH2, SA, lr0, c1, f.h2[kt][2]); st(sH2, SA, lr1, c1, f.h2[kt][3]);
        st(sZ1, SA, lr0, c0, az1[kt][0]); st(sZ1, SA, lr1, c0, az1[kt][1]);
        st(sZ1, SA, lr0, c1, az1[kt][2]); st(sZ1, SA, lr1, c1, az1[kt][3]);
        st(sZ2, SA, lr0, c0, az2[kt][0]); st(sZ2, SA, lr1, c0, az2[kt][1]);
        st(sZ2, SA, lr0, c1, az2[kt][2]); st(sZ2, SA, lr1, c1, az2[kt][3]);
      }
      st(sY, SX, lr0, 2 * t, ady[0]);
      st(sY, SX, lr1, 2 * t, ady[1]);
    }
    __syncthreads();
    // weight gradients over the block's 64 samples (K = samples)
    auto afrag = [&](const uint16_t* base, int stride, int m0, int kt, uint32_t a[4]) {
      // A[m][k] = base[k][m]: rows m0+g, m0+g+8; samples 16kt + 2t (+1, +8, +9)
      const int s0 = 16 * kt + 2 * t;
      const uint16_t* p = base + m0 + g;
      a[0] = (uint32_t)p[s0 * stride] | ((uint32_t)p[(s0 + 1) * stride] << 16);
      a[1] = (uint32_t)p[s0 * stride + 8] | ((uint32_t)p[(s0 + 1) * stride + 8] << 16);
      a[2] = (uint32_t)p[(s0 + 8) * stride] | ((uint32_t)p[(s0 + 9) * stride] << 16);
      a[3] = (uint32_t)p[(s0 + 8) * stride + 8] | ((uint32_t)p[(s0 + 9) * stride + 8] << 16);
    };
    auto bfrag = [&](const uint16_t* base, int stride, int n0, int kt, uint32_t& b0, uint32_t& b1) {
      // B[k][n] = base[k][n]: n = n0 + g; samples 16kt + 2t (+1), +8 (+9)
      const int s0 = 16 * kt + 2 * t;
      const uint16_t* p = base + n0 + g;
      b0 = (uint32_t)p[s0 * stride] | ((uint32_t)p[(s0 + 1) * stride] << 16);
      b1 = (uint32_t)p[(s0 + 8) * stride] | ((uint32_t)p[(s0 + 9) * stride] << 16);
    };
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      uint32_t a[4], b0, b1;
      // dW2[16w.., :] += H1^T dZ2
      afrag(sH1, SA, 16 * w, kt, a);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        bfrag(sZ2, SA, 8 * nt, kt, b0, b1);
        mma(aW2[nt], a, b0, b1);
      }
      // dW3[16w.., 0..7] += H2^T dY
      afrag(sH2, SA, 16 * w, kt, a);
      bfrag(sY, SX, 0, kt, b0, b1);
      mma(aW3, a, b0, b1);
      // dW1[0..15, 16w..16w+15] += X^T dZ1
      afrag(sX, SX, 0, kt, a);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        bfrag(sZ1, SA, 16 * w + 8 * q, kt, b0, b1);
        mma(aW1[q], a, b0, b1);
      }
    }
    // bias gradients: thread c < 64 sums column c of dZ1, 64 <= c < 128
    // column c-64 of dZ2; column sums of dY are added by threads 0..2 below.
    {
      const int c = threadIdx.x;
      const uint16_t* col = c < 64 ? sZ1 + c : sZ2 + (c - 64);
      float s = 0.f;
      for (int r = 0; r < kTileRows; ++r) s += bf(col[r * SA]);
      bsum += s;
    }
    if (threadIdx.x < OUT) {
      float s = 0.f;
      for (int r = 0; r < kTileRows; ++r) s += bf(sY[r * SX + threadIdx.x]);
      atomicAdd(grad + pB3 + threadIdx.x, s);
    }
    __syncthreads();
  }
  // flush the block's partial gradients
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = 16 * w + g + (q >= 2 ? 8 : 0), o = 8 * nt + 2 * t + (q & 1);
      atomicAdd(grad + pW2 + i * HID + o, aW2[nt][q]);
    }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = 16 * w + g + (q >= 2 ? 8 : 0), o = 2 * t + (q & 1);
    if (o < OUT) atomicAdd(grad + pW3 + i * OUT + o, aW3[q]);
  }
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = g + (q >= 2 ? 8 : 0), o = 16 * w + 8 * h + 2 * t + (q & 1);
      atomicAdd(grad + pW1 + i * HID + o, aW1[h][q]);
    }
  atomicAdd(grad + (threadIdx.x < 64 ? pB1 + threadIdx.x : pB2 + threadIdx.x - 64), bsum);
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) atomicAdd(loss, lsum * inv_count);
}

// Adam on the FP32 master parameters.
__global__ void k_adam(float* __restrict__ prm, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ grad, int count, float lr, float beta1,
                       float beta2, float eps, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gr = grad[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * gr;
  const float vi = beta2 * v[i] + (1.f - beta2) * gr * gr;
  m[i] = mi;
  v[i] = vi;
  prm[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

}  // namespace mlp
}  // namespace sph

using namespace sph;
using namespace sph::mlp;

namespace {
constexpr int kTrainSmem = kPackedBytes + kStageHalves * 2;

int mlp_kernels_ready() {
  static int rc = -1;
  if (rc < 0) {
    rc = cuda_check(cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kTrainSmem),
                    "mlp: shared memory limit");
  }
  return rc;
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

// ---- tcgen05 inference ------------------------------------------------------
// The forward pass on the 5th-generation tensor cores: one CTA of 128
// threads per 128-particle tile (grid-stride over tiles).  Each layer is a
// tcgen05.mma chain (layer 1: 128x16 . 16x64, one instruction; layer 2:
// 128x64 . 64x64 and layer 3: 128x64 . 64x16, four of K = 16 each) with BF16
// operands in shared memory (K-major core-matrix layout, no swizzle) and FP32
// accumulators in one 64-column TMEM allocation that the three layers use in
// turn.  Each layer's accumulators start from its bias (tcgen05.st), as the
// mma.sync pass's fragments do, so both round the same sums.  Each warp reads
// its 32 rows (TMEM lanes 32w..32w+31) back with tcgen05.ld; tanh runs in
// registers and the BF16 activations go back to shared memory as the next
// layer's A operand.  The input tile and the layer-1 and layer-2 activations
// share one buffer: each is dead once the MMA that reads it has completed.
// Only outputs 0..2 of layer 3 are kept, so rows 3..15 of its B operand are
// don't-care: row 3 holds b3, rows 4..7 the biases b1 and b2, rows 8..15 are
// the first bytes of W2^T.  That keeps a CTA at 27.0 KB of shared memory, so
// 8 fit an SM with 8 x 64 = 512 TMEM columns.  Thread 0 issues the MMAs and
// commits them to one mbarrier; every wait on it is bounded (kTcSpins polls),
// after which the CTA records an error (sph_mlp_status), writes NaN to the
// rows it did not finish, and still frees its TMEM.
namespace tcg {
constexpr uint32_t kTcSpins = 1u << 22;
// shared memory (bytes)
constexpr uint32_t oH = 0;        // X 128 x 16, then H1 and H2 128 x 64 (BF16): 16 x 8 x 128 B
constexpr uint32_t oW1 = 16384;   // W1^T 64 x 16 (N x K): 8 x 2 x 128 B
constexpr uint32_t oW3 = 18432;   // W3^T rows 0..7 x 64: 8 x 128 B; rows 8..15 = oW2
constexpr uint32_t oW2 = 19456;   // W2^T 64 x 64: 8 x 8 x 128 B
constexpr uint32_t oBar = 27648;  // mbarrier (8 B)
constexpr uint32_t oTmem = 27656; // TMEM base address written by tcgen05.alloc
constexpr uint32_t kSmem = 27664;
constexpr uint32_t kCols = 64;
constexpr uint32_t kBlocksPerSm = 8;  // 8 x 64 = the 512 TMEM columns
static_assert(kBlocksPerSm * kCols <= 512, "TMEM columns of the resident CTAs");
static_assert(kBlocksPerSm * (kSmem + 1024) <= 233472, "shared memory of the resident CTAs");
static_assert(oW3 + 1024 == oW2, "rows 8..15 of W3^T are read from W2^T");
// bias value e of b1 (e < 64) or b2 (64 <= e < 128): K-core e / 16 of W3^T,
// rows 4..7 (bytes 64..127), 16 floats per core
__host__ __device__ constexpr uint32_t bias_off(uint32_t e) { return oW3 + (e >> 4) * 128u + 64u + (e & 15u) * 4u; }
constexpr uint32_t oB3 = oW3 + 48;  // b3[3], 0: row 3 of K-core 0 of W3^T

// Byte offset of element (r, k) (BF16) of a K-major operand made of 8-row x
// 16-byte core matrices, `kc` cores along K: K-adjacent cores 128 B apart
// (the descriptor's leading offset), row-adjacent cores 128 * kc B apart
// (its stride offset).
__host__ __device__ constexpr uint32_t core_off(uint32_t r, uint32_t k, uint32_t kc) {
  return ((r >> 3) * kc + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all >> 4), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(phase)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, uint32_t spins) {
  for (uint32_t k = 0; k < spins; ++k)
    if (mbar_try(bar, phase)) return true;
  return false;
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Orders this CTA's shared-memory stores and TMEM reads before what thread 0
// issues next (the tensor core reads shared memory through the async proxy).
__device__ __forceinline__ void sync_for_mma() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  fence_before();
  __syncthreads();
  fence_after();
}
__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void ld4(uint32_t taddr, float* v) {
  uint32_t r[4];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 4; ++k) v[k] = __uint_as_float(r[k]);
}
// Seeds this thread's TMEM lane with a layer's bias (columns 0..63), as
// the mma.sync pass seeds its accumulators: the MMAs then add the products
// to it, so both passes round the same sums.  `layer` 0 is b1, 1 is b2.
__device__ __forceinline__ void st16(uint32_t taddr, const float* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};" ::"r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])) : "memory");
}
__device__ __forceinline__ void seed_bias(uint32_t lane_base, const uint8_t* sm, uint32_t layer) {
#pragma unroll 1
  for (int q = 0; q < 4; ++q) {
    float v[16];
    const float4* b4 = reinterpret_cast<const float4*>(sm + bias_off(64u * layer + 16u * q));
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float4 b = b4[j];
      v[4 * j] = b.x;
      v[4 * j + 1] = b.y;
      v[4 * j + 2] = b.z;
      v[4 * j + 3] = b.w;
    }
    st16(lane_base + 16u * q, v);
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void seed_out_bias(uint32_t lane_base, const uint8_t* sm) {
  const float4 b = *reinterpret_cast<const float4*>(sm + oB3);
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(lane_base),
               "r"(__float_as_uint(b.x)), "r"(__float_as_uint(b.y)), "r"(__float_as_uint(b.z)),
               "r"(__float_as_uint(b.w))
               : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
// tanh of this thread's row of the accumulators (64 columns, bias included)
// as BF16 into row t of the activation buffer (core-matrix layout, 8
// K-cores).
__device__ __forceinline__ void activate(uint32_t lane_base, uint8_t* hbuf, uint32_t t) {
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    ld32(lane_base + 32u * half, v);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const uint32_t c0 = 32u * half + 16u * q;
      uint32_t pk[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) pk[j] = tanh_pack2(v[16 * q + 2 * j], v[16 * q + 2 * j + 1]);
      *reinterpret_cast<uint4*>(hbuf + core_off(t, c0, 8)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      *reinterpret_cast<uint4*>(hbuf + core_off(t, c0 + 8, 8)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
  }
}
}  // namespace tcg

__device__ uint32_t g_tc_status;  // non-zero: a tcgen05 wait ran out (sph_mlp_status)

// `spins` bounds each wait; `withhold` (a test of the timeout path) issues
// no MMA and commits nothing, so that the first wait runs out.
__global__ void __launch_bounds__(128, tcg::kBlocksPerSm) k_forward_tc(const uint16_t* __restrict__ img,
                                                                       const uint16_t* __restrict__ x,
                                                                       uint32_t n, float* __restrict__ y,
                                                                       uint32_t spins, bool withhold) {
  using namespace tcg;
  extern __shared__ __align__(128) uint8_t sm[];
  const uint32_t t = threadIdx.x, w = t >> 5;
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(sm);
  const uint32_t tiles = (n + 127) / 128;
  // this thread's row of the next tile is fetched while the current one runs
  uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0;
  auto fetch = [&](uint32_t tile) {
    const uint32_t r = tile * 128 + t;
    c0 = c1 = make_uint4(0, 0, 0, 0);
    if (tile < tiles && r < n) {
      const uint4* src = reinterpret_cast<const uint4*>(x + (size_t)r * IN);
      c0 = src[0];
      c1 = src[1];
    }
  };
  fetch(blockIdx.x);
  // weights into the core-matrix layout (16-byte rows of 8 inputs; the
  // image's row strides, 48 and 144 bytes, keep them aligned) and the biases
  {
    const uint32_t o = t >> 1, c = t & 1u;  // W1^T: 64 rows x 2 chunks
    *reinterpret_cast<uint4*>(sm + oW1 + core_off(o, 8 * c, 2)) =
        *reinterpret_cast<const uint4*>(img + oWT1 + o * S1 + 8 * c);
  }
  for (uint32_t e = t; e < 64 * 8; e += 128) {  // W2^T: 64 rows x 8 chunks
    const uint32_t o = e >> 3, c = e & 7u;
    *reinterpret_cast<uint4*>(sm + oW2 + core_off(o, 8 * c, 8)) =
        *reinterpret_cast<const uint4*>(img + oWT2 + o * S2 + 8 * c);
  }
  const float* bimg = reinterpret_cast<const float*>(img + kHalves);  // b1 b2 b3
  if (t < 3 * 8) {  // W3^T rows 0..2 x 8 chunks
    const uint32_t o = t >> 3, c = t & 7u;
    *reinterpret_cast<uint4*>(sm + oW3 + core_off(o, 8 * c, 8)) =
        *reinterpret_cast<const uint4*>(img + oWT3 + o * S2 + 8 * c);
  }
  *reinterpret_cast<float*>(sm + bias_off(t)) = bimg[t];  // b1, b2 (128 values)
  if (t < 4) reinterpret_cast<float*>(sm + oB3)[t] = t < OUT ? bimg[2 * HID + t] : 0.f;
  if (t == 0) mbar_init(sb + oBar);
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sb + oTmem),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  sync_for_mma();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + oTmem);
  const uint32_t lane_base = tmem + ((32u * w) << 16);
  uint32_t phase = 0;
  bool ok = true, pending = false;
  // thread 0 issues, everyone waits (bounded); false when the wait ran out
  auto run = [&](auto issue) {
    if (t == 0 && !withhold) {
      issue();
      commit(sb + oBar);
    }
    pending = !withhold;
    ok = __syncthreads_and(mbar_wait(sb + oBar, phase, spins));
    if (!ok) return false;
    pending = false;
    phase ^= 1u;
    fence_after();
    return true;
  };
  uint32_t tile = blockIdx.x;
  for (; tile < tiles; tile += gridDim.x) {
    const uint32_t row = tile * 128 + t;
    *reinterpret_cast<uint4*>(sm + oH + core_off(t, 0, 2)) = c0;
    *reinterpret_cast<uint4*>(sm + oH + core_off(t, 8, 2)) = c1;
    fetch(tile + gridDim.x);
    seed_bias(lane_base, sm, 0);
    sync_for_mma();
    if (!run([&] { umma(tmem, sdesc(sb + oH, 128, 256), sdesc(sb + oW1, 128, 256), idesc(128, 64), 1u); }))
      break;
    activate(lane_base, sm + oH, t);  // H1
    seed_bias(lane_base, sm, 1);
    sync_for_mma();
    if (!run([&] {
          const uint64_t a = sdesc(sb + oH, 128, 1024), b = sdesc(sb + oW2, 128, 1024);
#pragma unroll 1
          for (uint32_t kk = 0; kk < 4; ++kk)  // K step of 16: 256 B, 16 in the address field
            umma(tmem, a + 16u * kk, b + 16u * kk, idesc(128, 64), 1u);
        }))
      break;
    activate(lane_base, sm + oH, t);  // H2
    seed_out_bias(lane_base, sm);
    sync_for_mma();
    if (!run([&] {
          const uint64_t a = sdesc(sb + oH, 128, 1024), b = sdesc(sb + oW3, 128, 1024);
#pragma unroll 1
          for (uint32_t kk = 0; kk < 4; ++kk)
            umma(tmem, a + 16u * kk, b + 16u * kk, idesc(128, 16), 1u);
        }))
      break;
    float o[4];
    ld4(lane_base, o);
    if (row < n) {
      y[(size_t)row * OUT + 0] = o[0];
      y[(size_t)row * OUT + 1] = o[1];
      y[(size_t)row * OUT + 2] = o[2];
    }
    // this thread's next tcgen05.st comes after its own reads (wait::ld);
    // the next tile's first sync_for_mma orders them all before its MMA
  }
  if (!ok) {
    if (t == 0) atomicOr(&g_tc_status, 1u);
    if (pending) __syncthreads_and(mbar_wait(sb + oBar, phase, spins));  // the MMAs still in flight
    // the rows this CTA did not finish become NaN, which a caller's
    // finiteness check sees
    for (; tile < tiles; tile += gridDim.x) {
      const uint32_t row = tile * 128 + t;
      if (row < n) y[(size_t)row * OUT + 0] = y[(size_t)row * OUT + 1] = y[(size_t)row * OUT + 2] = __int_as_float(0x7fc00000);
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (w == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
}

// ---- tcgen05 training --------------------------------------------------------
// One training pass (sph_mlp_train_pass_tc) on the 5th-generation tensor
// cores: one CTA of 128 threads per 128-sample tile (grid-stride over
// tiles), thread t owning sample t of the tile.  Per tile, every product
// is a tcgen05.mma chain with BF16 operands in shared memory and FP32
// accumulators in tensor memory:
//   forward   Z1 = X W1 + b1, Z2 = H1 W2 + b2, Y = H2 W3 + b3 (as k_forward_tc)
//   backward  dH2 = dY W3^T, dH1 = dZ2 W2^T   (dZ = dH (1 - H^2), per thread)
//   gradients G2 = dZ2^T [H1 | 1], G3 = dY^T [H2 | 1], G1 = dZ1^T [X | 1]
// The weight-gradient products contract over the tile's samples.  They read
// the activations and gradients where the forward and backward products
// left them (rows = samples): as operands whose M or N dimension is the
// contiguous one (MN-major, transpose bits 15 and 16 of the instruction
// descriptor; leading byte offset = the stride between core matrices along
// K, the samples, and stride byte offset = the stride along M or N), so no
// transposed copy is made.  A ones column appended to H1, H2 and X puts the
// bias gradients (column sums of dZ2, dY, dZ1) in column 64, 64 and 16 of
// G2, G3 and G1.  The M dimension of every product is 128: G2 and G1 have
// 64 real rows and G3 3; the other rows read whatever lies beyond the
// operand in shared memory and are never used (row r of a product depends
// on row r of A alone).  The three gradient accumulators stay in tensor
// memory across all tiles of the CTA (256 columns: scratch 0-63, G2 64-143,
// G3 144-223, G1 224-255) and are added to `grad` once at the end, one
// atomicAdd per parameter and CTA.  BF16 roundings are the mma.sync pass's
// (k_train): X, H1, H2, dY, dZ2, dZ1 and the weights.  Every wait is
// bounded; a CTA whose wait runs out sets status bit 1, adds NaN to *loss
// and adds nothing to `grad`.
namespace tct {
using namespace tcg;
// shared memory (bytes); the operands whose garbage rows read past their
// end (dZ2, dZ1: 1 KB; dY: 1.8 KB) are followed by other buffers
constexpr uint32_t tDZ2 = 0;        // 128 x 64, 8 K-cores per row group
constexpr uint32_t tDZ1 = 16384;    // 128 x 64
constexpr uint32_t tDY = 32768;     // 128 x 16 (outputs 0..2, then zeros)
constexpr uint32_t tX = 36864;      // 128 x 32: inputs 0..15, a one, zeros
constexpr uint32_t tH1 = 45056;     // 128 x 80: hidden 0..63, a one, zeros
constexpr uint32_t tH2 = 65536;     // 128 x 80
constexpr uint32_t tW1 = 86016;     // W1^T 64 x 16
constexpr uint32_t tW2 = 88064;     // W2^T 64 x 64
constexpr uint32_t tW3 = 96256;     // W3^T 16 x 64 (rows 3..15 zero)
constexpr uint32_t tW3r = 98304;    // W3 64 x 16 (in-major; columns 3..15 zero)
constexpr uint32_t tW2r = 100352;   // W2 64 x 64 (in-major)
constexpr uint32_t tBias = 108544;  // b1[64] b2[64] b3[4]
constexpr uint32_t tBar = 109088;
constexpr uint32_t tTmem = 109096;
constexpr uint32_t kTrSmem = 109184;
constexpr uint32_t kTrCols = 256;
constexpr uint32_t cG2 = 64, cG3 = 144, cG1 = 224;  // TMEM columns of the gradients
constexpr uint32_t kTrBlocks = 2;
static_assert(kTrBlocks * kTrCols <= 512, "TMEM columns of the resident CTAs");
static_assert(kTrBlocks * (kTrSmem + 1024) <= 233472, "shared memory of the resident CTAs");
static_assert(tDZ2 + 15 * 128 + 15 * 1024 + 128 <= tDY, "dZ2 garbage rows stay in shared memory");
static_assert(tDZ1 + 15 * 128 + 15 * 1024 + 128 <= tX, "dZ1 garbage rows stay in shared memory");
static_assert(tDY + 15 * 128 + 15 * 256 + 128 <= kTrSmem, "dY garbage rows stay in shared memory");
static_assert(tTmem + 4 <= kTrSmem, "layout");
constexpr uint32_t kMN = (1u << 15) | (1u << 16);  // A and B MN-major

__device__ __forceinline__ void ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
// 64 bias values (b1 or b2) into this thread's scratch columns 0..63.
__device__ __forceinline__ void seed64(uint32_t lane_base, const float* b) {
#pragma unroll 1
  for (int q = 0; q < 4; ++q) st16(lane_base + 16u * q, b + 16 * q);
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
// tanh of this thread's 64 scratch columns as BF16 into row t of an
// activation buffer of 10 K-cores per row group.
__device__ __forceinline__ void activate10(uint32_t lane_base, uint8_t* hbuf, uint32_t t) {
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    ld32(lane_base + 32u * half, v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t pk[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) pk[j] = tanh_pack2(v[8 * q + 2 * j], v[8 * q + 2 * j + 1]);
      *reinterpret_cast<uint4*>(hbuf + core_off(t, 32u * half + 8u * q, 10)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
  }
}
// dZ = dH (1 - h^2) for this thread's row: dH from scratch columns 0..63,
// h (BF16) from row t of `hbuf` (10 K-cores), dZ as BF16 into row t of
// `zbuf` (8 K-cores).
__device__ __forceinline__ void grad_act(uint32_t lane_base, const uint8_t* hbuf, uint8_t* zbuf, uint32_t t) {
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    ld32(lane_base + 32u * half, v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t c0 = 32u * half + 8u * q;
      const uint4 h = *reinterpret_cast<const uint4*>(hbuf + core_off(t, c0, 10));
      const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
      uint32_t pk[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float h0 = lo_of(hw[j]), h1 = hi_of(hw[j]);
        pk[j] = pack2(v[8 * q + 2 * j] * (1.f - h0 * h0), v[8 * q + 2 * j + 1] * (1.f - h1 * h1));
      }
      *reinterpret_cast<uint4*>(zbuf + core_off(t, c0, 8)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
  }
}
}  // namespace tct

__global__ void __launch_bounds__(128, tct::kTrBlocks) k_train_tc(const uint16_t* __restrict__ img,
                                                                     const uint16_t* __restrict__ x,
                                                                     const float* __restrict__ target,
                                                                     uint32_t n, float inv_count,
                                                                     float* __restrict__ grad,
                                                                     float* __restrict__ loss,
                                                                     uint32_t spins, bool withhold) {
  using namespace tct;
  extern __shared__ __align__(128) uint8_t sm[];
  const uint32_t t = threadIdx.x, w = t >> 5;
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(sm);
  const uint32_t tiles = (n + 127) / 128;
  // weights (K-major core-matrix layout) and biases, once per CTA
  {
    const uint32_t o = t >> 1, c = t & 1u;  // W1^T, W3 in-major: 64 rows x 2 chunks
    *reinterpret_cast<uint4*>(sm + tW1 + core_off(o, 8 * c, 2)) =
        *reinterpret_cast<const uint4*>(img + oWT1 + o * S1 + 8 * c);
    *reinterpret_cast<uint4*>(sm + tW3r + core_off(o, 8 * c, 2)) =
        *reinterpret_cast<const uint4*>(img + mlp::oW3r + o * S3r + 8 * c);
  }
  for (uint32_t e = t; e < 64 * 8; e += 128) {  // W2^T and W2: 64 rows x 8 chunks
    const uint32_t o = e >> 3, c = e & 7u;
    *reinterpret_cast<uint4*>(sm + tW2 + core_off(o, 8 * c, 8)) =
        *reinterpret_cast<const uint4*>(img + oWT2 + o * S2 + 8 * c);
    *reinterpret_cast<uint4*>(sm + tW2r + core_off(o, 8 * c, 8)) =
        *reinterpret_cast<const uint4*>(img + mlp::oW2r + o * S2 + 8 * c);
  }
  {  // W3^T: rows 0..7 from the image (3..7 are zero there), rows 8..15 zero
    const uint32_t o = t >> 3, c = t & 7u;  // 16 rows x 8 chunks
    *reinterpret_cast<uint4*>(sm + tW3 + core_off(o, 8 * c, 8)) =
        o < 8 ? *reinterpret_cast<const uint4*>(img + oWT3 + o * S2 + 8 * c) : make_uint4(0, 0, 0, 0);
  }
  const float* bimg = reinterpret_cast<const float*>(img + kHalves);  // b1 b2 b3
  float* sbias = reinterpret_cast<float*>(sm + tBias);
  sbias[t] = bimg[t];
  if (t < 4) sbias[128 + t] = t < OUT ? bimg[2 * HID + t] : 0.f;
  // the constant columns: X 16..31 = (1, 0, ...), H1 and H2 64..79 = (1, 0, ...)
  const uint4 one = make_uint4(0x3F80u, 0u, 0u, 0u), zero = make_uint4(0u, 0u, 0u, 0u);
  *reinterpret_cast<uint4*>(sm + tX + core_off(t, 16, 4)) = one;
  *reinterpret_cast<uint4*>(sm + tX + core_off(t, 24, 4)) = zero;
  *reinterpret_cast<uint4*>(sm + tH1 + core_off(t, 64, 10)) = one;
  *reinterpret_cast<uint4*>(sm + tH1 + core_off(t, 72, 10)) = zero;
  *reinterpret_cast<uint4*>(sm + tH2 + core_off(t, 64, 10)) = one;
  *reinterpret_cast<uint4*>(sm + tH2 + core_off(t, 72, 10)) = zero;
  if (t == 0) mbar_init(sb + tBar);
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sb + tTmem),
                 "r"(kTrCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  sync_for_mma();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + tTmem);
  const uint32_t lane_base = tmem + ((32u * w) << 16);
  uint32_t phase = 0;
  bool ok = true, pending = false, started = false;
  auto run = [&](auto issue) {
    if (t == 0 && !withhold) {
      issue();
      commit(sb + tBar);
    }
    pending = !withhold;
    ok = __syncthreads_and(mbar_wait(sb + tBar, phase, spins));
    if (!ok) return false;
    pending = false;
    phase ^= 1u;
    fence_after();
    return true;
  };
  float lsum = 0.f;
  for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const uint32_t row = tile * 128 + t;
    {  // X row t (zeros past n: such rows get dY = 0 and add nothing)
      uint4 c0 = zero, c1 = zero;
      if (row < n) {
        const uint4* src = reinterpret_cast<const uint4*>(x + (size_t)row * IN);
        c0 = src[0];
        c1 = src[1];
      }
      *reinterpret_cast<uint4*>(sm + tX + core_off(t, 0, 4)) = c0;
      *reinterpret_cast<uint4*>(sm + tX + core_off(t, 8, 4)) = c1;
    }
    seed64(lane_base, sbias);
    sync_for_mma();
    if (!run([&] { umma(tmem, sdesc(sb + tX, 128, 512), sdesc(sb + tW1, 128, 256), idesc(128, 64), 1u); }))
      break;
    activate10(lane_base, sm + tH1, t);
    seed64(lane_base, sbias + 64);
    sync_for_mma();
    if (!run([&] {
          const uint64_t a = sdesc(sb + tH1, 128, 1280), b = sdesc(sb + tW2, 128, 1024);
#pragma unroll 1
          for (uint32_t kk = 0; kk < 4; ++kk) umma(tmem, a + 16u * kk, b + 16u * kk, idesc(128, 64), 1u);
        }))
      break;
    activate10(lane_base, sm + tH2, t);
    {
      const float4 b3 = *reinterpret_cast<const float4*>(sbias + 128);
      asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(lane_base),
                   "r"(__float_as_uint(b3.x)), "r"(__float_as_uint(b3.y)), "r"(__float_as_uint(b3.z)),
                   "r"(__float_as_uint(b3.w))
                   : "memory");
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    sync_for_mma();
    if (!run([&] {
          const uint64_t a = sdesc(sb + tH2, 128, 1280), b = sdesc(sb + tW3, 128, 1024);
#pragma unroll 1
          for (uint32_t kk = 0; kk < 4; ++kk) umma(tmem, a + 16u * kk, b + 16u * kk, idesc(128, 16), 1u);
        }))
      break;
    {  // dL/dy = 2 (y - target) / count for the 3 outputs, BF16 into dY row t
      float y[4];
      ld4(lane_base, y);
      float d[3] = {0.f, 0.f, 0.f};
      if (row < n) {
#pragma unroll
        for (int c = 0; c < OUT; ++c) {
          const float e = y[c] - target[(size_t)row * OUT + c];
          lsum = fmaf(e, e, lsum);
          d[c] = 2.f * e * inv_count;
        }
      }
      *reinterpret_cast<uint4*>(sm + tDY + core_off(t, 0, 2)) = make_uint4(pack2(d[0], d[1]), pack2(d[2], 0.f), 0u, 0u);
      *reinterpret_cast<uint4*>(sm + tDY + core_off(t, 8, 2)) = zero;
    }
    sync_for_mma();
    if (!run([&] { umma(tmem, sdesc(sb + tDY, 128, 256), sdesc(sb + tW3r, 128, 256), idesc(128, 64), 0u); }))
      break;
    grad_act(lane_base, sm + tH2, sm + tDZ2, t);  // dZ2
    sync_for_mma();
    if (!run([&] {
          {  // dH1 = dZ2 W2^T
            const uint64_t a = sdesc(sb + tDZ2, 128, 1024), b = sdesc(sb + tW2r, 128, 1024);
#pragma unroll 1
            for (uint32_t kk = 0; kk < 4; ++kk) umma(tmem, a + 16u * kk, b + 16u * kk, idesc(128, 64), kk > 0);
          }
          // G2 += dZ2^T [H1 | 1], G3 += dY^T [H2 | 1]: K = the tile's 128 samples
          const uint64_t a2 = sdesc(sb + tDZ2, 1024, 128), b2 = sdesc(sb + tH1, 1280, 128);
          const uint64_t a3 = sdesc(sb + tDY, 256, 128), b3 = sdesc(sb + tH2, 1280, 128);
#pragma unroll 1
          for (uint32_t kk = 0; kk < 8; ++kk) {
            const uint32_t acc = started || kk > 0;
            umma(tmem + cG2, a2 + 128u * kk, b2 + 160u * kk, idesc(128, 80) | kMN, acc);
            umma(tmem + cG3, a3 + 32u * kk, b3 + 160u * kk, idesc(128, 80) | kMN, acc);
          }
        }))
      break;
    grad_act(lane_base, sm + tH1, sm + tDZ1, t);  // dZ1
    sync_for_mma();
    if (!run([&] {  // G1 += dZ1^T [X | 1]
          const uint64_t a = sdesc(sb + tDZ1, 1024, 128), b = sdesc(sb + tX, 512, 128);
#pragma unroll 1
          for (uint32_t kk = 0; kk < 8; ++kk)
            umma(tmem + cG1, a + 128u * kk, b + 64u * kk, idesc(128, 32) | kMN, started || kk > 0);
        }))
      break;
    started = true;
  }
  if (ok && started) {
    // G2 row o = t (t < 64): dW2[i][o] in columns i, db2[o] in column 64;
    // G1 row i = t: dW1[j][i] in columns j, db1[i] in column 16;
    // G3 row c = t (t < 3): dW3[i][c] in columns i, db3[c] in column 64.
    // tcgen05.ld is warp-wide, so warps 0 and 1 (rows 0..63) read them.
    if (w < 2) {
#pragma unroll 1
      for (int half = 0; half < 2; ++half) {
        float v[32];
        ld32(lane_base + cG2 + 32u * half, v);
#pragma unroll 8
        for (int k = 0; k < 32; ++k) atomicAdd(grad + pW2 + (32 * half + k) * HID + t, v[k]);
      }
      float v[16];
      ld16(lane_base + cG2 + 64u, v);
      atomicAdd(grad + pB2 + t, v[0]);
      ld16(lane_base + cG1, v);
#pragma unroll
      for (int j = 0; j < IN; ++j) atomicAdd(grad + pW1 + j * HID + t, v[j]);
      float vb[16];
      ld16(lane_base + cG1 + 16u, vb);
      atomicAdd(grad + pB1 + t, vb[0]);
    }
    if (w == 0) {
#pragma unroll 1
      for (int half = 0; half < 2; ++half) {
        float v[32];
        ld32(lane_base + cG3 + 32u * half, v);
        if (t < OUT)
#pragma unroll 8
          for (int k = 0; k < 32; ++k) atomicAdd(grad + pW3 + (32 * half + k) * OUT + t, v[k]);
      }
      float v[16];
      ld16(lane_base + cG3 + 64u, v);
      if (t < OUT) atomicAdd(grad + pB3 + t, v[0]);
    }
  }
  if (!ok) {
    if (t == 0) {
      atomicOr(&g_tc_status, 2u);
      atomicAdd(loss, __int_as_float(0x7fc00000));
    }
    if (pending) __syncthreads_and(mbar_wait(sb + tBar, phase, spins));  // the MMAs still in flight
  } else {
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((t & 31u) == 0) atomicAdd(loss, lsum * inv_count);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (w == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTrCols) : "memory");
}
}  // namespace

extern "C" {

int sph_mlp_param_count(void) { return kParams; }
int sph_mlp_packed_bytes(void) { return kPackedBytes; }

int sph_mlp_pack(const float* params, void* packed, void* stream) {
  if (!params || !packed) return fail(SPH_ERR_ARG, "mlp_pack: null pointer");
  k_pack<<<26, 512, 0, (cudaStream_t)stream>>>(params, (uint16_t*)packed);
  return cuda_check(cudaGetLastError(), "mlp_pack");
}

int sph_mlp_forward(const void* packed, const uint16_t* x, uint32_t n, float* y, void* stream) {
  if (!packed || (!x && n) || (!y && n)) return fail(SPH_ERR_ARG, "mlp_forward: null pointer");
  if (n == 0) return SPH_OK;
  const uint32_t tiles = (n + 15) / 16;
  const uint32_t blocks = (uint32_t)min((long long)(tiles + 3) / 4, (long long)sm_count() * 8);
  k_forward<<<blocks, 128, kPackedBytes, (cudaStream_t)stream>>>((const uint16_t*)packed, x, n, y);
  return cuda_check(cudaGetLastError(), "mlp_forward");
}

int sph_mlp_forward_tc(const void* packed, const uint16_t* x, uint32_t n, float* y, void* stream) {
  if (!packed || (!x && n) || (!y && n)) return fail(SPH_ERR_ARG, "mlp_forward_tc: null pointer");
  if ((uintptr_t)x & 15u) return fail(SPH_ERR_ARG, "mlp_forward_tc: features not 16-byte aligned");
  if (n == 0) return SPH_OK;
  const uint32_t tiles = (n + 127) / 128;
  const uint32_t blocks = (uint32_t)min((long long)tiles, (long long)sm_count() * tcg::kBlocksPerSm);
  k_forward_tc<<<blocks, 128, tcg::kSmem, (cudaStream_t)stream>>>((const uint16_t*)packed, x, n, y,
                                                                  tcg::kTcSpins, false);
  return cuda_check(cudaGetLastError(), "mlp_forward_tc");
}

int sph_mlp_forward_tc_withheld(const void* packed, const uint16_t* x, uint32_t n, float* y, void* stream) {
  if (!packed || (!x && n) || (!y && n)) return fail(SPH_ERR_ARG, "mlp_forward_tc_withheld: null pointer");
  if ((uintptr_t)x & 15u) return fail(SPH_ERR_ARG, "mlp_forward_tc_withheld: features not 16-byte aligned");
  if (n == 0) return SPH_OK;
  const uint32_t tiles = (n + 127) / 128;
  const uint32_t blocks = (uint32_t)min((long long)tiles, (long long)sm_count() * tcg::kBlocksPerSm);
  k_forward_tc<<<blocks, 128, tcg::kSmem, (cudaStream_t)stream>>>((const uint16_t*)packed, x, n, y, 1024u,
                                                                  true);
  return cuda_check(cudaGetLastError(), "mlp_forward_tc_withheld");
}

int sph_mlp_status(uint32_t* status) {
  if (!status) return fail(SPH_ERR_ARG, "mlp_status: null pointer");
  const uint32_t zero = 0;
  SPH_TRY(cuda_check(cudaMemcpyFromSymbol(status, g_tc_status, sizeof(uint32_t)), "mlp_status"));
  return cuda_check(cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(uint32_t)), "mlp_status");
}

int sph_mlp_train_pass(const void* packed, const uint16_t* x, const float* target, uint32_t n,
                       float* grad, float* loss, void* stream) {
  if (!packed || !x || !target || !grad || !loss) return fail(SPH_ERR_ARG, "mlp_train: null pointer");
  if (n == 0) return SPH_OK;
  SPH_TRY(mlp_kernels_ready());
  const uint32_t tiles = (n + kTileRows - 1) / kTileRows;
  const uint32_t blocks = (uint32_t)min((long long)tiles, (long long)sm_count() * 3);
  k_train<<<blocks, kTrainThreads, kTrainSmem, (cudaStream_t)stream>>>(
      (const uint16_t*)packed, x, target, n, 1.0f / (3.0f * (float)n), grad, loss);
  return cuda_check(cudaGetLastError(), "mlp_train");
}

static int train_tc(const void* packed, const uint16_t* x, const float* target, uint32_t n, float* grad,
                    float* loss, void* stream, uint32_t spins, bool withhold, const char* who) {
  if (!packed || !x || !target || !grad || !loss) return fail(SPH_ERR_ARG, "%s: null pointer", who);
  if ((uintptr_t)x & 15u) return fail(SPH_ERR_ARG, "%s: features not 16-byte aligned", who);
  if (n == 0) return SPH_OK;
  static int attr = -1;
  if (attr < 0)
    attr = cuda_check(cudaFuncSetAttribute(k_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)tct::kTrSmem),
                      "mlp_train_tc: shared memory limit");
  SPH_TRY(attr);
  const uint32_t tiles = (n + 127) / 128;
  const uint32_t blocks = (uint32_t)min((long long)tiles, (long long)sm_count() * tct::kTrBlocks);
  k_train_tc<<<blocks, 128, tct::kTrSmem, (cudaStream_t)stream>>>(
      (const uint16_t*)packed, x, target, n, 1.0f / (3.0f * (float)n), grad, loss, spins, withhold);
  return cuda_check(cudaGetLastError(), who);
}

int sph_mlp_train_pass_tc(const void* packed, const uint16_t* x, const float* target, uint32_t n,
                          float* grad, float* loss, void* stream) {
  return train_tc(packed, x, target, n, grad, loss, stream, tcg::kTcSpins, false, "mlp_train_tc");
}

int sph_mlp_train_pass_tc_withheld(const void* packed, const uint16_t* x, const float* target, uint32_t n,
                                   float* grad, float* loss, void* stream) {
  return train_tc(packed, x, target, n, grad, loss, stream, 1024u, true, "mlp_train_tc_withheld");
}

int sph_mlp_adam(float* params, float* m, float* v, const float* grad, float lr, float beta1,
                 float beta2, float eps, uint32_t step, void* stream) {
  if (!params || !m || !v || !grad || step == 0) return fail(SPH_ERR_ARG, "mlp_adam: bad arguments");
  const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
  k_adam<<<(kParams + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, m, v, grad, kParams, lr,
                                                                  beta1, beta2, eps, bc1, bc2);
  return cuda_check(cudaGetLastError(), "mlp_adam");
}

}  // extern "C"

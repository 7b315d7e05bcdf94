// Learned curvature closure: a 16 -> 64 -> 64 -> 1 ReLU perceptron trained
// and evaluated on the GPU with BF16 tensor-core MMA (mma.sync m16n8k16,
// FP32 accumulate).
//
// Layout.  Parameters are one FP32 vector [W1 (64x16, row = output neuron),
// b1 (64), W2 (64x64), b2 (64), w3 (64), b3 (1)] (master copy, Adam state,
// gradient accumulators).  The matrix operands of the MMAs are BF16: the
// weights as rounded each step from the master copy, inputs and activations as
// they enter a product.  Products and sums are FP32.
//
// Fragment conventions (PTX ISA, mma.m16n8k16 .bf16): with g = lane / 4 and
// t = lane % 4, a thread holds A rows g and g + 8, columns 2t, 2t+1 (+8);
// B rows (k) 2t, 2t+1 (+8), column (n) g; C rows g, g + 8, columns 2t, 2t+1.
// So the C fragments of one layer are, after BF16 rounding, exactly the A
// fragments of the next: activations stay in registers from layer to layer.
//
// A warp owns 16 samples; a block of 8 warps one 128-sample tile.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>

#include "sbfs_gb300.h"
#include "sbfs_kernels.cuh"

using namespace sbfs;

namespace {

constexpr int NF = 16, NH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;
constexpr int TILE = 128, WARPS = 8;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p) {
  return *reinterpret_cast<const uint32_t *>(p);
}

__device__ __forceinline__ uint32_t pair2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  __nv_bfloat162 v;
  v.x = lo;
  v.y = hi;
  return *reinterpret_cast<const uint32_t *>(&v);
}

// D = A (16x16 bf16) * B (16x8 bf16) + C (16x8 f32)
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// weights in shared memory for one block
struct SmemW {
  __nv_bfloat16 W1[NH][NF];       // B operand of X W1^T: B[k][n] = W1[n][k]
  __nv_bfloat16 W2[NH][NH + 8];   // padded rows
  float b1[NH], b2[NH], w3[NH];
  float b3;
};

__device__ void load_weights(SmemW &s, const float *__restrict__ p) {
  for (int i = threadIdx.x; i < NH * NF; i += blockDim.x) s.W1[i / NF][i % NF] = __float2bfloat16_rn(p[OFF_W1 + i]);
  for (int i = threadIdx.x; i < NH * NH; i += blockDim.x) s.W2[i / NH][i % NH] = __float2bfloat16_rn(p[OFF_W2 + i]);
  for (int i = threadIdx.x; i < NH; i += blockDim.x) {
    s.b1[i] = p[OFF_B1 + i];
    s.b2[i] = p[OFF_B2 + i];
    s.w3[i] = p[OFF_W3 + i];
  }
  if (threadIdx.x == 0) s.b3 = p[OFF_B3];
}

// forward pass of 16 samples held by one warp: x_frag = A fragment of the
// input (16x16); returns the hidden C fragments (after ReLU) and the output
// of rows g and g + 8 (valid in every lane of the group)
struct Fwd {
  float h1[8][4], h2[8][4];
  float out0, out1;
};

__device__ void forward16(const SmemW &s, const uint32_t (&xa)[4], Fwd &f) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  // layer 1: 8 n-tiles, one k-step
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const int n = nt * 8 + g;
    const uint32_t b[2] = {pair2(s.W1[n][2 * t], s.W1[n][2 * t + 1]), pair2(s.W1[n][2 * t + 8], s.W1[n][2 * t + 9])};
    mma16816(d, xa, b);
    const float bb0 = s.b1[nt * 8 + 2 * t], bb1 = s.b1[nt * 8 + 2 * t + 1];
    f.h1[nt][0] = fmaxf(d[0] + bb0, 0.f);
    f.h1[nt][1] = fmaxf(d[1] + bb1, 0.f);
    f.h1[nt][2] = fmaxf(d[2] + bb0, 0.f);
    f.h1[nt][3] = fmaxf(d[3] + bb1, 0.f);
  }
  // layer 2: A = h1 (bf16, register-local re-layout), 4 k-steps
  uint32_t ha[4][4];
#pragma unroll
  for (int kt = 0; kt < 4; ++kt) {
    ha[kt][0] = pack_bf16(f.h1[2 * kt][0], f.h1[2 * kt][1]);
    ha[kt][1] = pack_bf16(f.h1[2 * kt][2], f.h1[2 * kt][3]);
    ha[kt][2] = pack_bf16(f.h1[2 * kt + 1][0], f.h1[2 * kt + 1][1]);
    ha[kt][3] = pack_bf16(f.h1[2 * kt + 1][2], f.h1[2 * kt + 1][3]);
  }
  float o0 = 0.f, o1 = 0.f;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const int n = nt * 8 + g;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const int k = kt * 16 + 2 * t;
      const uint32_t b[2] = {pair2(s.W2[n][k], s.W2[n][k + 1]), pair2(s.W2[n][k + 8], s.W2[n][k + 9])};
      mma16816(d, ha[kt], b);
    }
    const int c0 = nt * 8 + 2 * t;
    f.h2[nt][0] = fmaxf(d[0] + s.b2[c0], 0.f);
    f.h2[nt][1] = fmaxf(d[1] + s.b2[c0 + 1], 0.f);
    f.h2[nt][2] = fmaxf(d[2] + s.b2[c0], 0.f);
    f.h2[nt][3] = fmaxf(d[3] + s.b2[c0 + 1], 0.f);
    o0 = fmaf(f.h2[nt][0], s.w3[c0], fmaf(f.h2[nt][1], s.w3[c0 + 1], o0));
    o1 = fmaf(f.h2[nt][2], s.w3[c0], fmaf(f.h2[nt][3], s.w3[c0 + 1], o1));
  }
  o0 += __shfl_xor_sync(0xffffffffu, o0, 1);
  o0 += __shfl_xor_sync(0xffffffffu, o0, 2);
  o1 += __shfl_xor_sync(0xffffffffu, o1, 1);
  o1 += __shfl_xor_sync(0xffffffffu, o1, 2);
  f.out0 = o0 + s.b3;
  f.out1 = o1 + s.b3;
}

// A fragment of 16 feature rows stored row-major as bf16 [16][16]
__device__ void load_x_frag(const __nv_bfloat16 *x16, uint32_t (&xa)[4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  xa[0] = ld_pair(x16 + g * NF + 2 * t);
  xa[1] = ld_pair(x16 + (g + 8) * NF + 2 * t);
  xa[2] = ld_pair(x16 + g * NF + 2 * t + 8);
  xa[3] = ld_pair(x16 + (g + 8) * NF + 2 * t + 8);
}

struct SmemTrain {
  SmemW w;
  __nv_bfloat16 x[TILE][NF];
  __nv_bfloat16 h1[TILE][NH + 8];
  __nv_bfloat16 dz2[TILE][NH + 8];
  __nv_bfloat16 dz1[TILE][NH + 8];
  float gsum[WARPS][3][NH];  // per warp: its sums of gb1, gb2, gw3
  float gb3[WARPS];
  double loss[WARPS];
};

// gradients of the mean-square loss over a batch of `nbatch` rows, one
// 128-row tile per block: rows idx[tile*128 + r] of X (bf16 [n][16]) with
// targets y.  Block b writes its gradient to gblk[b * NPARAM ..] and its
// squared-error sum to lblk[b]; k_mlp_adam or k_mlp_reduce add the blocks in
// order.  No atomics: every sum has a fixed order, so training is
// reproducible bit for bit.
__global__ void __launch_bounds__(TILE * 2) k_mlp_grad(const float *__restrict__ params,
                                                      const __nv_bfloat16 *__restrict__ X,
                                                      const float *__restrict__ Y, const int *__restrict__ idx,
                                                      int nbatch, float *__restrict__ gblk, double *__restrict__ lblk) {
  extern __shared__ unsigned char smraw[];
  SmemTrain &s = *reinterpret_cast<SmemTrain *>(smraw);
  load_weights(s.w, params);
  const int base = blockIdx.x * TILE;
  for (int i = threadIdx.x; i < TILE * NF; i += blockDim.x) {
    const int r = i / NF, c = i % NF;
    const int row = base + r;
    s.x[r][c] = row < nbatch ? X[(size_t)idx[row] * NF + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const float invn = 2.f / (float)nbatch;
  if (warp < WARPS) {
    const int r0 = warp * 16;
    uint32_t xa[4];
    load_x_frag(&s.x[r0][0], xa);
    Fwd f;
    forward16(s.w, xa, f);
    const int ra = base + r0 + g, rb = ra + 8;
    const float ya = ra < nbatch ? Y[idx[ra]] : 0.f, yb = rb < nbatch ? Y[idx[rb]] : 0.f;
    const float ea = ra < nbatch ? f.out0 - ya : 0.f, eb = rb < nbatch ? f.out1 - yb : 0.f;
    const float da = ea * invn, db = eb * invn;  // d loss / d out
    {
      // the warp's sums over its 16 rows (the lanes t = 0 hold each row once)
      double lw = t == 0 ? (double)ea * ea + (double)eb * eb : 0.;
      float bw = t == 0 ? da + db : 0.f;
#pragma unroll
      for (int m = 1; m < 32; m <<= 1) {
        lw += __shfl_xor_sync(0xffffffffu, lw, m);
        bw += __shfl_xor_sync(0xffffffffu, bw, m);
      }
      if (lane == 0) {
        s.loss[warp] = lw;
        s.gb3[warp] = bw;
      }
    }
    // gw3 (column sums of h2 * dout), gb2, dz2 and h1 to shared memory
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int c0 = nt * 8 + 2 * t;
      float gw0 = f.h2[nt][0] * da + f.h2[nt][2] * db, gw1 = f.h2[nt][1] * da + f.h2[nt][3] * db;
      const float z0 = f.h2[nt][0] > 0.f ? da * s.w.w3[c0] : 0.f, z1 = f.h2[nt][1] > 0.f ? da * s.w.w3[c0 + 1] : 0.f;
      const float z2 = f.h2[nt][2] > 0.f ? db * s.w.w3[c0] : 0.f, z3 = f.h2[nt][3] > 0.f ? db * s.w.w3[c0 + 1] : 0.f;
      float gb0 = z0 + z2, gb1 = z1 + z3;
#pragma unroll
      for (int m = 4; m < 32; m <<= 1) {
        gw0 += __shfl_xor_sync(0xffffffffu, gw0, m);
        gw1 += __shfl_xor_sync(0xffffffffu, gw1, m);
        gb0 += __shfl_xor_sync(0xffffffffu, gb0, m);
        gb1 += __shfl_xor_sync(0xffffffffu, gb1, m);
      }
      if (g == 0) {
        s.gsum[warp][2][c0] = gw0;
        s.gsum[warp][2][c0 + 1] = gw1;
        s.gsum[warp][1][c0] = gb0;
        s.gsum[warp][1][c0 + 1] = gb1;
      }
      s.dz2[r0 + g][c0] = __float2bfloat16_rn(z0);
      s.dz2[r0 + g][c0 + 1] = __float2bfloat16_rn(z1);
      s.dz2[r0 + g + 8][c0] = __float2bfloat16_rn(z2);
      s.dz2[r0 + g + 8][c0 + 1] = __float2bfloat16_rn(z3);
      s.h1[r0 + g][c0] = __float2bfloat16_rn(f.h1[nt][0]);
      s.h1[r0 + g][c0 + 1] = __float2bfloat16_rn(f.h1[nt][1]);
      s.h1[r0 + g + 8][c0] = __float2bfloat16_rn(f.h1[nt][2]);
      s.h1[r0 + g + 8][c0 + 1] = __float2bfloat16_rn(f.h1[nt][3]);
    }
    __syncwarp();
    // dz1 = (dz2 W2) * (h1 > 0): A = dz2 rows of this warp, B[k][n] = W2[k][n]
    uint32_t za[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
      const int k = kt * 16 + 2 * t;
      za[kt][0] = ld_pair(&s.dz2[r0 + g][k]);
      za[kt][1] = ld_pair(&s.dz2[r0 + g + 8][k]);
      za[kt][2] = ld_pair(&s.dz2[r0 + g][k + 8]);
      za[kt][3] = ld_pair(&s.dz2[r0 + g + 8][k + 8]);
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      const int n = nt * 8 + g;
#pragma unroll
      for (int kt = 0; kt < 4; ++kt) {
        const int k = kt * 16 + 2 * t;
        const uint32_t b[2] = {pair2(s.w.W2[k][n], s.w.W2[k + 1][n]), pair2(s.w.W2[k + 8][n], s.w.W2[k + 9][n])};
        mma16816(d, za[kt], b);
      }
      const int c0 = nt * 8 + 2 * t;
      const float z0 = f.h1[nt][0] > 0.f ? d[0] : 0.f, z1 = f.h1[nt][1] > 0.f ? d[1] : 0.f;
      const float z2 = f.h1[nt][2] > 0.f ? d[2] : 0.f, z3 = f.h1[nt][3] > 0.f ? d[3] : 0.f;
      float gb0 = z0 + z2, gb1 = z1 + z3;
#pragma unroll
      for (int m = 4; m < 32; m <<= 1) {
        gb0 += __shfl_xor_sync(0xffffffffu, gb0, m);
        gb1 += __shfl_xor_sync(0xffffffffu, gb1, m);
      }
      if (g == 0) {
        s.gsum[warp][0][c0] = gb0;
        s.gsum[warp][0][c0 + 1] = gb1;
      }
      s.dz1[r0 + g][c0] = __float2bfloat16_rn(z0);
      s.dz1[r0 + g][c0 + 1] = __float2bfloat16_rn(z1);
      s.dz1[r0 + g + 8][c0] = __float2bfloat16_rn(z2);
      s.dz1[r0 + g + 8][c0 + 1] = __float2bfloat16_rn(z3);
    }
  }
  __syncthreads();
  // weight gradients over the tile (K = 128 samples):
  //   gW2 = dz2^T h1 (64x64: 4 m-tiles x 8 n-tiles), gW1 = dz1^T x (64x16: 4 x 2)
  if (warp < WARPS) {
    for (int tile = warp; tile < 4 * 8 + 4 * 2; tile += WARPS) {
      const bool l2 = tile < 32;
      const int mt = l2 ? tile / 8 : (tile - 32) / 2, nt = l2 ? tile % 8 : (tile - 32) % 2;
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      for (int kt = 0; kt < TILE / 16; ++kt) {
        const int k = kt * 16 + 2 * t;  // sample index
        const int m = mt * 16 + g;      // output neuron
        uint32_t a[4];
        // A[m][k] = dz[k][m] (transposed read)
        if (l2) {
          a[0] = pair2(s.dz2[k][m], s.dz2[k + 1][m]);
          a[1] = pair2(s.dz2[k][m + 8], s.dz2[k + 1][m + 8]);
          a[2] = pair2(s.dz2[k + 8][m], s.dz2[k + 9][m]);
          a[3] = pair2(s.dz2[k + 8][m + 8], s.dz2[k + 9][m + 8]);
        } else {
          a[0] = pair2(s.dz1[k][m], s.dz1[k + 1][m]);
          a[1] = pair2(s.dz1[k][m + 8], s.dz1[k + 1][m + 8]);
          a[2] = pair2(s.dz1[k + 8][m], s.dz1[k + 9][m]);
          a[3] = pair2(s.dz1[k + 8][m + 8], s.dz1[k + 9][m + 8]);
        }
        const int n = nt * 8 + g;
        uint32_t b[2];
        if (l2) {
          b[0] = pair2(s.h1[k][n], s.h1[k + 1][n]);
          b[1] = pair2(s.h1[k + 8][n], s.h1[k + 9][n]);
        } else {
          b[0] = pair2(s.x[k][n], s.x[k + 1][n]);
          b[1] = pair2(s.x[k + 8][n], s.x[k + 9][n]);
        }
        mma16816(d, a, b);
      }
      const int row = mt * 16 + g, col = nt * 8 + 2 * t;
      float *G = gblk + (size_t)blockIdx.x * NPARAM + (l2 ? OFF_W2 : OFF_W1);
      const int ld = l2 ? NH : NF;
      G[row * ld + col] = d[0];
      G[row * ld + col + 1] = d[1];
      G[(row + 8) * ld + col] = d[2];
      G[(row + 8) * ld + col + 1] = d[3];
    }
  }
  __syncthreads();
  // the bias and last-layer sums of the warps, in warp order
  float *G = gblk + (size_t)blockIdx.x * NPARAM;
  for (int i = threadIdx.x; i < 3 * NH; i += blockDim.x) {
    const int q = i / NH, c = i - q * NH;
    float v = 0.f;
    for (int w = 0; w < WARPS; ++w) v += s.gsum[w][q][c];
    G[(q == 0 ? OFF_B1 : (q == 1 ? OFF_B2 : OFF_W3)) + c] = v;
  }
  if (threadIdx.x == 0) {
    float b = 0.f;
    double l = 0.;
    for (int w = 0; w < WARPS; ++w) {
      b += s.gb3[w];
      l += s.loss[w];
    }
    G[OFF_B3] = b;
    lblk[blockIdx.x] = l;
  }
}

// sum of the nb block gradients, in block order: grad[i] = sum_b gblk[b][i];
// loss += sum_b lblk[b]
__device__ __forceinline__ float block_sum(const float *__restrict__ gblk, int nb, int i) {
  float v = 0.f;
  for (int b = 0; b < nb; ++b) v += gblk[(size_t)b * NPARAM + i];
  return v;
}
__device__ __forceinline__ void loss_sum(const double *__restrict__ lblk, int nb, double *__restrict__ loss) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double l = 0.;
    for (int b = 0; b < nb; ++b) l += lblk[b];
    *loss += l;
  }
}

__global__ void k_mlp_reduce(const float *__restrict__ gblk, const double *__restrict__ lblk, int nb,
                             float *__restrict__ grad, double *__restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  loss_sum(lblk, nb, loss);
  if (i < NPARAM) grad[i] = block_sum(gblk, nb, i);
}

// Adam step on the master parameters with the gradient summed over the nb
// blocks of k_mlp_grad (in block order); the batch's squared error is added
// to loss.  Padding columns 11..15 of W1 stay zero.
__global__ void k_mlp_adam(float *__restrict__ p, const float *__restrict__ gblk, const double *__restrict__ lblk,
                           int nb, double *__restrict__ loss, float *__restrict__ m1, float *__restrict__ m2, float lr,
                           float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  loss_sum(lblk, nb, loss);
  if (i >= NPARAM) return;
  const float gr = block_sum(gblk, nb, i);
  if (i < OFF_B1 && (i % NF) >= 11) return;
  const float a = b1 * m1[i] + (1.f - b1) * gr;
  const float b = b2 * m2[i] + (1.f - b2) * gr * gr;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a * c1) / (sqrtf(b * c2) + eps);
}

// predictions for n feature rows (bf16 [n][16]); one 16-row slice per warp
__global__ void __launch_bounds__(TILE * 2) k_mlp_predict(const float *__restrict__ params,
                                                         const __nv_bfloat16 *__restrict__ X, int n,
                                                         float *__restrict__ out) {
  extern __shared__ unsigned char smraw[];
  SmemW &w = *reinterpret_cast<SmemW *>(smraw);
  __nv_bfloat16(*xs)[16][NF] = reinterpret_cast<__nv_bfloat16(*)[16][NF]>(smraw + sizeof(SmemW));
  load_weights(w, params);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int nwarps = blockDim.x >> 5;
  for (int r0 = (blockIdx.x * nwarps + warp) * 16; r0 < n; r0 += gridDim.x * nwarps * 16) {
    for (int i = lane; i < 16 * NF; i += 32) {
      const int r = r0 + i / NF;
      xs[warp][i / NF][i % NF] = r < n ? X[(size_t)r * NF + i % NF] : __float2bfloat16_rn(0.f);
    }
    __syncwarp();
    uint32_t xa[4];
    load_x_frag(&xs[warp][0][0], xa);
    Fwd f;
    forward16(w, xa, f);
    if (t == 0) {
      if (r0 + g < n) out[r0 + g] = f.out0;
      if (r0 + g + 8 < n) out[r0 + g + 8] = f.out1;
    }
    __syncwarp();
  }
}

// 0 <= v <= 1 and lo <= v <= hi (0 < lo < hi) as integer tests on the bit
// pattern, the same answers as the FP64 comparisons (-0 counts as 0, NaN as
// out of range) without their FP64 instructions
__device__ __forceinline__ bool in_unit(double v) {
  const long long b = __double_as_longlong(v);
  return (b >= 0 && b <= 0x3FF0000000000000LL) || b == (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool in_pos_range(double v, double lo, double hi) {
  const long long b = __double_as_longlong(v);
  return b >= __double_as_longlong(lo) && b <= __double_as_longlong(hi);
}

// In the fused step: curvature of the listed interface cells from the
// network when the stencil is inside the training distribution (centre vof in
// [0.01, 0.99], all stencil values in [0, 1], |kappa dx| in [lo, hi]); the
// plain curvature already in `curv` stays otherwise.  Square cells.  Every
// lane of a warp builds one feature row (32 rows, two 16-row MMA tiles), so
// the FP64 work of the gather fills whole warps.
__global__ void __launch_bounds__(TILE * 2) k_mlp_curv(Grid g, const float *__restrict__ params,
                                                      const double *__restrict__ vof, const double *__restrict__ dvof,
                                                      const int *__restrict__ list, const int *__restrict__ count,
                                                      double *__restrict__ curv, int *__restrict__ used, float lo,
                                                      float hi) {
  pdl_entry();
  extern __shared__ unsigned char smraw[];
  SmemW &w = *reinterpret_cast<SmemW *>(smraw);
  __nv_bfloat16(*xs)[32][NF] = reinterpret_cast<__nv_bfloat16(*)[32][NF]>(smraw + sizeof(SmemW));
  load_weights(w, params);
  __syncthreads();
  // batches: case blockIdx.z has its own list and rows z ny .. z ny + ny - 1
  list += (size_t)blockIdx.z * g.nx * g.ny;
  count += blockIdx.z;
  const int zr = blockIdx.z * g.ny;
  const int n = *count;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const double2 *dv = reinterpret_cast<const double2 *>(dvof);
  const size_t q = g.p2 / 2;
  int nused = 0;
  for (int e0 = (blockIdx.x * nwarps + warp) * 32; e0 < n; e0 += gridDim.x * nwarps * 32) {
    bool ok = false;
    int cell = -1;
    {
      const int e = e0 + lane;
      float fr[NF];
      for (int c = 0; c < NF; ++c) fr[c] = 0.f;
      if (e < n) {
        cell = list[e];
        const int rc = cell / g.nx, I = cell - rc * g.nx + 1;
        const int J = rc + 1, r = rc + zr;
        ok = true;
        for (int dy = -1; dy <= 1; ++dy) {
          const int rr = wrap(J + dy, g.ny) + zr;
          for (int dx = -1; dx <= 1; ++dx) {
            const double v = vof[(size_t)rr * g.p1 + I + dx];
            ok = ok && in_unit(v);
            fr[(dy + 1) * 3 + (dx + 1)] = (float)v;
          }
        }
        ok = ok && in_pos_range(vof[(size_t)r * g.p1 + I], 0.01, 0.99);
        // the solver's cell normal: sum of the four unit corner normals, normalised
        const int rp = wrap(J + 1, g.ny) + zr;
        const double2 d00 = dv[(size_t)r * q + (I - 1)], d10 = dv[(size_t)r * q + I];
        const double2 d01 = dv[(size_t)rp * q + (I - 1)], d11 = dv[(size_t)rp * q + I];
        const double mx = ((d00.x + d10.x) + d01.x) + d11.x, my = ((d00.y + d10.y) + d01.y) + d11.y;
        const double inv = inv_norm(mx * mx + my * my);
        fr[9] = (float)(mx * inv);
        fr[10] = (float)(my * inv);
      }
      for (int c = 0; c < NF; ++c) xs[warp][lane][c] = __float2bfloat16_rn(fr[c]);
    }
    __syncwarp();
    // tile h holds rows 16 h .. 16 h + 15; their outputs come out in lanes
    // 4 gq .. 4 gq + 3 (rows gq and gq + 8); lane L takes row L
    float o = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint32_t xa[4];
      load_x_frag(&xs[warp][16 * h][0], xa);
      Fwd f;
      forward16(w, xa, f);
      const float oa = __shfl_sync(0xffffffffu, f.out0, (lane & 7) * 4);
      const float ob = __shfl_sync(0xffffffffu, f.out1, (lane & 7) * 4);
      if ((lane >> 4) == h) o = (lane & 8) ? ob : oa;
    }
    if (ok) {
      const float a = fabsf(o);
      if (a >= lo && a <= hi) {
        const int rc = cell / g.nx, I = cell - rc * g.nx + 1;
        curv[(size_t)(rc + zr) * g.p1 + I] = (double)o * g.idx;
        ++nused;
      }
    }
    __syncwarp();
  }
  if (used) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) nused += __shfl_xor_sync(0xffffffffu, nused, m);
    if (lane == 0 && nused) atomicAdd(used, nused);
  }
}

// ---- host side state of the closure
float *g_params = nullptr, *g_grad = nullptr, *g_m1 = nullptr, *g_m2 = nullptr;
double *g_loss = nullptr;
// per-block gradients and squared errors of k_mlp_grad (g_nblk blocks)
float *g_gblk = nullptr;
double *g_lblk = nullptr;
int g_nblk = 0;
int *g_used = nullptr;
int g_adam_t = 0;
char g_mlp_err[256];

int mlp_fail(const char *what, cudaError_t e) {
  snprintf(g_mlp_err, sizeof(g_mlp_err), "%s: %s", what, cudaGetErrorString(e));
  return 1;
}

#define MCK(call)                                   \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return mlp_fail(#call, e_); \
  } while (0)

int ensure_alloc() {
  if (g_params) return 0;
  MCK(cudaMalloc(&g_params, sizeof(float) * NPARAM));
  MCK(cudaMalloc(&g_grad, sizeof(float) * NPARAM));
  MCK(cudaMalloc(&g_m1, sizeof(float) * NPARAM));
  MCK(cudaMalloc(&g_m2, sizeof(float) * NPARAM));
  MCK(cudaMalloc(&g_loss, sizeof(double)));
  MCK(cudaMalloc(&g_used, sizeof(int)));
  MCK(cudaMemset(g_params, 0, sizeof(float) * NPARAM));
  MCK(cudaMemset(g_grad, 0, sizeof(float) * NPARAM));
  MCK(cudaMemset(g_m1, 0, sizeof(float) * NPARAM));
  MCK(cudaMemset(g_m2, 0, sizeof(float) * NPARAM));
  MCK(cudaMemset(g_used, 0, sizeof(int)));
  MCK(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemTrain)));
  return 0;
}

int ensure_blocks(int nb) {
  if (nb <= g_nblk) return 0;
  if (g_gblk) cudaFree(g_gblk);
  if (g_lblk) cudaFree(g_lblk);
  g_gblk = nullptr;
  g_lblk = nullptr;
  g_nblk = 0;
  MCK(cudaMalloc(&g_gblk, sizeof(float) * NPARAM * (size_t)nb));
  MCK(cudaMalloc(&g_lblk, sizeof(double) * (size_t)nb));
  g_nblk = nb;
  return 0;
}

// weights and per warp (8 warps) up to 32 feature rows
size_t smem_infer() { return sizeof(SmemW) + sizeof(__nv_bfloat16) * 8 * 32 * NF; }

}  // namespace

// ---- entry points used by the solver (sbfs_api.cu)
namespace sbfs {
bool mlp_ready() { return g_params != nullptr; }
// the closure's range in |kappa dx|: the curvatures of the training circles,
// radii 2 .. 128 cells
float g_kappa_lo = 0.0078125f, g_kappa_hi = 0.5f;
unsigned g_mlp_epoch = 0;  // bumped whenever the closure's parameters or range change
void mlp_range(float *lo, float *hi) {
  *lo = g_kappa_lo;
  *hi = g_kappa_hi;
}
void launch_mlp_curv(cudaStream_t s, const Grid &g, const Bufs &b) {
  launch_pdl(k_mlp_curv, dim3(max(2, (2 * 152 + g.nc - 1) / g.nc), 1, g.nc), 256, smem_infer(), s,
      g, g_params, b.vof, b.dvof, b.ilist, b.icount, b.curv, g_used, g_kappa_lo, g_kappa_hi);
}
}  // namespace sbfs

extern "C" {

const char *sbfs_mlp_last_error(void) { return g_mlp_err; }

int sbfs_mlp_set_range(double lo, double hi) {
  if (!(lo >= 0. && hi > lo)) {
    snprintf(g_mlp_err, sizeof(g_mlp_err), "bad closure range [%g, %g]", lo, hi);
    return 1;
  }
  sbfs::g_kappa_lo = (float)lo;
  sbfs::g_kappa_hi = (float)hi;
  ++sbfs::g_mlp_epoch;
  return 0;
}

int sbfs_mlp_nparams(void) { return NPARAM; }

int sbfs_mlp_set_params(const float *host, int n) {
  if (n != NPARAM) return mlp_fail("sbfs_mlp_set_params: wrong parameter count", cudaErrorInvalidValue);
  if (ensure_alloc()) return 1;
  MCK(cudaMemcpy(g_params, host, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  MCK(cudaMemset(g_m1, 0, sizeof(float) * NPARAM));
  MCK(cudaMemset(g_m2, 0, sizeof(float) * NPARAM));
  MCK(cudaMemset(g_grad, 0, sizeof(float) * NPARAM));
  g_adam_t = 0;
  ++sbfs::g_mlp_epoch;
  return 0;
}

int sbfs_mlp_get_params(float *host, int n) {
  if (n != NPARAM || !g_params) return mlp_fail("sbfs_mlp_get_params: no parameters", cudaErrorInvalidValue);
  MCK(cudaMemcpy(host, g_params, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return 0;
}

// gradient of the mean-square loss over rows idx[0..n) (device arrays);
// returns it to host `grad_out` (NPARAM floats) and the loss
int sbfs_mlp_gradient(const void *X, const float *Y, const int *idx, int n, float *grad_out, double *loss_out) {
  if (ensure_alloc()) return 1;
  const int nb = (n + TILE - 1) / TILE;
  if (ensure_blocks(nb)) return 1;
  MCK(cudaMemset(g_loss, 0, sizeof(double)));
  k_mlp_grad<<<nb, TILE * 2, sizeof(SmemTrain)>>>(g_params, static_cast<const __nv_bfloat16 *>(X), Y, idx, n, g_gblk,
                                                   g_lblk);
  k_mlp_reduce<<<(NPARAM + 255) / 256, 256>>>(g_gblk, g_lblk, nb, g_grad, g_loss);
  MCK(cudaGetLastError());
  MCK(cudaMemcpy(grad_out, g_grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  double l = 0.;
  MCK(cudaMemcpy(&l, g_loss, sizeof(double), cudaMemcpyDeviceToHost));
  *loss_out = l / n;
  return 0;
}

// one epoch of Adam steps over batches idx[b*batch .. (b+1)*batch) of the
// device permutation `idx` (length n); mean loss over the epoch returned
int sbfs_mlp_train_epoch(const void *X, const float *Y, const int *idx, int n, int batch, float lr,
                         double *mean_loss) {
  if (ensure_alloc()) return 1;
  const int nb = (batch + TILE - 1) / TILE;
  if (ensure_blocks(nb)) return 1;
  ++sbfs::g_mlp_epoch;  // the parameters change
  MCK(cudaMemset(g_loss, 0, sizeof(double)));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int off = 0; off + batch <= n; off += batch) {
    k_mlp_grad<<<nb, TILE * 2, sizeof(SmemTrain)>>>(g_params, static_cast<const __nv_bfloat16 *>(X), Y, idx + off,
                                                     batch, g_gblk, g_lblk);
    ++g_adam_t;
    const float c1 = 1.f / (1.f - powf(b1, (float)g_adam_t)), c2 = 1.f / (1.f - powf(b2, (float)g_adam_t));
    k_mlp_adam<<<(NPARAM + 255) / 256, 256>>>(g_params, g_gblk, g_lblk, nb, g_loss, g_m1, g_m2, lr, b1, b2, eps, c1,
                                              c2);
  }
  MCK(cudaGetLastError());
  double l = 0.;
  MCK(cudaMemcpy(&l, g_loss, sizeof(double), cudaMemcpyDeviceToHost));
  *mean_loss = l / (double)((n / batch) * batch);
  return 0;
}

int sbfs_mlp_predict(const void *X, int n, float *out) {
  if (ensure_alloc()) return 1;
  k_mlp_predict<<<2 * 152, 256, smem_infer()>>>(g_params, static_cast<const __nv_bfloat16 *>(X), n, out);
  MCK(cudaGetLastError());
  MCK(cudaDeviceSynchronize());
  return 0;
}

// number of interface cells whose curvature came from the network since the
// last call (the rest used the plain curvature)
int sbfs_mlp_take_usage(long long *used) {
  if (!g_used) {
    *used = 0;
    return 0;
  }
  int h = 0;
  MCK(cudaMemcpy(&h, g_used, sizeof(int), cudaMemcpyDeviceToHost));
  MCK(cudaMemset(g_used, 0, sizeof(int)));
  *used = h;
  return 0;
}

}  // extern "C"

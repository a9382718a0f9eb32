// fst_hybrid.cu — learned smoothness classifier routing faces between WENO5
// and the linear optimal-weight upwind flux (FST_MODE_HYBRID), and the CUDA
// kernels that train it.
//
// Per face (the 6-cell WENO stencil c-2..c+3 across face c+1/2):
//   features  5 undivided differences of density, pressure, face-normal
//             velocity and the largest mass fraction, each normalised by the
//             sum of the 5 magnitudes plus a small floor (20 values in [-1,1])
//   label     1 (needs WENO) when, for density or pressure on either upwind
//             stencil, max(beta_k) / min(beta_k) of the WENO5 smoothness
//             indicators exceeds a ratio
//   network   20 -> 32 -> 32 -> 1, ReLU, ReLU, sigmoid
//
// Inference: each warp classifies 32 faces with BF16 mma.sync m16n8k16 on the
// tensor cores (FP32 accumulation).  The first layer's accumulator fragments
// are the second layer's A fragments (C -> A register reuse), so only the
// feature tile goes through shared memory.  One classification per time step
// (stage 1), reused by stage 2; every `audit_every` steps the step runs full
// WENO and the classifier's decisions are compared with the labels.
//
// Training: minibatch Adam on FP32 CUDA cores.  A block takes 64 samples,
// one per thread, runs forward and backward in registers with the weights in
// shared memory, stages activations and deltas in shared memory, and then
// forms the weight gradients as sums over its 64 samples (one thread per
// weight), adding them to the global gradient with one atomicAdd per weight
// per block.  Gradients are checked against a float64 restatement
// (oracle/mlp_oracle.py, tests/test_gpu_hybrid.py).
#include <cuda_bf16.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "fst_mixed_dev.cuh"

using namespace fstm;

namespace {

constexpr int NI = FST_MLP_IN;   // 20
constexpr int NH = FST_MLP_HID;  // 32
constexpr int KP = 40;           // padded row stride (bf16) of the tensor-core tiles
// packed parameter offsets
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NH, NP = OB3 + 1;
static_assert(NP == FST_MLP_PARAMS, "parameter packing");

struct MlpDev {
  float p[NP];
  __nv_bfloat16 w1[NH][KP];  // [n][k], k >= 20 zero
  __nv_bfloat16 w2[NH][KP];  // [n][k], k >= 32 zero
};

struct HybridState {
  MlpDev* mlp;
  float* ymax;
  float threshold;
  float label_ratio;
};

// ---------------------------------------------------------------------------
// features and labels
// ---------------------------------------------------------------------------
__device__ __forceinline__ void diffs5(const float a[6], float floor_abs, float* out) {
  float d[5], s = floor_abs;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    d[k] = a[k + 1] - a[k];
    s += fabsf(d[k]);
  }
  const float r = __fdividef(1.0f, s);
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const float v = d[k] * r;
    out[k] = isfinite(v) ? v : 0.f;  // a non-finite state gives no feature signal
  }
}

__device__ __forceinline__ void face_features(const Geo& g, const MixedView& M, const float* ymax,
                                              long long c, int f, float* feat) {
  const long long sf = f == 0 ? 1 : f == 1 ? g.sy : g.sz;
  float r[6], p[6], u[6], y[6];
  const float* un = M.vel + g.sv * f;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const long long cc = c + (k - 2) * sf;
    r[k] = __ldg(M.rho + cc);
    p[k] = M.pp ? __ldg(M.pp + cc) : d2f(__ldg(M.p + cc));
    u[k] = __ldg(un + cc);
    y[k] = __ldg(ymax + cc);
  }
  const float rm = 0.5f * (fabsf(r[2]) + fabsf(r[3])), pm = 0.5f * (fabsf(p[2]) + fabsf(p[3]));
  const float vs = sqrtf(fmaxf(pm, 1e-30f) / fmaxf(rm, 1e-30f));  // velocity scale
  diffs5(r, 1e-3f * rm + 1e-30f, feat + 0);
  diffs5(p, 1e-3f * pm + 1e-30f, feat + 5);
  diffs5(u, 1e-3f * vs + 1e-30f, feat + 10);
  diffs5(y, 1e-3f, feat + 15);
}

__device__ __forceinline__ float beta_ratio(float f1, float f2, float f3, float f4, float f5) {
  float a1 = f1 - 2.0f * f2 + f3, a2 = f1 - 4.0f * f2 + 3.0f * f3;
  const float b1 = (13.0f / 12.0f) * a1 * a1 + 0.25f * a2 * a2;
  a1 = f2 - 2.0f * f3 + f4;
  a2 = f2 - f4;
  const float b2 = (13.0f / 12.0f) * a1 * a1 + 0.25f * a2 * a2;
  a1 = f3 - 2.0f * f4 + f5;
  a2 = 3.0f * f3 - 4.0f * f4 + f5;
  const float b3 = (13.0f / 12.0f) * a1 * a1 + 0.25f * a2 * a2;
  const float eps = 1e-10f * f3 * f3 + 1e-30f;
  return __fdividef(fmaxf(b1, fmaxf(b2, b3)) + eps, fminf(b1, fminf(b2, b3)) + eps);
}

__device__ __forceinline__ bool face_label(const Geo& g, const MixedView& M, long long c, int f,
                                           float ratio) {
  const long long sf = f == 0 ? 1 : f == 1 ? g.sy : g.sz;
  float r[6], p[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const long long cc = c + (k - 2) * sf;
    r[k] = __ldg(M.rho + cc);
    p[k] = M.pp ? __ldg(M.pp + cc) : d2f(__ldg(M.p + cc));
  }
  const float q = fmaxf(fmaxf(beta_ratio(r[0], r[1], r[2], r[3], r[4]),
                              beta_ratio(r[5], r[4], r[3], r[2], r[1])),
                        fmaxf(beta_ratio(p[0], p[1], p[2], p[3], p[4]),
                              beta_ratio(p[5], p[4], p[3], p[2], p[1])));
  return q > ratio;
}

// largest mass fraction per cell (all cells)
__global__ void k_ymax(Geo g, const float* __restrict__ Q, const float* __restrict__ rho,
                       float* __restrict__ ymax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.ngi) return;
  const long long c = (long long)i + g.sy * blockIdx.y + g.sz * blockIdx.z;
  const int s0 = g.ndim + 1;
  float m = 0.f;
  for (int s = 0; s < g.ns; ++s) m = fmaxf(m, Q[c + g.sv * (s0 + s)]);
  ymax[c] = m / rho[c];
}

// ---------------------------------------------------------------------------
// MLP: FP32 reference forward (CUDA cores) and BF16 tensor-core forward
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + __expf(-z)); }

// logits of one sample with FP32 weights in shared memory
__device__ __forceinline__ float mlp_fp32(const float* __restrict__ W, const float* x, float* h1,
                                          float* h2) {
#pragma unroll 4
  for (int n = 0; n < NH; ++n) {
    float a = W[OB1 + n];
#pragma unroll
    for (int k = 0; k < NI; ++k) a += W[OW1 + n * NI + k] * x[k];
    h1[n] = fmaxf(a, 0.f);
  }
#pragma unroll 4
  for (int n = 0; n < NH; ++n) {
    float a = W[OB2 + n];
#pragma unroll
    for (int k = 0; k < NH; ++k) a += W[OW2 + n * NH + k] * h1[k];
    h2[n] = fmaxf(a, 0.f);
  }
  float z = W[OB3];
#pragma unroll
  for (int k = 0; k < NH; ++k) z += W[OW3 + k] * h2[k];
  return z;
}

__device__ __forceinline__ void mma_bf16(float* d, unsigned a0, unsigned a1, unsigned a2,
                                         unsigned a3, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const unsigned*>(&v);
}

__device__ __forceinline__ unsigned ld32(const __nv_bfloat16* p) {
  return *reinterpret_cast<const unsigned*>(p);
}

// Classifier probability of the calling lane's face for all 32 lanes of the
// warp (all lanes must call).  F: this warp's [32][KP] bf16 feature tile;
// out: 32 floats of shared memory for this warp.
__device__ float mlp_warp_tc(const MlpDev& W, __nv_bfloat16 (*F)[KP], float* out,
                             const float* feat) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
#pragma unroll
  for (int k = 0; k < 32; k += 2) {
    const float v0 = k < NI ? feat[k] : 0.f, v1 = k + 1 < NI ? feat[k + 1] : 0.f;
    *reinterpret_cast<unsigned*>(&F[lane][k]) = pack_bf16(v0, v1);
  }
  __syncwarp();
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const int r0 = 16 * mt + g, r1 = r0 + 8;
    float acc[4][4];
#pragma unroll
    for (int t = 0; t < 4; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int kc = 16 * s + 2 * q;
      const unsigned a0 = ld32(&F[r0][kc]), a1 = ld32(&F[r1][kc]), a2 = ld32(&F[r0][kc + 8]),
                     a3 = ld32(&F[r1][kc + 8]);
#pragma unroll
      for (int t = 0; t < 4; ++t)
        mma_bf16(acc[t], a0, a1, a2, a3, ld32(&W.w1[8 * t + g][kc]), ld32(&W.w1[8 * t + g][kc + 8]));
    }
    // bias + ReLU; the accumulator layout of two n-tiles is the A layout of
    // one k-step of the next layer
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int n = 8 * t + 2 * q;
      acc[t][0] = fmaxf(acc[t][0] + W.p[OB1 + n], 0.f);
      acc[t][1] = fmaxf(acc[t][1] + W.p[OB1 + n + 1], 0.f);
      acc[t][2] = fmaxf(acc[t][2] + W.p[OB1 + n], 0.f);
      acc[t][3] = fmaxf(acc[t][3] + W.p[OB1 + n + 1], 0.f);
    }
    float acc2[4][4];
#pragma unroll
    for (int t = 0; t < 4; ++t) acc2[t][0] = acc2[t][1] = acc2[t][2] = acc2[t][3] = 0.f;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const unsigned a0 = pack_bf16(acc[2 * s][0], acc[2 * s][1]);
      const unsigned a1 = pack_bf16(acc[2 * s][2], acc[2 * s][3]);
      const unsigned a2 = pack_bf16(acc[2 * s + 1][0], acc[2 * s + 1][1]);
      const unsigned a3 = pack_bf16(acc[2 * s + 1][2], acc[2 * s + 1][3]);
      const int kc = 16 * s + 2 * q;
#pragma unroll
      for (int t = 0; t < 4; ++t)
        mma_bf16(acc2[t], a0, a1, a2, a3, ld32(&W.w2[8 * t + g][kc]), ld32(&W.w2[8 * t + g][kc + 8]));
    }
    float zlo = 0.f, zhi = 0.f;
#pragma unroll
    for (int t = 0; t < 4; ++t)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int n = 8 * t + 2 * q + j;
        const float w3 = W.p[OW3 + n], b2 = W.p[OB2 + n];
        zlo += fmaxf(acc2[t][j] + b2, 0.f) * w3;
        zhi += fmaxf(acc2[t][2 + j] + b2, 0.f) * w3;
      }
    zlo += __shfl_xor_sync(0xffffffffu, zlo, 1);
    zlo += __shfl_xor_sync(0xffffffffu, zlo, 2);
    zhi += __shfl_xor_sync(0xffffffffu, zhi, 1);
    zhi += __shfl_xor_sync(0xffffffffu, zhi, 2);
    if (q == 0) {
      out[r0] = sigmoidf_(zlo + W.p[OB3]);
      out[r1] = sigmoidf_(zhi + W.p[OB3]);
    }
  }
  __syncwarp();
  const float o = out[lane];
  __syncwarp();
  return o;
}

// ---------------------------------------------------------------------------
// classification of every face of the face box (3 faces per index in 3D)
// ---------------------------------------------------------------------------
constexpr int CB = 128;  // threads per classify block (4 warps)

__global__ void __launch_bounds__(CB) k_classify(Geo g, MixedView M, HybridState H,
                                                 unsigned char* __restrict__ smap,
                                                 unsigned long long* __restrict__ cnt, int audit) {
  __shared__ MlpDev W;
  __shared__ __nv_bfloat16 F[CB / 32][32][KP];
  __shared__ float outb[CB / 32][32];
  for (int q = threadIdx.x; q < (int)(sizeof(MlpDev) / 4); q += CB)
    reinterpret_cast<float*>(&W)[q] = reinterpret_cast<const float*>(H.mlp)[q];
  __syncthreads();
  const int nfx = g.nci + 1, nfy = g.ncj + 1;
  const long long nf = (long long)nfx * nfy * (g.ndim == 3 ? g.nck + 1 : 1);
  const long long t = (long long)blockIdx.x * CB + threadIdx.x;
  const bool active = t < nf;
  int i = 0, j = 0, k = 0;
  if (active) {
    i = g.ng - 1 + (int)(t % nfx);
    j = g.ng - 1 + (int)((t / nfx) % nfy);
    k = g.ndim == 3 ? g.ng - 1 + (int)(t / ((long long)nfx * nfy)) : 0;
  }
  const long long c = (long long)i + g.sy * j + g.sz * k;
  const int wid = threadIdx.x >> 5;
  unsigned long long nfaces = 0, nweno = 0, nlab = 0, nmiss = 0;
  for (int f = 0; f < g.ndim; ++f) {
    float feat[NI];
    if (active) face_features(g, M, H.ymax, c, f, feat);
    else
      for (int q = 0; q < NI; ++q) feat[q] = 0.f;
    const float prob = mlp_warp_tc(W, F[wid], outb[wid], feat);
    if (!active) continue;
    // faces adjacent to an interior cell (the ones the RHS uses)
    const bool in_i = f == 0 || (i >= g.ng && i < g.ngi - g.ng);
    const bool in_j = f == 1 || (j >= g.ng && j < g.ngj - g.ng);
    const bool in_k = g.ndim == 2 || f == 2 || (k >= g.ng && k < g.ngk - g.ng);
    const bool used = in_i && in_j && in_k;
    const bool weno = prob > H.threshold;
    smap[c * 3 + f] = weno ? 0 : 1;
    if (used) {
      ++nfaces;
      nweno += weno;
      if (audit) {
        const bool lab = face_label(g, M, c, f, H.label_ratio);
        nlab += lab;
        nmiss += lab && !weno;
      }
    }
  }
  // warp-aggregated counters
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nfaces += __shfl_xor_sync(0xffffffffu, nfaces, o);
    nweno += __shfl_xor_sync(0xffffffffu, nweno, o);
    nlab += __shfl_xor_sync(0xffffffffu, nlab, o);
    nmiss += __shfl_xor_sync(0xffffffffu, nmiss, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (audit) {
      atomicAdd(&cnt[2], nfaces);
      atomicAdd(&cnt[3], nlab);
      atomicAdd(&cnt[4], nmiss);
    } else {
      atomicAdd(&cnt[0], nfaces);
      atomicAdd(&cnt[1], nweno);
    }
  }
}

// features + labels of every face (training data)
__global__ void k_features(Geo g, MixedView M, const float* __restrict__ ymax, float ratio,
                           float* __restrict__ out, unsigned char* __restrict__ lab,
                           long long cap) {
  const int nfx = g.nci + 1, nfy = g.ncj + 1;
  const long long nf = (long long)nfx * nfy * (g.ndim == 3 ? g.nck + 1 : 1);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf) return;
  const int i = g.ng - 1 + (int)(t % nfx);
  const int j = g.ng - 1 + (int)((t / nfx) % nfy);
  const int k = g.ndim == 3 ? g.ng - 1 + (int)(t / ((long long)nfx * nfy)) : 0;
  const long long c = (long long)i + g.sy * j + g.sz * k;
  for (int f = 0; f < g.ndim; ++f) {
    const long long row = t * g.ndim + f;
    if (row >= cap) return;
    float feat[NI];
    face_features(g, M, ymax, c, f, feat);
    for (int q = 0; q < NI; ++q) out[row * NI + q] = feat[q];
    lab[row] = face_label(g, M, c, f, ratio) ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// training
// ---------------------------------------------------------------------------
constexpr int TB = 64;  // samples (threads) per training block (fits 48 KB static smem)

// Gradient of the weighted BCE loss over samples [base, base + TB) of the
// dataset, added to grad; loss sum added to loss.
__global__ void __launch_bounds__(TB) k_mlp_grad(const float* __restrict__ X,
                                                 const unsigned char* __restrict__ Y, long long n,
                                                 long long begin, long long end,
                                                 const float* __restrict__ params, float pos_w,
                                                 float* __restrict__ grad, float* __restrict__ loss) {
  __shared__ float W[NP];
  __shared__ float sX[TB][NI + 1];
  __shared__ float sH1[TB][NH + 1], sH2[TB][NH + 1], sD1[TB][NH + 1], sD2[TB][NH + 1];
  __shared__ float sDz[TB];
  for (int q = threadIdx.x; q < NP; q += TB) W[q] = params[q];
  __syncthreads();
  const long long s = begin + (long long)blockIdx.x * TB + threadIdx.x;
  const bool ok = s < end && s < n;
  float x[NI], h1[NH], h2[NH];
  for (int q = 0; q < NI; ++q) x[q] = ok ? X[s * NI + q] : 0.f;
  const float z = mlp_fp32(W, x, h1, h2);
  const float y = ok ? (float)Y[s] : 0.f;
  // weighted BCE with logits: w*(softplus(z) - y*z), w = pos_w for y = 1
  const float wgt = ok ? (y > 0.5f ? pos_w : 1.0f) : 0.f;
  const float sp = z > 0.f ? z + log1pf(__expf(-z)) : log1pf(__expf(z));
  const float l = wgt * (sp - y * z);
  const float dz = wgt * (sigmoidf_(z) - y);
  // backward through the two hidden layers
  float d2[NH];
  for (int k = 0; k < NH; ++k) d2[k] = h2[k] > 0.f ? dz * W[OW3 + k] : 0.f;
  float d1[NH];
  for (int k = 0; k < NH; ++k) {
    float a = 0.f;
    for (int n2 = 0; n2 < NH; ++n2) a += W[OW2 + n2 * NH + k] * d2[n2];
    d1[k] = h1[k] > 0.f ? a : 0.f;
  }
  const int t = threadIdx.x;
  for (int q = 0; q < NI; ++q) sX[t][q] = x[q];
  for (int q = 0; q < NH; ++q) {
    sH1[t][q] = h1[q];
    sH2[t][q] = h2[q];
    sD1[t][q] = d1[q];
    sD2[t][q] = d2[q];
  }
  sDz[t] = dz;
  // block loss
  float lw = l;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lw += __shfl_xor_sync(0xffffffffu, lw, o);
  if ((t & 31) == 0) atomicAdd(loss, lw);
  __syncthreads();
  // weight gradients: sums over the block's samples, one thread per weight
  for (int w = t; w < NP; w += TB) {
    float a = 0.f;
    if (w < OB1) {
      const int n1 = w / NI, k = w % NI;
      for (int r = 0; r < TB; ++r) a += sD1[r][n1] * sX[r][k];
    } else if (w < OW2) {
      const int n1 = w - OB1;
      for (int r = 0; r < TB; ++r) a += sD1[r][n1];
    } else if (w < OB2) {
      const int n2 = (w - OW2) / NH, k = (w - OW2) % NH;
      for (int r = 0; r < TB; ++r) a += sD2[r][n2] * sH1[r][k];
    } else if (w < OW3) {
      const int n2 = w - OB2;
      for (int r = 0; r < TB; ++r) a += sD2[r][n2];
    } else if (w < OB3) {
      const int k = w - OW3;
      for (int r = 0; r < TB; ++r) a += sDz[r] * sH2[r][k];
    } else {
      for (int r = 0; r < TB; ++r) a += sDz[r];
    }
    atomicAdd(&grad[w], a);
  }
}

__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ grad, float scale, float lr, float b1, float b2,
                       float c1, float c2) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= NP) return;
  const float gw = grad[w] * scale;
  m[w] = b1 * m[w] + (1.f - b1) * gw;
  v[w] = b2 * v[w] + (1.f - b2) * gw * gw;
  p[w] -= lr * (m[w] / c1) / (sqrtf(v[w] / c2) + 1e-8f);
}

__global__ void k_forward(const float* __restrict__ X, long long n, const float* __restrict__ params,
                          float* __restrict__ out) {
  __shared__ float W[NP];
  for (int q = threadIdx.x; q < NP; q += blockDim.x) W[q] = params[q];
  __syncthreads();
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float x[NI], h1[NH], h2[NH];
  for (int q = 0; q < NI; ++q) x[q] = X[s * NI + q];
  out[s] = sigmoidf_(mlp_fp32(W, x, h1, h2));
}

// parameters -> MlpDev (FP32 copy and BF16 tensor-core tiles)
__global__ void k_pack(const float* __restrict__ params, MlpDev* __restrict__ W) {
  for (int q = threadIdx.x; q < NP; q += blockDim.x) W->p[q] = params[q];
  for (int q = threadIdx.x; q < NH * KP; q += blockDim.x) {
    const int n = q / KP, k = q % KP;
    W->w1[n][k] = __float2bfloat16_rn(k < NI ? params[OW1 + n * NI + k] : 0.f);
    W->w2[n][k] = __float2bfloat16_rn(k < NH ? params[OW2 + n * NH + k] : 0.f);
  }
}

__global__ void k_forward_tc(const float* __restrict__ X, long long n, const MlpDev* __restrict__ Wg,
                             float* __restrict__ out) {
  __shared__ MlpDev W;
  __shared__ __nv_bfloat16 F[CB / 32][32][KP];
  __shared__ float outb[CB / 32][32];
  for (int q = threadIdx.x; q < (int)(sizeof(MlpDev) / 4); q += CB)
    reinterpret_cast<float*>(&W)[q] = reinterpret_cast<const float*>(Wg)[q];
  __syncthreads();
  const long long s = (long long)blockIdx.x * CB + threadIdx.x;
  float feat[NI];
  for (int q = 0; q < NI; ++q) feat[q] = s < n ? X[s * NI + q] : 0.f;
  const int wid = threadIdx.x >> 5;
  const float prob = mlp_warp_tc(W, F[wid], outb[wid], feat);
  if (s < n) out[s] = prob;
}

__global__ void k_scale(float* __restrict__ a, int n, float f) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) a[q] *= f;
}

inline unsigned cdivh(long long a, int b) { return (unsigned)((a + b - 1) / b); }

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int fst_hybrid_alloc(const fst_config& cf, const Geo& g, MixedBufs& b, const fst_alloc_fn& alloc) {
  b.hyb_active = false;
  b.audit_every = cf.audit_every;
  b.classify_every = cf.classify_every > 1 ? cf.classify_every : 1;
  (void)g;  // the map and ymax follow the primitive arrays' geometry
  int rc = alloc((void**)&b.smooth, (size_t)b.gq.sv * 3);
  if (!rc) rc = alloc((void**)&b.ymax, sizeof(float) * (size_t)b.gq.sv);
  if (!rc) rc = alloc(&b.mlp, sizeof(MlpDev));
  b.threshold = 0.5f;
  b.label_ratio = 20.0f;
  return rc;
}

int fst_hybrid_classify(const Geo& g, const Phys& P, const MixedBufs& b, const MixedView& M,
                        cudaStream_t st, Prof* prof, const unsigned char** smooth, bool audit) {
  (void)P;
  int n = 0;
  const dim3 pg(cdivh(g.ngi, 256), g.ngj, g.ngk);
  FST_LAUNCH(prof, "ymax", st, n, k_ymax<<<pg, 256, 0, st>>>(g, M.Q, M.rho, b.ymax));
  HybridState H{(MlpDev*)b.mlp, b.ymax, b.threshold, b.label_ratio};
  const long long nf = (long long)(g.nci + 1) * (g.ncj + 1) * (g.ndim == 3 ? g.nck + 1 : 1);
  FST_LAUNCH(prof, "classify", st, n,
             k_classify<<<cdivh(nf, CB), CB, 0, st>>>(g, M, H, b.smooth, b.counters, audit ? 1 : 0));
  *smooth = b.smooth;
  return n;
}

int fst_hybrid_features_impl(const Geo& g, const MixedBufs& b, const MixedView& M, float* out,
                             unsigned char* lab, size_t cap, float ratio, size_t* count,
                             cudaStream_t st) {
  const dim3 pg(cdivh(g.ngi, 256), g.ngj, g.ngk);
  float* ymax = b.ymax;
  k_ymax<<<pg, 256, 0, st>>>(g, M.Q, M.rho, ymax);
  const long long nf = (long long)(g.nci + 1) * (g.ncj + 1) * (g.ndim == 3 ? g.nck + 1 : 1);
  k_features<<<cdivh(nf, 128), 128, 0, st>>>(g, M, ymax, ratio, out, lab, (long long)cap);
  const size_t total = (size_t)nf * g.ndim;
  *count = total < cap ? total : cap;
  return cudaGetLastError() == cudaSuccess ? FST_OK : FST_ERR_CUDA;
}

int fst_hybrid_pack(MixedBufs& b, const float* h_params, cudaStream_t st) {
  MlpDev* W = reinterpret_cast<MlpDev*>(b.mlp);
  cudaError_t e = cudaMemcpyAsync(W->p, h_params, NP * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return FST_ERR_CUDA;
  k_pack<<<1, 256, 0, st>>>(W->p, W);  // rewrites p with itself, fills the BF16 tiles
  e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? FST_OK : FST_ERR_CUDA;
}

extern "C" {

int fst_mlp_grad(const float* X, const unsigned char* Y, size_t n, const float* params,
                 float pos_weight, float* grad, float* h_loss, void* stream) {
  if (!X || !Y || !params || !grad || n == 0) return FST_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  float* dloss = nullptr;
  if (cudaMallocAsync((void**)&dloss, sizeof(float), st) != cudaSuccess) return FST_ERR_OOM;
  cudaMemsetAsync(grad, 0, NP * sizeof(float), st);
  cudaMemsetAsync(dloss, 0, sizeof(float), st);
  k_mlp_grad<<<cdivh((long long)n, TB), TB, 0, st>>>(X, Y, (long long)n, 0, (long long)n, params,
                                                     pos_weight, grad, dloss);
  k_scale<<<cdivh(NP, 256), 256, 0, st>>>(grad, NP, 1.0f / (float)n);  // mean over samples
  float h = 0.f;
  cudaMemcpyAsync(&h, dloss, sizeof(float), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(dloss, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return FST_ERR_CUDA;
  if (h_loss) *h_loss = h / (float)n;
  return FST_OK;
}

int fst_mlp_train_epoch(const float* X, const unsigned char* Y, size_t n, float* params, float* m,
                        float* v, int* step, float lr, float pos_weight, int batch,
                        float* h_mean_loss, void* stream) {
  if (!X || !Y || !params || !m || !v || !step || n == 0 || batch < TB) return FST_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  float* work = nullptr;  // gradient + loss accumulator
  if (cudaMallocAsync((void**)&work, (NP + 1) * sizeof(float), st) != cudaSuccess)
    return FST_ERR_OOM;
  float* grad = work;
  float* dloss = work + NP;
  cudaMemsetAsync(dloss, 0, sizeof(float), st);
  const float b1 = 0.9f, b2 = 0.999f;
  for (size_t s0 = 0; s0 < n; s0 += (size_t)batch) {
    const size_t s1 = s0 + (size_t)batch < n ? s0 + (size_t)batch : n;
    cudaMemsetAsync(grad, 0, NP * sizeof(float), st);
    k_mlp_grad<<<cdivh((long long)(s1 - s0), TB), TB, 0, st>>>(
        X, Y, (long long)n, (long long)s0, (long long)s1, params, pos_weight, grad, dloss);
    *step += 1;
    const float c1 = 1.f - powf(b1, (float)*step), c2 = 1.f - powf(b2, (float)*step);
    k_adam<<<cdivh(NP, 256), 256, 0, st>>>(params, m, v, grad, 1.0f / (float)(s1 - s0), lr, b1,
                                          b2, c1, c2);
  }
  float h = 0.f;
  cudaMemcpyAsync(&h, dloss, sizeof(float), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(work, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return FST_ERR_CUDA;
  if (h_mean_loss) *h_mean_loss = h / (float)n;
  return FST_OK;
}

int fst_mlp_forward(const float* X, size_t n, const float* params, float* out, int tensor_cores,
                    void* stream) {
  if (!X || !params || !out) return FST_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  if (!tensor_cores) {
    k_forward<<<cdivh((long long)n, 128), 128, 0, st>>>(X, (long long)n, params, out);
  } else {
    MlpDev* W = nullptr;
    if (cudaMallocAsync((void**)&W, sizeof(MlpDev), st) != cudaSuccess) return FST_ERR_OOM;
    k_pack<<<1, 256, 0, st>>>(params, W);
    k_forward_tc<<<cdivh((long long)n, CB), CB, 0, st>>>(X, (long long)n, W, out);
    cudaFreeAsync(W, st);
  }
  cudaError_t e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? FST_OK : FST_ERR_CUDA;
}

}  // extern "C"

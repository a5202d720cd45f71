// Kernels of the learned initial-guess network (3-D convolutional
// encoder-decoder on periodic grids): 3x3x3 periodic convolutions (forward,
// input gradient, weight and bias gradients), 2x average pooling and nearest
// upsampling with their adjoints, SiLU, the normalised squared-error loss and
// the Adam update.  No reference counterpart (the reference has no learned
// guess).
//
// Layout: activations [C][D][H][W] FP32 (one structure at a time); weights
// [C_out][C_in][27] in BF16 for the arithmetic (FP32 master copies are kept
// for the optimiser), tap = (dz+1)*9 + (dy+1)*3 + (dx+1); FP32 accumulation.
// The input gradient is the same convolution with the weights transposed in
// (C_out, C_in) and the taps reversed (tap -> 26 - tap), so one kernel does
// both.  All reductions are per-CTA partials combined in a fixed order
// (deterministic).
#include <cuda_bf16.h>
#include <math.h>

#include "plan.h"

namespace {

constexpr int kVox = 256;     // output voxels per CTA (one per thread)
constexpr int kCiT = 8;       // input channels staged per round

// kCoT output channels per CTA (32, or 16 / 4 for narrower layers such as
// the 1-channel head, so no CTA computes unused channels)
template <int kCoT>
__global__ void __launch_bounds__(kVox) k_conv3d(const float* __restrict__ in, int cin,
                                                  const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                                  float* __restrict__ out, int cout, int D, int H, int W,
                                                  int transposed) {
  __shared__ __align__(16) float ws[kCiT * 27 * kCoT];
  const int HW = H * W;
  const int64_t N = (int64_t)D * HW;
  const int64_t v = (int64_t)blockIdx.x * kVox + threadIdx.x;
  const int co0 = blockIdx.y * kCoT;
  const bool ok = v < N;
  int oz[3], oy[3], ox[3];
  {
    const int z = ok ? (int)(v / HW) : 0, r = ok ? (int)(v % HW) : 0;
    const int y = r / W, x = r % W;
    oz[0] = ((z + D - 1) % D) * HW; oz[1] = z * HW; oz[2] = ((z + 1) % D) * HW;
    oy[0] = ((y + H - 1) % H) * W; oy[1] = y * W; oy[2] = ((y + 1) % H) * W;
    ox[0] = (x + W - 1) % W; ox[1] = x; ox[2] = (x + 1) % W;
  }
  float acc[kCoT];
#pragma unroll
  for (int c = 0; c < kCoT; ++c) acc[c] = (bias && co0 + c < cout) ? bias[co0 + c] : 0.0f;
  for (int ci0 = 0; ci0 < cin; ci0 += kCiT) {
    __syncthreads();
    // weights of this round as ws[ci][tap][co] (FP32)
    for (int i = threadIdx.x; i < kCiT * 27 * kCoT; i += kVox) {
      const int c = i % kCoT, t = (i / kCoT) % 27, ci = i / (kCoT * 27);
      const int cg = ci0 + ci, og = co0 + c;
      float val = 0.0f;
      if (cg < cin && og < cout) {
        const int64_t idx = transposed ? ((int64_t)cg * cout + og) * 27 + (26 - t) : ((int64_t)og * cin + cg) * 27 + t;
        val = __bfloat162float(w[idx]);
      }
      ws[i] = val;
    }
    __syncthreads();
    if (!ok) continue;
    const int nci = min(kCiT, cin - ci0);
    for (int ci = 0; ci < nci; ++ci) {
      const float* base = in + (int64_t)(ci0 + ci) * N;
      const float4* wrow = reinterpret_cast<const float4*>(ws + ci * 27 * kCoT);
#pragma unroll
      for (int t = 0; t < 27; ++t) {
        const float x = __ldg(base + oz[t / 9] + oy[(t / 3) % 3] + ox[t % 3]);
#pragma unroll
        for (int q = 0; q < kCoT / 4; ++q) {
          const float4 w4 = wrow[t * (kCoT / 4) + q];
          acc[4 * q] += w4.x * x;
          acc[4 * q + 1] += w4.y * x;
          acc[4 * q + 2] += w4.z * x;
          acc[4 * q + 3] += w4.w * x;
        }
      }
    }
  }
  if (!ok) return;
#pragma unroll
  for (int c = 0; c < kCoT; ++c)
    if (co0 + c < cout) out[(int64_t)(co0 + c) * N + v] = acc[c];
}

// The same convolution for grids too small to fill the GPU with k_conv3d's
// (256 voxels x 32 channels) CTAs -- the network's coarsest levels, a few
// hundred voxels with 64-128 channels.  One CTA per (output channel, 64
// voxels); its 256 threads are 64 voxels x 4 groups of input channels (the
// warp's weight loads are one broadcast, its input loads contiguous), and the
// four groups' sums are added in a fixed order (deterministic).
constexpr int kKsVox = 64, kKsGroups = 4;

__global__ void __launch_bounds__(kKsVox * kKsGroups) k_conv3d_ks(const float* __restrict__ in, int cin,
                                                                  const __nv_bfloat16* __restrict__ w,
                                                                  const float* __restrict__ bias,
                                                                  float* __restrict__ out, int cout, int D, int H,
                                                                  int W, int transposed) {
  __shared__ float red[kKsGroups][kKsVox];
  const int HW = H * W;
  const int64_t N = (int64_t)D * HW;
  const int lane = threadIdx.x % kKsVox, grp = threadIdx.x / kKsVox;
  const int64_t v = (int64_t)blockIdx.x * kKsVox + lane;
  const int co = blockIdx.y;
  float acc = 0.0f;
  if (v < N) {
    const int z = (int)(v / HW), r = (int)(v % HW);
    const int y = r / W, x = r % W;
    const int oz[3] = {((z + D - 1) % D) * HW, z * HW, ((z + 1) % D) * HW};
    const int oy[3] = {((y + H - 1) % H) * W, y * W, ((y + 1) % H) * W};
    const int ox[3] = {(x + W - 1) % W, x, (x + 1) % W};
    const int c0 = (int)((int64_t)cin * grp / kKsGroups), c1 = (int)((int64_t)cin * (grp + 1) / kKsGroups);
    for (int ci = c0; ci < c1; ++ci) {
      const float* base = in + (int64_t)ci * N;
      const int64_t w0 = transposed ? ((int64_t)ci * cout + co) * 27 : ((int64_t)co * cin + ci) * 27;
#pragma unroll
      for (int t = 0; t < 27; ++t) {
        const float xv = __ldg(base + oz[t / 9] + oy[(t / 3) % 3] + ox[t % 3]);
        const float wv = __bfloat162float(w[w0 + (transposed ? 26 - t : t)]);
        acc += wv * xv;
      }
    }
  }
  red[grp][lane] = acc;
  __syncthreads();
  if (grp == 0 && v < N) {
    float s = bias ? bias[co] : 0.0f;
#pragma unroll
    for (int g = 0; g < kKsGroups; ++g) s += red[g][lane];
    out[(int64_t)co * N + v] = s;
  }
}

// weight gradient of one (co, ci) pair over all voxels: gw[co][ci][tap] =
// sum_v gout[co][v] in[ci][v + d_tap]; the ci == 0 CTAs also reduce the bias
// gradient gb[co] = sum_v gout[co][v]
constexpr int kWgThreads = 256;

__global__ void __launch_bounds__(kWgThreads) k_conv3d_wgrad(const float* __restrict__ in, int cin,
                                                              const float* __restrict__ gout, int cout, int D, int H,
                                                              int W, float* __restrict__ gw, float* __restrict__ gb) {
  const int co = blockIdx.x / cin, ci = blockIdx.x % cin;
  const int HW = H * W;
  const int64_t N = (int64_t)D * HW;
  const float* g = gout + (int64_t)co * N;
  const float* x = in + (int64_t)ci * N;
  float acc[28];
#pragma unroll
  for (int t = 0; t < 28; ++t) acc[t] = 0.0f;
  for (int64_t v = threadIdx.x; v < N; v += kWgThreads) {
    const int z = (int)(v / HW), r = (int)(v % HW), y = r / W, xx = r % W;
    const int oz[3] = {((z + D - 1) % D) * HW, z * HW, ((z + 1) % D) * HW};
    const int oy[3] = {((y + H - 1) % H) * W, y * W, ((y + 1) % H) * W};
    const int ox[3] = {(xx + W - 1) % W, xx, (xx + 1) % W};
    const float gv = __ldg(g + v);
#pragma unroll
    for (int t = 0; t < 27; ++t) acc[t] += gv * __ldg(x + oz[t / 9] + oy[(t / 3) % 3] + ox[t % 3]);
    acc[27] += gv;
  }
  __shared__ float red[kWgThreads / 32][28];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < 28; ++t) {
    float s = acc[t];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[warp][t] = s;
  }
  __syncthreads();
  if (threadIdx.x < 28) {
    float s = 0.0f;
    for (int w2 = 0; w2 < kWgThreads / 32; ++w2) s += red[w2][threadIdx.x];
    if (threadIdx.x < 27) gw[((int64_t)co * cin + ci) * 27 + threadIdx.x] = s;
    else if (gb && ci == 0) gb[co] = s;
  }
}

// pointwise operations
enum { PW_SILU = 0, PW_SILU_BWD = 1, PW_ADD = 2, PW_POOL2 = 3, PW_POOL2_BWD = 4, PW_UP2 = 5, PW_UP2_BWD = 6,
       PW_UPLIN = 7, PW_UPLIN_BWD = 8 };

// Periodic 2x linear upsampling in cell-centred coordinates (the inverse
// pairing of the 2x average pool): fine point i of an axis sits at coarse
// coordinate i/2 - 1/4, so it takes 3/4 of coarse point i/2 and 1/4 of its
// neighbour on the side of i (i/2 - 1 for even i, i/2 + 1 for odd i),
// periodically; trilinear = the product over the three axes.
__device__ __forceinline__ void uplin_axis(int i, int n2, int& j0, int& j1) {
  j0 = i >> 1;
  j1 = (i & 1) ? (j0 + 1 == n2 ? 0 : j0 + 1) : (j0 == 0 ? n2 - 1 : j0 - 1);
}

__global__ void k_pointwise(int op, int64_t n, const float* __restrict__ a, const float* __restrict__ b,
                            float* __restrict__ out, int C, int D, int H, int W) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    switch (op) {
      case PW_SILU: {  // out = a sigma(a)
        const float z = a[i];
        out[i] = z / (1.0f + __expf(-z));
        break;
      }
      case PW_SILU_BWD: {  // out = b * d/dz silu(a)
        const float z = a[i], s = 1.0f / (1.0f + __expf(-z));
        out[i] = b[i] * s * (1.0f + z * (1.0f - s));
        break;
      }
      case PW_ADD:
        out[i] = a[i] + b[i];
        break;
      case PW_POOL2: {  // out (C, D/2, H/2, W/2) from a (C, D, H, W)
        const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
        const int x = (int)(i % w2), y = (int)((i / w2) % h2), z = (int)((i / ((int64_t)w2 * h2)) % d2);
        const int64_t c = i / ((int64_t)w2 * h2 * d2);
        const float* s = a + c * (int64_t)D * H * W;
        float acc = 0.0f;
        for (int dz = 0; dz < 2; ++dz)
          for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) acc += s[((int64_t)(2 * z + dz) * H + 2 * y + dy) * W + 2 * x + dx];
        out[i] = 0.125f * acc;
        break;
      }
      case PW_POOL2_BWD: {  // out (C, D, H, W) = a (C, D/2, H/2, W/2) / 8 at the parent
        const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)((i / ((int64_t)W * H)) % D);
        const int64_t c = i / ((int64_t)W * H * D);
        out[i] = 0.125f * a[((c * (D / 2) + z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2];
        break;
      }
      case PW_UP2: {  // out (C, D, H, W) from a (C, D/2, H/2, W/2)
        const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)((i / ((int64_t)W * H)) % D);
        const int64_t c = i / ((int64_t)W * H * D);
        out[i] = a[((c * (D / 2) + z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2];
        break;
      }
      case PW_UPLIN: {  // out (C, D, H, W) from a (C, D/2, H/2, W/2), periodic trilinear
        const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)((i / ((int64_t)W * H)) % D);
        const int64_t c = i / ((int64_t)W * H * D);
        const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
        int x0, x1, y0, y1, z0, z1;
        uplin_axis(x, w2, x0, x1);
        uplin_axis(y, h2, y0, y1);
        uplin_axis(z, d2, z0, z1);
        const float* s = a + c * (int64_t)d2 * h2 * w2;
        const int zz[2] = {z0, z1}, yy[2] = {y0, y1}, xx[2] = {x0, x1};
        const float wt[2] = {0.75f, 0.25f};
        float acc = 0.0f;
        for (int dz = 0; dz < 2; ++dz)
          for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx)
              acc += wt[dz] * wt[dy] * wt[dx] * s[((int64_t)zz[dz] * h2 + yy[dy]) * w2 + xx[dx]];
        out[i] = acc;
        break;
      }
      case PW_UPLIN_BWD: {  // out (C, D/2, H/2, W/2): the adjoint of PW_UPLIN applied to a (C, D, H, W)
        const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
        const int x = (int)(i % w2), y = (int)((i / w2) % h2), z = (int)((i / ((int64_t)w2 * h2)) % d2);
        const int64_t c = i / ((int64_t)w2 * h2 * d2);
        const float* s = a + c * (int64_t)D * H * W;
        // coarse j feeds fine 2j and 2j+1 (3/4), 2j-1 and 2j+2 (1/4), periodically
        const float wt[4] = {0.25f, 0.75f, 0.75f, 0.25f};
        float acc = 0.0f;
        for (int dz = 0; dz < 4; ++dz) {
          const int fz = (2 * z - 1 + dz + D) % D;
          for (int dy = 0; dy < 4; ++dy) {
            const int fy = (2 * y - 1 + dy + H) % H;
            for (int dx = 0; dx < 4; ++dx) {
              const int fx = (2 * x - 1 + dx + W) % W;
              acc += wt[dz] * wt[dy] * wt[dx] * s[((int64_t)fz * H + fy) * W + fx];
            }
          }
        }
        out[i] = acc;
        break;
      }
      case PW_UP2_BWD: {  // out (C, D/2, H/2, W/2) = sum of the 8 children in a (C, D, H, W)
        const int w2 = W / 2, h2 = H / 2, d2 = D / 2;
        const int x = (int)(i % w2), y = (int)((i / w2) % h2), z = (int)((i / ((int64_t)w2 * h2)) % d2);
        const int64_t c = i / ((int64_t)w2 * h2 * d2);
        const float* s = a + c * (int64_t)D * H * W;
        float acc = 0.0f;
        for (int dz = 0; dz < 2; ++dz)
          for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) acc += s[((int64_t)(2 * z + dz) * H + 2 * y + dy) * W + 2 * x + dx];
        out[i] = acc;
        break;
      }
    }
  }
}

constexpr int kRedBlocks = 256;

// loss = sum (p - t)^2 / sum t^2 (per-CTA partials of both sums), grad = 2 (p - t) / sum t^2
__global__ void k_sqerr_partial(int64_t n, const float* __restrict__ p, const float* __restrict__ t,
                                double* __restrict__ part) {
  double se = 0.0, st = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = (double)p[i] - (double)t[i];
    se += d * d;
    st += (double)t[i] * (double)t[i];
  }
  __shared__ double red[2][8];
  se = warp_sum(se);
  st = warp_sum(st);
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = se; red[1][threadIdx.x >> 5] = st; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += red[0][w]; b += red[1][w]; }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
}

__global__ void k_sqerr_final(int64_t n, const float* __restrict__ p, const float* __restrict__ t,
                              const double* __restrict__ part, int nb, float* __restrict__ grad,
                              double* __restrict__ loss_out) {
  __shared__ double s_se, s_st;
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < nb; ++i) { a += part[2 * i]; b += part[2 * i + 1]; }
    s_se = a;
    s_st = b;
    if (blockIdx.x == 0 && loss_out) *loss_out = a / b;
  }
  __syncthreads();
  const float scale = (float)(2.0 / s_st);
  if (grad)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      grad[i] = scale * (p[i] - t[i]);
}

__global__ void k_adam(int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

__global__ void k_to_bf16(int64_t n, const float* __restrict__ a, __nv_bfloat16* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16(a[i]);
}

int blocks_of(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

}  // namespace

extern "C" {

int gbofdft_nn_conv3d(const float* in, int cin, const void* w_bf16, const float* bias, float* out, int cout, int D,
                      int H, int W, int transposed, void* stream) {
  GB_REQUIRE(in && w_bf16 && out, "nn_conv3d: null argument");
  GB_REQUIRE(cin > 0 && cout > 0 && D > 0 && H > 0 && W > 0, "nn_conv3d: bad shape");
  GB_REQUIRE(!transposed || !bias, "nn_conv3d: the transposed (input-gradient) convolution has no bias");
  const int64_t N = (int64_t)D * H * W;
  const unsigned nv = (unsigned)((N + kVox - 1) / kVox);
  const __nv_bfloat16* wb = reinterpret_cast<const __nv_bfloat16*>(w_bf16);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t tiles = cout <= 16 ? 1 : (cout + 31) / 32;
  if ((int64_t)nv * tiles < 76 && cout <= 65535) {
    // too few k_conv3d CTAs for the GPU: one CTA per (channel, 64 voxels)
    const dim3 grid((unsigned)((N + kKsVox - 1) / kKsVox), (unsigned)cout);
    k_conv3d_ks<<<grid, kKsVox * kKsGroups, 0, st>>>(in, cin, wb, bias, out, cout, D, H, W, transposed);
  } else if (cout <= 4) {
    k_conv3d<4><<<dim3(nv, 1), kVox, 0, st>>>(in, cin, wb, bias, out, cout, D, H, W, transposed);
  } else if (cout <= 16) {
    k_conv3d<16><<<dim3(nv, 1), kVox, 0, st>>>(in, cin, wb, bias, out, cout, D, H, W, transposed);
  } else {
    k_conv3d<32><<<dim3(nv, (unsigned)((cout + 31) / 32)), kVox, 0, st>>>(in, cin, wb, bias, out, cout, D, H, W,
                                                                         transposed);
  }
  GB_CHECK_LAUNCH();
  gb_count_launch();
  return GBOFDFT_OK;
}

int gbofdft_nn_conv3d_wgrad(const float* in, int cin, const float* gout, int cout, int D, int H, int W, float* gw,
                            float* gb, void* stream) {
  GB_REQUIRE(in && gout && gw, "nn_conv3d_wgrad: null argument");
  GB_REQUIRE(cin > 0 && cout > 0 && D > 0 && H > 0 && W > 0, "nn_conv3d_wgrad: bad shape");
  k_conv3d_wgrad<<<cout * cin, kWgThreads, 0, (cudaStream_t)stream>>>(in, cin, gout, cout, D, H, W, gw, gb);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  return GBOFDFT_OK;
}

int gbofdft_nn_pointwise(int op, const float* a, const float* b, float* out, int C, int D, int H, int W,
                         void* stream) {
  GB_REQUIRE(a && out && op >= PW_SILU && op <= PW_UPLIN_BWD, "nn_pointwise: bad arguments");
  GB_REQUIRE(!(op == PW_SILU_BWD || op == PW_ADD) || b, "nn_pointwise: second operand missing");
  const bool half_out = op == PW_POOL2 || op == PW_UP2_BWD || op == PW_UPLIN_BWD;
  GB_REQUIRE(!(op >= PW_POOL2) || (D % 2 == 0 && H % 2 == 0 && W % 2 == 0),
             "nn_pointwise: pooling needs even extents (got %d %d %d)", D, H, W);
  // (D, H, W) are the fine extents for the resampling operations
  const int64_t n = (int64_t)C * D * H * W / (half_out ? 8 : 1);
  k_pointwise<<<blocks_of(n), 256, 0, (cudaStream_t)stream>>>(op, n, a, b, out, C, D, H, W);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  return GBOFDFT_OK;
}

int gbofdft_nn_sqerr(const float* pred, const float* target, int64_t n, float* grad, double* loss_dev, void* work,
                     void* stream) {
  GB_REQUIRE(pred && target && work && n > 0, "nn_sqerr: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  double* part = reinterpret_cast<double*>(work);
  k_sqerr_partial<<<kRedBlocks, 256, 0, st>>>(n, pred, target, part);
  GB_CHECK_LAUNCH();
  k_sqerr_final<<<blocks_of(n), 256, 0, st>>>(n, pred, target, part, kRedBlocks, grad, loss_dev);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  gb_count_launch();
  return GBOFDFT_OK;
}

int gbofdft_nn_sqerr_work_bytes(int64_t* bytes) {
  GB_REQUIRE(bytes, "nn_sqerr_work_bytes: null argument");
  *bytes = sizeof(double) * 2 * kRedBlocks;
  return GBOFDFT_OK;
}

int gbofdft_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, int64_t n, double lr, double b1,
                    double b2, double eps, int step, void* stream) {
  GB_REQUIRE(w && g && m && v && n > 0 && step >= 1, "nn_adam: bad arguments");
  const float c1 = (float)(1.0 - pow(b1, step)), c2 = (float)(1.0 - pow(b2, step));
  k_adam<<<blocks_of(n), 256, 0, (cudaStream_t)stream>>>(n, w, g, m, v, reinterpret_cast<__nv_bfloat16*>(w_bf16),
                                                         (float)lr, (float)b1, (float)b2, (float)eps, c1, c2);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  return GBOFDFT_OK;
}

int gbofdft_nn_to_bf16(const float* a, void* b, int64_t n, void* stream) {
  GB_REQUIRE(a && b && n > 0, "nn_to_bf16: bad arguments");
  k_to_bf16<<<blocks_of(n), 256, 0, (cudaStream_t)stream>>>(n, a, reinterpret_cast<__nv_bfloat16*>(b));
  GB_CHECK_LAUNCH();
  gb_count_launch();
  return GBOFDFT_OK;
}

}  // extern "C"

// dvc_cnn.cu — the learned initial-guess proposer (no reference counterpart).
//
// A small 3D CNN reads the reference and correlate patches (32^3 voxels each,
// centred on the ROI point, normalised to zero mean and unit variance) and
// proposes the point's 12 search parameters (u v w, phi the psi, exx eyy ezz
// exy eyz exz) in place of the reference's start estimate and coarse grid
// (Search::starting_param + trgrid_global, Core/Search.cpp:277-377,934-1043).
//
//   conv 2->16, 3^3, stride 2, pad 1, ReLU      32^3 -> 16^3
//   conv 16->32                                  16^3 -> 8^3
//   conv 32->64                                  8^3  -> 4^3
//   conv 64->96                                  4^3  -> 2^3
//   dense 768 -> 128, ReLU; dense 128 -> 12
//
// Outputs are the parameters divided by fixed scales (kScale). Training: mean
// squared error against parameters the plain search converged to, Adam.
// Every kernel here is hand-written FP32 (forward, both backward passes, the
// optimizer); weight gradients are block reductions in a fixed order, so a
// training step is deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/dvc_gpu.h"
#include "dvc_internal.h"

namespace {

constexpr int kP = 32;  // patch side
constexpr int kNL = 4;  // conv layers
const int kCin[kNL] = {2, 16, 32, 64};
constexpr int kCinC[kNL] = {2, 16, 32, 64};
const int kCout[kNL] = {16, 32, 64, 96};
const int kDin[kNL] = {32, 16, 8, 4};
constexpr int kF0 = 768, kF1 = 128, kF2 = 12;
// parameter scales: translations (voxels), rotations (rad), strains
const float kScale[12] = {10.f, 10.f, 10.f, 0.05f, 0.05f, 0.05f, 0.02f, 0.02f, 0.02f, 0.02f, 0.02f, 0.02f};

struct Layout {
  size_t w[kNL + 2], b[kNL + 2], total;
  Layout() {
    size_t o = 0;
    for (int l = 0; l < kNL; l++) {
      w[l] = o;
      o += (size_t)kCout[l] * kCin[l] * 27;
      b[l] = o;
      o += kCout[l];
    }
    w[kNL] = o;
    o += (size_t)kF1 * kF0;
    b[kNL] = o;
    o += kF1;
    w[kNL + 1] = o;
    o += (size_t)kF2 * kF1;
    b[kNL + 1] = o;
    o += kF2;
    total = o;
  }
};
const Layout kLay;

// ------------------------------------------------------------- kernels ---
// conv forward, register-blocked: each thread computes one output voxel of
// one sample for 8 consecutive output channels; the block's 8 channels of
// weights sit in shared memory as [ci][tap][8] (two 16-byte loads per tap,
// the same address for every lane). blockIdx.y = channel group.
constexpr int kCoG = 8;
__global__ void __launch_bounds__(256) conv_fwd8(const float *__restrict__ in, const float *__restrict__ w,
                                                 const float *__restrict__ bias, float *__restrict__ out, int B,
                                                 int Cin, int Cout, int Din) {
  extern __shared__ float4 sw4[];  // [Cin * 27][2]
  const int Do = Din / 2, n3 = Do * Do * Do, din3 = Din * Din * Din;
  const int co0 = blockIdx.y * kCoG;
  float *sw = reinterpret_cast<float *>(sw4);
  for (int e = threadIdx.x; e < Cin * 27 * kCoG; e += blockDim.x) {
    const int c = e % kCoG, ck = e / kCoG;  // ck = ci * 27 + k
    sw[e] = w[((size_t)(co0 + c) * Cin) * 27 + ck];
  }
  __syncthreads();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * n3) return;
  const int o = (int)(t % n3), b = (int)(t / n3);
  const int ox = o % Do, oy = (o / Do) % Do, oz = o / (Do * Do);
  float acc[kCoG];
#pragma unroll
  for (int c = 0; c < kCoG; c++) acc[c] = bias[co0 + c];
  // taps inside the volume (padding 1): ranges per axis
  const int z0 = 2 * oz - 1, y0 = 2 * oy - 1, x0 = 2 * ox - 1;
  for (int ci = 0; ci < Cin; ci++) {
    const float *ib = in + ((size_t)b * Cin + ci) * din3;
    const float4 *wk = sw4 + (size_t)ci * 27 * 2;
#pragma unroll
    for (int k = 0; k < 27; k++) {
      const int kx = k % 3, ky = (k / 3) % 3, kz = k / 9;
      const int iz = z0 + kz, iy = y0 + ky, ix = x0 + kx;
      if (iz < 0 || iy < 0 || ix < 0 || iz >= Din || iy >= Din || ix >= Din) continue;
      const float v = ib[((size_t)iz * Din + iy) * Din + ix];
      const float4 wa = wk[2 * k], wb = wk[2 * k + 1];
      acc[0] = fmaf(wa.x, v, acc[0]);
      acc[1] = fmaf(wa.y, v, acc[1]);
      acc[2] = fmaf(wa.z, v, acc[2]);
      acc[3] = fmaf(wa.w, v, acc[3]);
      acc[4] = fmaf(wb.x, v, acc[4]);
      acc[5] = fmaf(wb.y, v, acc[5]);
      acc[6] = fmaf(wb.z, v, acc[6]);
      acc[7] = fmaf(wb.w, v, acc[7]);
    }
  }
#pragma unroll
  for (int c = 0; c < kCoG; c++) out[((size_t)b * Cout + co0 + c) * n3 + o] = fmaxf(acc[c], 0.f);
}


// ---------------------------------------------- tensor-core convolution ---
// The forward convolutions as implicit GEMMs on the 5th-generation tensor
// cores: D[m][n] = sum_k A[m][k] B[n][k], m an output voxel of the batch
// (128 per tile), n an output channel, k a (tap, input channel) pair, padded
// with zeros to a multiple of 16. A is gathered by the threads (im2col,
// padding 1, stride 2): for the first layer from the FP32 patches, k = ci *
// 27 + tap, rounded to BF16 element by element; for the others from the
// previous layer's BF16 output in channels-last order, k = tap * Cin + ci, so
// eight consecutive k (one tap, eight channels) are one 16-byte load stored
// as it is. B is the weights in BF16 in the same k order (conv_weights_bf16).
// Both are
// written to shared memory in the canonical K-major layout without swizzle
// (8 x 16-byte core matrices; K-adjacent core matrices 128 bytes apart,
// row-group-adjacent ones 256 bytes apart), one 16-wide K slice per MMA.
// One thread issues tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128,
// N = Cout) into a TMEM accumulator; K runs in chunks of 64 through two
// shared-memory stages, the gather of chunk c + 1 overlapping the MMAs of
// chunk c (tcgen05.commit onto the stage's mbarrier). The epilogue reads the
// accumulator with tcgen05.ld (warp w: lanes 32w..32w+31, one output voxel
// per thread), adds the bias, applies ReLU and stores the activation: BF16
// channels-last for the next convolution (16-byte stores) and, when given,
// FP32 in the layout of the FP32 kernels (the dense layer's input, the
// backward pass). Each CTA walks tiles grid-stride. Every
// mbarrier wait is bounded; one that gives up records an error (tc_error)
// that dvc_cnn_forward reports.
__device__ int tc_error = 0;

constexpr int kTcM = 128, kTcKC = 64, kTcThreads = 128;

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t phase) {
  for (long long i = 0; i < (1LL << 24); i++) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(bar), "r"(phase)
        : "memory");
    if (ok) return true;
    if (i > 32) __nanosleep(32);
  }
  atomicExch(&tc_error, 1);
  return false;
}

// shared-memory matrix descriptor: no swizzle, K-major; LBO = byte distance
// of K-adjacent core matrices, SBO = of row-group-adjacent ones; version 1
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

template <int CIN, int COUT, int DIN>
__global__ void __launch_bounds__(kTcThreads) conv_fwd_tc(const float *__restrict__ in,
                                                          const __nv_bfloat16 *__restrict__ in_b,
                                                          const __nv_bfloat16 *__restrict__ wb,
                                                          const float *__restrict__ bias,
                                                          float *__restrict__ out,
                                                          __nv_bfloat16 *__restrict__ out_b, long long m_total) {
  constexpr bool IN_B = CIN % 8 == 0;  // BF16 channels-last input, k = tap * CIN + ci
  static_assert(!IN_B || (CIN & (CIN - 1)) == 0, "channel count a power of two");
  constexpr int DO = DIN / 2, DO3 = DO * DO * DO, DIN3 = DIN * DIN * DIN;
  constexpr int K = CIN * 27, KP = (K + 15) / 16 * 16;  // padded K (the weights' row length)
  constexpr int NCH = (KP + kTcKC - 1) / kTcKC;         // K chunks
  constexpr int A_SLICE = kTcM * 16 * 2, B_SLICE = COUT * 16 * 2;
  constexpr int A_STAGE = A_SLICE * (kTcKC / 16), B_STAGE = B_SLICE * (kTcKC / 16);
  constexpr uint32_t TCOLS = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : (COUT <= 128 ? 128 : 256));
  constexpr uint32_t IDESC = tc_idesc(kTcM, COUT);
  static_assert(COUT % 16 == 0 && COUT >= 16 && COUT <= 256, "MMA N");
  extern __shared__ __align__(128) unsigned char tsm[];  // [2][A_STAGE] then [2][B_STAGE]
  __shared__ __align__(8) unsigned long long bar[2];
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t a0 = tc_smem(tsm), b0 = a0 + 2 * A_STAGE;
  const uint32_t bars[2] = {tc_smem(&bar[0]), tc_smem(&bar[1])};
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars[0]) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars[1]) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_base)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;
  uint32_t uses[2] = {0u, 0u};  // issued uses of each stage
  bool ok = true;                // block-uniform: every wait's outcome is agreed at a barrier
  const long long n_tiles = (m_total + kTcM - 1) / kTcM;
  for (long long tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    // this thread's output voxel (row tid of the tile); rows past the batch
    // gather zeros and store nothing
    const long long m = tile * kTcM + tid;
    const bool row = m < m_total;
    const int b = row ? (int)(m / DO3) : 0, vox = row ? (int)(m % DO3) : 0;
    const int ox = vox % DO, oy = (vox / DO) % DO, oz = vox / (DO * DO);
    const float *ib = in + (size_t)b * CIN * DIN3;
    for (int c = 0; c < NCH; c++) {
      const int st = c & 1;
      // the MMAs that last read this stage must have finished
      const bool lost = uses[st] > 0 && !tc_wait(bars[st], (uses[st] - 1) & 1);
      // A: this thread's row, K values 64c .. 64c + 63, as 8 groups of 8
      const uint32_t arow = a0 + st * A_STAGE + (tid >> 3) * 256 + (tid & 7) * 16;
      // every load of the chunk is issued before the first shared-memory
      // store (one round trip per chunk, not one per group)
      if constexpr (IN_B) {
        const __nv_bfloat16 *rb = in_b + (size_t)b * DIN3 * CIN;
        uint4 v[kTcKC / 8];
#pragma unroll
        for (int g = 0; g < kTcKC / 8; g++) {
          const int k0 = c * kTcKC + g * 8;
          const int tap = k0 / CIN, ci0 = k0 % CIN;
          v[g] = make_uint4(0u, 0u, 0u, 0u);
          if (row && tap < 27) {
            const int iz = 2 * oz - 1 + tap / 9, iy = 2 * oy - 1 + (tap / 3) % 3, ix = 2 * ox - 1 + tap % 3;
            if ((unsigned)iz < (unsigned)DIN && (unsigned)iy < (unsigned)DIN && (unsigned)ix < (unsigned)DIN)
              v[g] = __ldg(reinterpret_cast<const uint4 *>(rb + ((size_t)(iz * DIN + iy) * DIN + ix) * CIN + ci0));
          }
        }
#pragma unroll
        for (int g = 0; g < kTcKC / 8; g++) {
          const uint32_t dst = arow + (g >> 1) * A_SLICE + (g & 1) * 128;
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst), "r"(v[g].x), "r"(v[g].y),
                       "r"(v[g].z), "r"(v[g].w));
        }
      } else {
      float f[kTcKC];
#pragma unroll
      for (int j = 0; j < kTcKC; j++) {
        const int k = c * kTcKC + j;
        f[j] = 0.f;
        if (row && k < K) {
          const int ci = k / 27, tap = k % 27;
          const int iz = 2 * oz - 1 + tap / 9, iy = 2 * oy - 1 + (tap / 3) % 3, ix = 2 * ox - 1 + tap % 3;
          if ((unsigned)iz < (unsigned)DIN && (unsigned)iy < (unsigned)DIN && (unsigned)ix < (unsigned)DIN)
            f[j] = __ldg(ib + (size_t)ci * DIN3 + ((size_t)iz * DIN + iy) * DIN + ix);
        }
      }
#pragma unroll
      for (int g = 0; g < kTcKC / 8; g++) {
        uint32_t packed[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
          const __nv_bfloat162 p2 = __floats2bfloat162_rn(f[g * 8 + 2 * h], f[g * 8 + 2 * h + 1]);
          packed[h] = *reinterpret_cast<const uint32_t *>(&p2);
        }
        const uint32_t dst = arow + (g >> 1) * A_SLICE + (g & 1) * 128;
        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst), "r"(packed[0]), "r"(packed[1]),
                     "r"(packed[2]), "r"(packed[3]));
      }
      }
      // B: weights [COUT][KP] (BF16), K values 64c .. 64c + 63, 16-byte pieces
      {
        constexpr int NQ = (COUT * (kTcKC / 8) + kTcThreads - 1) / kTcThreads;
        uint4 w[NQ];
#pragma unroll
        for (int i = 0; i < NQ; i++) {
          const int q = tid + i * kTcThreads;
          const int n = q / (kTcKC / 8), g = q % (kTcKC / 8);
          const int k0 = c * kTcKC + g * 8;
          w[i] = make_uint4(0u, 0u, 0u, 0u);
          if (q < COUT * (kTcKC / 8) && k0 < KP) w[i] = __ldg(reinterpret_cast<const uint4 *>(wb + (size_t)n * KP + k0));
        }
#pragma unroll
        for (int i = 0; i < NQ; i++) {
          const int q = tid + i * kTcThreads;
          if (q >= COUT * (kTcKC / 8)) break;
          const int n = q / (kTcKC / 8), g = q % (kTcKC / 8);
          const uint32_t dst = b0 + st * B_STAGE + (g >> 1) * B_SLICE + (n >> 3) * 256 + (g & 1) * 128 + (n & 7) * 16;
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst), "r"(w[i].x), "r"(w[i].y),
                       "r"(w[i].z), "r"(w[i].w));
        }
      }
      // generic-proxy writes visible to the tensor cores, then one thread issues
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (__syncthreads_or(lost)) {
        ok = false;
        break;
      }
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int nk = min(kTcKC, KP - c * kTcKC) / 16;
        for (int j = 0; j < nk; j++) {
          const uint64_t ad = tc_desc(a0 + st * A_STAGE + j * A_SLICE, 128, 256);
          const uint64_t bd = tc_desc(b0 + st * B_STAGE + j * B_SLICE, 128, 256);
          const uint32_t acc = (c > 0 || j > 0) ? 1u : 0u;
          asm volatile(
              "{ .reg .pred p; setp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
              : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bars[st])
                     : "memory");
      }
      uses[st] += 1;
    }
    if (!ok) break;
    // the last chunk's commit tracks every MMA of the tile (the other stage's
    // last commit, issued earlier, has completed too; its phase is waited on
    // again, at once, before that stage's next use)
    {
      const int st = (NCH - 1) & 1;
      if (__syncthreads_or(!tc_wait(bars[st], (uses[st] - 1) & 1))) {
        ok = false;
        break;
      }
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // epilogue: lane = tid (warp w holds lanes 32w..32w+31), 16 columns at a time
    float *ob = out + (size_t)b * COUT * DO3 + vox;
#pragma unroll
    for (int c0 = 0; c0 < COUT; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
          "%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = fmaxf(__uint_as_float(r[j]) + __ldg(bias + c0 + j), 0.f);
        if (out) {
#pragma unroll
          for (int j = 0; j < 16; j++) ob[(size_t)(c0 + j) * DO3] = v[j];
        }
        if (out_b) {
          uint32_t pk[8];
#pragma unroll
          for (int j = 0; j < 8; j++) {
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
            pk[j] = *reinterpret_cast<const uint32_t *>(&h2);
          }
          uint4 *dst = reinterpret_cast<uint4 *>(out_b + ((size_t)b * DO3 + vox) * COUT + c0);
          dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
          dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
      }
    }
    // the accumulator is read before the next tile's first MMA overwrites it
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  // every issued MMA has completed before the accumulator is released
  for (int st = 0; st < 2; st++)
    if (ok && uses[st] > 0) tc_wait(bars[st], (uses[st] - 1) & 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS) : "memory");
  }
}

// FP32 weights [Cout][Cin][27] -> BF16 rows padded with zeros to kp, in the
// convolution's k order: ci * 27 + tap, or tap * cin + ci (tap_major)
__global__ void conv_weights_bf16(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, int cout, int cin,
                                  int kp, int tap_major) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cout * kp) return;
  const int n = t / kp, j = t % kp, k = cin * 27;
  float v = 0.f;
  if (j < k) {
    const int ci = tap_major ? j % cin : j / 27, tap = tap_major ? j / cin : j % 27;
    v = w[((size_t)n * cin + ci) * 27 + tap];
  }
  wb[t] = __float2bfloat16_rn(v);
}

// conv forward, blocked further: each thread computes CT output channels of
// VX consecutive output voxels along x. Per input channel and (kz, ky) the
// 2 VX + 1 input values of the row segment are read once and feed 3 VX CT
// FMAs (weights from shared memory as [ci][tap][CT], float4 broadcasts).
// Taps outside the volume read 0 (fma(w, 0, acc) == acc: the same result as
// skipping them), and every output accumulates over ci, kz, ky, kx in the
// order of conv_fwd8, so the results are bit-identical to it.
template <int CT, int VX>
__global__ void __launch_bounds__(128) conv_fwd_t(const float *__restrict__ in, const float *__restrict__ w,
                                                  const float *__restrict__ bias, float *__restrict__ out,
                                                  int B, int Cin, int Cout, int Din) {
  extern __shared__ float4 swt[];  // [Cin * 27][CT / 4]
  const int Do = Din / 2, n3 = Do * Do * Do, din3 = Din * Din * Din, nxg = Do / VX;
  const int co0 = blockIdx.y * CT;
  float *sw = reinterpret_cast<float *>(swt);
  for (int e = threadIdx.x; e < Cin * 27 * CT; e += blockDim.x) {
    const int c = e % CT, ck = e / CT;  // ck = ci * 27 + k
    sw[e] = w[((size_t)(co0 + c) * Cin) * 27 + ck];
  }
  __syncthreads();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * Do * Do * nxg) return;
  const int xg = (int)(t % nxg);
  const long long r = t / nxg;
  const int oy = (int)(r % Do), oz = (int)((r / Do) % Do), b = (int)(r / ((long long)Do * Do));
  const int ox0 = xg * VX, x0 = 2 * ox0 - 1;
  float acc[VX][CT];
#pragma unroll
  for (int c = 0; c < CT; c++) {
    const float bv = bias[co0 + c];
#pragma unroll
    for (int vx = 0; vx < VX; vx++) acc[vx][c] = bv;
  }
  for (int ci = 0; ci < Cin; ci++) {
    const float *ib = in + ((size_t)b * Cin + ci) * din3;
#pragma unroll
    for (int kz = 0; kz < 3; kz++) {
      const int iz = 2 * oz - 1 + kz;
#pragma unroll
      for (int ky = 0; ky < 3; ky++) {
        const int iy = 2 * oy - 1 + ky;
        const bool rok = iz >= 0 && iz < Din && iy >= 0 && iy < Din;
        const float *row = ib + ((size_t)(rok ? iz : 0) * Din + (rok ? iy : 0)) * Din;
        float v[2 * VX + 1];
#pragma unroll
        for (int j = 0; j < 2 * VX + 1; j++) {
          const int ix = x0 + j;
          v[j] = (rok && ix >= 0 && ix < Din) ? __ldg(row + ix) : 0.f;
        }
        const float4 *wk = swt + (size_t)(ci * 27 + kz * 9 + ky * 3) * (CT / 4);
#pragma unroll
        for (int kx = 0; kx < 3; kx++)
#pragma unroll
          for (int c4 = 0; c4 < CT / 4; c4++) {
            const float4 wv = wk[kx * (CT / 4) + c4];
#pragma unroll
            for (int vx = 0; vx < VX; vx++) {
              const float iv = v[2 * vx + kx];
              acc[vx][4 * c4 + 0] = fmaf(wv.x, iv, acc[vx][4 * c4 + 0]);
              acc[vx][4 * c4 + 1] = fmaf(wv.y, iv, acc[vx][4 * c4 + 1]);
              acc[vx][4 * c4 + 2] = fmaf(wv.z, iv, acc[vx][4 * c4 + 2]);
              acc[vx][4 * c4 + 3] = fmaf(wv.w, iv, acc[vx][4 * c4 + 3]);
            }
          }
      }
    }
  }
  const int o0 = (oz * Do + oy) * Do + ox0;
#pragma unroll
  for (int c = 0; c < CT; c++)
#pragma unroll
    for (int vx = 0; vx < VX; vx++) out[((size_t)b * Cout + co0 + c) * n3 + o0 + vx] = fmaxf(acc[vx][c], 0.f);
}

// gradient w.r.t. the conv input activation, times the input's ReLU mask:
// one thread per input (b, ci, z, y, x)
__global__ void conv_bwd_data(const float *__restrict__ dz, const float *__restrict__ w,
                              const float *__restrict__ act_in, float *__restrict__ dz_in, int B,
                              int Cin, int Cout, int Din) {
  const int Do = Din / 2, n3 = Din * Din * Din, o3 = Do * Do * Do;
  const long long total = (long long)B * Cin * n3;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n3);
    const int ci = (int)((t / n3) % Cin);
    const int b = (int)(t / ((long long)n3 * Cin));
    if (act_in[t] <= 0.f) {
      dz_in[t] = 0.f;
      continue;
    }
    const int ix = i % Din, iy = (i / Din) % Din, iz = i / (Din * Din);
    float acc = 0.f;
    for (int kz = 0; kz < 3; kz++) {
      const int zz = iz + 1 - kz;
      if (zz < 0 || (zz & 1)) continue;
      const int oz = zz >> 1;
      if (oz >= Do) continue;
      for (int ky = 0; ky < 3; ky++) {
        const int yy = iy + 1 - ky;
        if (yy < 0 || (yy & 1)) continue;
        const int oy = yy >> 1;
        if (oy >= Do) continue;
        for (int kx = 0; kx < 3; kx++) {
          const int xx = ix + 1 - kx;
          if (xx < 0 || (xx & 1)) continue;
          const int ox = xx >> 1;
          if (ox >= Do) continue;
          const int k = (kz * 3 + ky) * 3 + kx;
          const size_t od = ((size_t)oz * Do + oy) * Do + ox;
          for (int co = 0; co < Cout; co++)
            acc = fmaf(w[((size_t)co * Cin + ci) * 27 + k], dz[((size_t)b * Cout + co) * o3 + od], acc);
        }
      }
    }
    dz_in[t] = acc;
  }
}

// block sum of one value per thread (blockDim 256), result in thread 0
__device__ __forceinline__ float block_sum(float v) {
  __shared__ float ws[8];
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.f;
  if (threadIdx.x == 0)
    for (int k = 0; k < 8; k++) s += ws[k];
  __syncthreads();
  return s;
}

// weight gradient: one block per weight (co, ci, k), the batch and output
// positions strided over the threads; blocks beyond the weights do the biases
__global__ void __launch_bounds__(256) conv_bwd_weight(const float *__restrict__ act_in,
                                                       const float *__restrict__ dz,
                                                       float *__restrict__ dw, float *__restrict__ db,
                                                       int B, int Cin, int Cout, int Din) {
  const int Do = Din / 2, o3 = Do * Do * Do, n3 = Din * Din * Din;
  const int nw = Cout * Cin * 27;
  const int id = blockIdx.x;
  const long long terms = (long long)B * o3;
  float acc = 0.f;
  if (id < nw) {
    const int k = id % 27, ci = (id / 27) % Cin, co = id / (27 * Cin);
    const int kx = k % 3, ky = (k / 3) % 3, kz = k / 9;
    for (long long q = threadIdx.x; q < terms; q += blockDim.x) {
      const int o = (int)(q % o3), b = (int)(q / o3);
      const int ox = o % Do, oy = (o / Do) % Do, oz = o / (Do * Do);
      const int ix = 2 * ox - 1 + kx, iy = 2 * oy - 1 + ky, iz = 2 * oz - 1 + kz;
      if (ix < 0 || iy < 0 || iz < 0 || ix >= Din || iy >= Din || iz >= Din) continue;
      acc = fmaf(dz[((size_t)b * Cout + co) * o3 + o],
                 act_in[((size_t)b * Cin + ci) * n3 + ((size_t)iz * Din + iy) * Din + ix], acc);
    }
    const float s = block_sum(acc);
    if (threadIdx.x == 0) dw[id] = s;
  } else {
    const int co = id - nw;
    for (long long q = threadIdx.x; q < terms; q += blockDim.x) {
      const int o = (int)(q % o3), b = (int)(q / o3);
      acc += dz[((size_t)b * Cout + co) * o3 + o];
    }
    const float s = block_sum(acc);
    if (threadIdx.x == 0) db[co] = s;
  }
}

// dense forward y[b][j] = sum_i W[j][i] x[b][i] + bias[j] (optionally ReLU)
__global__ void fc_fwd(const float *__restrict__ x, const float *__restrict__ w,
                       const float *__restrict__ bias, float *__restrict__ y, int B, int Nin, int Nout,
                       int relu) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * Nout) return;
  const int j = t % Nout, b = t / Nout;
  float acc = bias[j];
  for (int i = 0; i < Nin; i++) acc = fmaf(w[(size_t)j * Nin + i], x[(size_t)b * Nin + i], acc);
  y[t] = relu ? fmaxf(acc, 0.f) : acc;
}

// dense forward with 128 outputs, tiled: a block takes 8 samples and 32 of
// the 128 outputs (blockIdx.y), 512 blocks per 1024 samples; input and
// weight slices of 32 pass through shared memory (coalesced reads; the weight
// tile padded to 33 columns against bank conflicts); thread (tb, tj)
// accumulates output 32 blockIdx.y + tj of sample tb over the inputs in
// ascending order from the bias, as fc_fwd does, so the results are
// bit-identical to it.
constexpr int kFcTB = 8, kFcIC = 32;
__global__ void __launch_bounds__(256) fc_fwd128(const float *__restrict__ x, const float *__restrict__ w,
                                                 const float *__restrict__ bias, float *__restrict__ y, int B,
                                                 int Nin, int relu) {
  __shared__ float sx[kFcTB][kFcIC];
  __shared__ float sw[32][kFcIC + 1];
  const int tid = threadIdx.x, tb = tid / 32, tj = tid % 32;
  const int b0 = blockIdx.x * kFcTB, j0 = blockIdx.y * 32;
  float acc = bias[j0 + tj];
  for (int i0 = 0; i0 < Nin; i0 += kFcIC) {
    {
      const int bb = tid / kFcIC, ii = tid % kFcIC;
      sx[bb][ii] = (b0 + bb < B) ? x[(size_t)(b0 + bb) * Nin + i0 + ii] : 0.f;
    }
    for (int e = tid; e < 32 * kFcIC; e += 256) {
      const int jj = e / kFcIC, ii = e % kFcIC;
      sw[jj][ii] = w[(size_t)(j0 + jj) * Nin + i0 + ii];
    }
    __syncthreads();
#pragma unroll 8
    for (int ii = 0; ii < kFcIC; ii++) acc = fmaf(sw[tj][ii], sx[tb][ii], acc);
    __syncthreads();
  }
  if (b0 + tb < B) y[(size_t)(b0 + tb) * 128 + j0 + tj] = relu ? fmaxf(acc, 0.f) : acc;
}

// dense input gradient times the input's ReLU mask
__global__ void fc_bwd_data(const float *__restrict__ dz, const float *__restrict__ w,
                            const float *__restrict__ act_in, float *__restrict__ dz_in, int B,
                            int Nin, int Nout) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * Nin) return;
  const int i = t % Nin, b = t / Nin;
  if (act_in[t] <= 0.f) {
    dz_in[t] = 0.f;
    return;
  }
  float acc = 0.f;
  for (int j = 0; j < Nout; j++) acc = fmaf(w[(size_t)j * Nin + i], dz[(size_t)b * Nout + j], acc);
  dz_in[t] = acc;
}

// dense weight and bias gradients: one thread per weight (j, i), then biases
__global__ void fc_bwd_weight(const float *__restrict__ x, const float *__restrict__ dz,
                              float *__restrict__ dw, float *__restrict__ db, int B, int Nin, int Nout) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < Nout * Nin) {
    const int i = t % Nin, j = t / Nin;
    float acc = 0.f;
    for (int b = 0; b < B; b++) acc = fmaf(dz[(size_t)b * Nout + j], x[(size_t)b * Nin + i], acc);
    dw[t] = acc;
  } else if (t < Nout * Nin + Nout) {
    const int j = t - Nout * Nin;
    float acc = 0.f;
    for (int b = 0; b < B; b++) acc += dz[(size_t)b * Nout + j];
    db[j] = acc;
  }
}

struct Scales {
  float s[12];
};

// mean squared error of the scaled outputs, its gradient, per-sample sums
__global__ void mse_grad(const float *__restrict__ y, const float *__restrict__ target, Scales sc,
                         float *__restrict__ dy, float *__restrict__ sq, int B) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * kF2) return;
  const float e = y[t] - target[t] / sc.s[t % kF2];
  dy[t] = 2.f * e / (float)(B * kF2);
  sq[t] = e * e;
}

__global__ void __launch_bounds__(256) sum_kernel(const float *__restrict__ v, int n, float *out) {
  float acc = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += v[i];
  const float s = block_sum(acc);
  if (threadIdx.x == 0) *out = s;
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// patches: one block per point; voxel of the patch at (x, y, z) is
// volume[round(p) - 16 + (x, y, z)] (0 outside); each patch normalised to zero
// mean and unit variance
template <typename VT>
__global__ void __launch_bounds__(256) patch_kernel(const VT *__restrict__ ref, const VT *__restrict__ cor,
                                                    int nx, int ny, int nz, const double *__restrict__ pts,
                                                    const int *__restrict__ idx, float *__restrict__ out) {
  const int n = idx ? idx[blockIdx.x] : blockIdx.x;
  int o[3];
  for (int d = 0; d < 3; d++) o[d] = (int)floor(pts[(size_t)n * 3 + d] + 0.5) - kP / 2;
  constexpr int N3 = kP * kP * kP;
  for (int v = 0; v < 2; v++) {
    const VT *vol = v == 0 ? ref : cor;
    float *dst = out + ((size_t)blockIdx.x * 2 + v) * N3;
    float s = 0.f;
    for (int i = threadIdx.x; i < N3; i += blockDim.x) {
      const int x = o[0] + i % kP, y = o[1] + (i / kP) % kP, z = o[2] + i / (kP * kP);
      float val = 0.f;
      if (x >= 0 && y >= 0 && z >= 0 && x < nx && y < ny && z < nz)
        val = (float)vol[((size_t)z * ny + y) * nx + x];
      dst[i] = val;
      s += val;
    }
    __shared__ float mean_s, inv_s;
    const float tot = block_sum(s);
    if (threadIdx.x == 0) mean_s = tot / N3;
    __syncthreads();
    const float mean = mean_s;
    float q = 0.f;
    for (int i = threadIdx.x; i < N3; i += blockDim.x) {
      const float dv = dst[i] - mean;
      q += dv * dv;
    }
    const float var = block_sum(q);
    if (threadIdx.x == 0) inv_s = 1.f / sqrtf(var / N3 + 1e-6f);
    __syncthreads();
    const float inv = inv_s;
    for (int i = threadIdx.x; i < N3; i += blockDim.x) dst[i] = (dst[i] - mean) * inv;
    __syncthreads();
  }
}

// network outputs -> start parameters (FP64, [n][12])
__global__ void denorm_kernel(const float *__restrict__ y, Scales sc, const int *__restrict__ idx,
                              double *__restrict__ params, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * kF2) return;
  const int k = t % kF2, r = t / kF2;
  const int p = idx ? idx[r] : r;
  params[(size_t)p * kF2 + k] = (double)(y[t] * sc.s[k]);
}

unsigned grid_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152LL * 64); }

}  // namespace

// ============================================================ network ===
struct dvc_cnn {
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  long long step = 0;
  int cap = 0;                         // batch capacity of the activation buffers
  float *act[kNL + 3] = {nullptr};     // input, conv1..4 outputs, dense1 output, dense2 output
  float *dact[kNL + 3] = {nullptr};    // gradients of the same (pre-ReLU where masked)
  float *sq = nullptr, *loss = nullptr;
  __nv_bfloat16 *wb[kNL] = {nullptr};  // conv weights in BF16 for the tensor-core convolutions
  __nv_bfloat16 *actb[kNL - 1] = {nullptr};  // conv 1..3 outputs, BF16 channels-last
  bool wb_valid = false;               // wb holds the current weights
  int num_sms = 0;
};

namespace {

size_t act_size(int l) {  // floats per sample of act[l]
  if (l == 0) return (size_t)2 * kP * kP * kP;
  if (l <= kNL) {
    const int d = kDin[l - 1] / 2;
    return (size_t)kCout[l - 1] * d * d * d;
  }
  return l == kNL + 1 ? (size_t)kF1 : (size_t)kF2;
}

int ensure_batch(dvc_cnn *c, int B) {
  if (B <= c->cap) return DVC_OK;
  for (int l = 0; l < kNL + 3; l++) {
    cudaFree(c->act[l]);
    cudaFree(c->dact[l]);
    c->act[l] = c->dact[l] = nullptr;
  }
  cudaFree(c->sq);
  for (int l = 0; l < kNL - 1; l++) {
    cudaFree(c->actb[l]);
    c->actb[l] = nullptr;
  }
  c->cap = 0;
  for (int l = 0; l < kNL + 3; l++) {
    if (cudaMalloc(&c->act[l], act_size(l) * B * 4) != cudaSuccess ||
        cudaMalloc(&c->dact[l], act_size(l) * B * 4) != cudaSuccess)
      return dvc_internal_set_error(DVC_E_NOMEM, "network activations");
  }
  if (cudaMalloc(&c->sq, (size_t)B * kF2 * 4) != cudaSuccess)
    return dvc_internal_set_error(DVC_E_NOMEM, "network loss buffer");
  for (int l = 0; l < kNL - 1; l++)
    if (cudaMalloc(&c->actb[l], act_size(l + 1) * B * sizeof(__nv_bfloat16)) != cudaSuccess)
      return dvc_internal_set_error(DVC_E_NOMEM, "network activations");
  c->cap = B;
  return DVC_OK;
}

Scales scales() {
  Scales s;
  for (int k = 0; k < 12; k++) s.s[k] = kScale[k];
  return s;
}

constexpr int kp_of(int l) { return (kCinC[l] * 27 + 15) / 16 * 16; }

template <int CIN, int COUT, int DIN>
constexpr size_t tc_smem_bytes() {
  return 2 * (size_t)kTcM * kTcKC * 2 + 2 * (size_t)COUT * kTcKC * 2;
}

template <int CIN, int COUT, int DIN>
int tc_attr() {
  return cudaFuncSetAttribute(conv_fwd_tc<CIN, COUT, DIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tc_smem_bytes<CIN, COUT, DIN>()) == cudaSuccess ? 0 : 1;
}

// layer l: input act[l] (FP32, the first layer) or actb[l - 1] (BF16
// channels-last); output actb[l] for the next convolution and, when fp32_out,
// act[l + 1] (the last layer always: the dense layer's input)
template <int CIN, int COUT, int DIN>
void tc_launch(dvc_cnn *c, int B, int l, bool fp32_out, cudaStream_t st) {
  const long long m_total = (long long)B * (DIN / 2) * (DIN / 2) * (DIN / 2);
  const long long tiles = (m_total + kTcM - 1) / kTcM;
  const unsigned grid = (unsigned)std::min<long long>(tiles, (long long)c->num_sms * 4);
  const bool last = l == kNL - 1;
  conv_fwd_tc<CIN, COUT, DIN><<<grid, kTcThreads, tc_smem_bytes<CIN, COUT, DIN>(), st>>>(
      c->act[l], l > 0 ? c->actb[l - 1] : nullptr, c->wb[l], c->p + kLay.b[l],
      (fp32_out || last) ? c->act[l + 1] : nullptr, last ? nullptr : c->actb[l], m_total);
}

// the BF16 copies of the conv weights, when the FP32 weights changed
void refresh_bf16(dvc_cnn *c, cudaStream_t st) {
  if (c->wb_valid) return;
  for (int l = 0; l < kNL; l++) {
    const int kp = kp_of(l), n = kCout[l] * kp;
    conv_weights_bf16<<<(n + 255) / 256, 256, 0, st>>>(c->p + kLay.w[l], c->wb[l], kCout[l], kCin[l], kp,
                                                        kCin[l] % 8 == 0 ? 1 : 0);
  }
  c->wb_valid = true;
}

// tensor-core errors recorded by the kernels (a bounded wait that gave up)
int tc_status() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, tc_error, sizeof v) != cudaSuccess)
    return dvc_internal_set_error(DVC_E_CUDA, "reading the convolution error flag");
  if (v) {
    const int z = 0;
    cudaMemcpyToSymbol(tc_error, &z, sizeof z);
    return dvc_internal_set_error(DVC_E_TIMEOUT, "a tensor-core convolution's wait gave up");
  }
  return DVC_OK;
}

template <int CT, int VX>
void conv_launch(dvc_cnn *c, int B, int l, cudaStream_t st) {
  const int Do = kDin[l] / 2;
  const size_t smem = (size_t)kCin[l] * 27 * CT * 4;
  const long long nthr = (long long)B * Do * Do * (Do / VX);
  const dim3 grid((unsigned)((nthr + 127) / 128), (unsigned)(kCout[l] / CT));
  conv_fwd_t<CT, VX><<<grid, 128, smem, st>>>(c->act[l], c->p + kLay.w[l], c->p + kLay.b[l], c->act[l + 1], B,
                                              kCin[l], kCout[l], kDin[l]);
}

// forward from act[0] (already holding the patches) to act[kNL + 2];
// keep: every layer's FP32 activation in act[] (the backward pass needs them)
void forward(dvc_cnn *c, int B, cudaStream_t st, bool keep = true) {
  // the convolutions on the tensor cores (BF16 operands, FP32 accumulation);
  // DVC_CNN_FP32: the FP32 CUDA-core kernels below, DVC_CNN_CONV8 the
  // one-output-per-thread ones (the measured alternatives)
  const bool one_voxel = getenv("DVC_CNN_CONV8") != nullptr;
  const bool fp32 = one_voxel || getenv("DVC_CNN_FP32") != nullptr;
  if (!fp32) {
    refresh_bf16(c, st);
    tc_launch<2, 16, 32>(c, B, 0, keep, st);
    tc_launch<16, 32, 16>(c, B, 1, keep, st);
    tc_launch<32, 64, 8>(c, B, 2, keep, st);
    tc_launch<64, 96, 4>(c, B, 3, keep, st);
  } else if (one_voxel) {
    for (int l = 0; l < kNL; l++) {
      const int Do = kDin[l] / 2;
      const size_t smem = (size_t)kCin[l] * 27 * kCoG * 4;
      const dim3 grid((unsigned)(((long long)B * Do * Do * Do + 255) / 256), (unsigned)(kCout[l] / kCoG));
      conv_fwd8<<<grid, 256, smem, st>>>(c->act[l], c->p + kLay.w[l], c->p + kLay.b[l], c->act[l + 1], B,
                                         kCin[l], kCout[l], kDin[l]);
    }
  } else {
    // output voxels per layer 16^3, 8^3, 4^3, 2^3; channel groups of 16 (8
    // for the last: its weights, 64 x 27 x 16 floats, would not fit), two
    // voxels per thread (measured: four voxels, 252 registers, ran the first
    // two layers 15-25% slower; narrower groups on the last two slower too)
    conv_launch<16, 2>(c, B, 0, st);
    conv_launch<16, 2>(c, B, 1, st);
    conv_launch<16, 2>(c, B, 2, st);
    conv_launch<8, 2>(c, B, 3, st);
  }
  static_assert(kF1 == 128 && kF0 % kFcIC == 0, "fc_fwd128 shape");
  if (one_voxel)
    fc_fwd<<<(B * kF1 + 255) / 256, 256, 0, st>>>(c->act[kNL], c->p + kLay.w[kNL], c->p + kLay.b[kNL],
                                                  c->act[kNL + 1], B, kF0, kF1, 1);
  else
    fc_fwd128<<<dim3((B + kFcTB - 1) / kFcTB, kF1 / 32), 256, 0, st>>>(c->act[kNL], c->p + kLay.w[kNL],
                                                                       c->p + kLay.b[kNL], c->act[kNL + 1], B,
                                                                       kF0, 1);
  fc_fwd<<<(B * kF2 + 255) / 256, 256, 0, st>>>(c->act[kNL + 1], c->p + kLay.w[kNL + 1],
                                                c->p + kLay.b[kNL + 1], c->act[kNL + 2], B, kF1, kF2, 0);
}

// loss and gradients into c->g (targets raw parameters [B][12] FP32)
void backward(dvc_cnn *c, int B, const float *targets, cudaStream_t st) {
  mse_grad<<<(B * kF2 + 255) / 256, 256, 0, st>>>(c->act[kNL + 2], targets, scales(), c->dact[kNL + 2],
                                                  c->sq, B);
  sum_kernel<<<1, 256, 0, st>>>(c->sq, B * kF2, c->loss);
  // dense 2
  fc_bwd_weight<<<(kF2 * kF1 + kF2 + 255) / 256, 256, 0, st>>>(c->act[kNL + 1], c->dact[kNL + 2],
                                                               c->g + kLay.w[kNL + 1], c->g + kLay.b[kNL + 1],
                                                               B, kF1, kF2);
  fc_bwd_data<<<(B * kF1 + 255) / 256, 256, 0, st>>>(c->dact[kNL + 2], c->p + kLay.w[kNL + 1],
                                                     c->act[kNL + 1], c->dact[kNL + 1], B, kF1, kF2);
  // dense 1
  fc_bwd_weight<<<(kF1 * kF0 + kF1 + 255) / 256, 256, 0, st>>>(c->act[kNL], c->dact[kNL + 1],
                                                               c->g + kLay.w[kNL], c->g + kLay.b[kNL], B,
                                                               kF0, kF1);
  fc_bwd_data<<<(B * kF0 + 255) / 256, 256, 0, st>>>(c->dact[kNL + 1], c->p + kLay.w[kNL], c->act[kNL],
                                                     c->dact[kNL], B, kF0, kF1);
  // conv layers, last to first (dact[l + 1] holds the gradient before ReLU)
  for (int l = kNL - 1; l >= 0; l--) {
    conv_bwd_weight<<<kCout[l] * kCin[l] * 27 + kCout[l], 256, 0, st>>>(
        c->act[l], c->dact[l + 1], c->g + kLay.w[l], c->g + kLay.b[l], B, kCin[l], kCout[l], kDin[l]);
    if (l > 0)
      conv_bwd_data<<<grid_for((long long)B * act_size(l)), 256, 0, st>>>(
          c->dact[l + 1], c->p + kLay.w[l], c->act[l], c->dact[l], B, kCin[l], kCout[l], kDin[l]);
  }
}

}  // namespace

extern "C" {

int dvc_cnn_param_count(void) { return (int)kLay.total; }

int dvc_cnn_create(dvc_cnn **out, unsigned seed) try {
  if (!out) return dvc_internal_set_error(DVC_E_ARG, "null argument");
  // the largest layer's weight group (64 x 27 x 8 floats) exceeds the default
  // 48 KB of dynamic shared memory
  const int big = kCin[kNL - 1] * 27 * 8 * 4;  // 55,296 bytes
  if (cudaFuncSetAttribute(conv_fwd8, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kCin[kNL - 1] * 27 * kCoG * 4) != cudaSuccess ||
      cudaFuncSetAttribute(conv_fwd_t<16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      cudaFuncSetAttribute(conv_fwd_t<8, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) != cudaSuccess ||
      tc_attr<2, 16, 32>() || tc_attr<16, 32, 16>() || tc_attr<32, 64, 8>() || tc_attr<64, 96, 4>())
    return dvc_internal_set_error(DVC_E_CUDA, "conv kernel attribute");
  dvc_cnn *c = new dvc_cnn();
  const size_t n = kLay.total;
  if (cudaMalloc(&c->p, n * 4) != cudaSuccess || cudaMalloc(&c->g, n * 4) != cudaSuccess ||
      cudaMalloc(&c->m, n * 4) != cudaSuccess || cudaMalloc(&c->v, n * 4) != cudaSuccess ||
      cudaMalloc(&c->loss, 4) != cudaSuccess) {
    dvc_cnn_destroy(c);
    return dvc_internal_set_error(DVC_E_NOMEM, "network parameters");
  }
  for (int l = 0; l < kNL; l++)
    if (cudaMalloc(&c->wb[l], (size_t)kCout[l] * kp_of(l) * sizeof(__nv_bfloat16)) != cudaSuccess) {
      dvc_cnn_destroy(c);
      return dvc_internal_set_error(DVC_E_NOMEM, "network parameters");
    }
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  // He-normal weights (fan-in), zero biases
  std::vector<float> h(n, 0.f);
  std::mt19937 gen(seed);
  auto fill = [&](size_t off, size_t cnt, int fan_in) {
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)fan_in));
    for (size_t i = 0; i < cnt; i++) h[off + i] = nd(gen);
  };
  for (int l = 0; l < kNL; l++) fill(kLay.w[l], (size_t)kCout[l] * kCin[l] * 27, kCin[l] * 27);
  fill(kLay.w[kNL], (size_t)kF1 * kF0, kF0);
  fill(kLay.w[kNL + 1], (size_t)kF2 * kF1, kF1);
  cudaMemcpy(c->p, h.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemset(c->m, 0, n * 4);
  cudaMemset(c->v, 0, n * 4);
  *out = c;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

void dvc_cnn_destroy(dvc_cnn *c) try {
  if (!c) return;
  cudaFree(c->p);
  cudaFree(c->g);
  cudaFree(c->m);
  cudaFree(c->v);
  cudaFree(c->loss);
  cudaFree(c->sq);
  for (int l = 0; l < kNL; l++) cudaFree(c->wb[l]);
  for (int l = 0; l < kNL - 1; l++) cudaFree(c->actb[l]);
  for (int l = 0; l < kNL + 3; l++) {
    cudaFree(c->act[l]);
    cudaFree(c->dact[l]);
  }
  delete c;
} catch (...) {
  dvc_internal_host_exception();
}

int dvc_cnn_get_weights(dvc_cnn *c, float *host, int n) try {
  if (!c || !host || n != (int)kLay.total) return dvc_internal_set_error(DVC_E_ARG, "bad weight buffer");
  if (cudaMemcpy(host, c->p, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return dvc_internal_set_error(DVC_E_CUDA, "weight copy");
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_cnn_set_weights(dvc_cnn *c, const float *host, int n) try {
  if (!c || !host || n != (int)kLay.total) return dvc_internal_set_error(DVC_E_ARG, "bad weight buffer");
  if (cudaMemcpy(c->p, host, (size_t)n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return dvc_internal_set_error(DVC_E_CUDA, "weight copy");
  cudaMemset(c->m, 0, (size_t)n * 4);
  cudaMemset(c->v, 0, (size_t)n * 4);
  c->step = 0;
  c->wb_valid = false;
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_cnn_forward(dvc_cnn *c, int batch, const float *patches_dev, float *out_dev, void *stream) try {
  if (!c || batch <= 0 || !patches_dev || !out_dev) return dvc_internal_set_error(DVC_E_ARG, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = ensure_batch(c, batch);
  if (rc) return rc;
  cudaMemcpyAsync(c->act[0], patches_dev, act_size(0) * batch * 4, cudaMemcpyDeviceToDevice, st);
  forward(c, batch, st, false);
  cudaMemcpyAsync(out_dev, c->act[kNL + 2], (size_t)batch * kF2 * 4, cudaMemcpyDeviceToDevice, st);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(e));
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_cnn_gradients(dvc_cnn *c, int batch, const float *patches_dev, const float *targets_dev,
                      float *grad_host, float *loss) try {
  if (!c || batch <= 0 || !patches_dev || !targets_dev) return dvc_internal_set_error(DVC_E_ARG, "bad arguments");
  int rc = ensure_batch(c, batch);
  if (rc) return rc;
  cudaMemcpy(c->act[0], patches_dev, act_size(0) * batch * 4, cudaMemcpyDeviceToDevice);
  forward(c, batch, 0);
  backward(c, batch, targets_dev, 0);
  float l = 0.f;
  if (cudaMemcpy(&l, c->loss, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return dvc_internal_set_error(DVC_E_CUDA, "loss copy");
  if (loss) *loss = l / (float)(batch * kF2);
  if (grad_host) cudaMemcpy(grad_host, c->g, kLay.total * 4, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(e));
  return tc_status();
} catch (...) {
  return dvc_internal_host_exception();
}

int dvc_cnn_train_step(dvc_cnn *c, int batch, const float *patches_dev, const float *targets_dev,
                       float lr, float *loss) try {
  int rc = dvc_cnn_gradients(c, batch, patches_dev, targets_dev, nullptr, loss);
  if (rc) return rc;
  c->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)c->step), c2 = 1.f - std::pow(b2, (float)c->step);
  adam_kernel<<<grid_for((long long)kLay.total), 256>>>(c->p, c->g, c->m, c->v, kLay.total, lr, b1, b2, 1e-8f,
                                                        c1, c2);
  c->wb_valid = false;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(e));
  return DVC_OK;
} catch (...) {
  return dvc_internal_host_exception();
}

}  // extern "C"

// the tensor-core convolutions' error flag (after the caller synchronised)
int dvc_internal_cnn_status() { return tc_status(); }

// patches of the points idx[0..n) (or 0..n) of an engine's volume pair
int dvc_internal_patches(const void *ref, const void *cor, int bpv, int nx, int ny, int nz,
                         int n, const double *pts_dev, const int *idx_dev, float *out_dev,
                         cudaStream_t st) {
  if (n <= 0) return DVC_OK;
  if (bpv == 1)
    patch_kernel<uint8_t><<<n, 256, 0, st>>>((const uint8_t *)ref, (const uint8_t *)cor, nx, ny, nz,
                                             pts_dev, idx_dev, out_dev);
  else
    patch_kernel<uint16_t><<<n, 256, 0, st>>>((const uint16_t *)ref, (const uint16_t *)cor, nx, ny, nz,
                                              pts_dev, idx_dev, out_dev);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(e));
  return DVC_OK;
}

// start parameters of points idx[0..n) from the network, written to
// params_dev[idx[r] * 12 ..] (FP64), in batches
int dvc_internal_cnn_seed(dvc_cnn *c, const void *ref, const void *cor, int bpv, int nx, int ny,
                          int nz, int n, const double *pts_dev, const int *idx_dev, double *params_dev,
                          cudaStream_t st) {
  const int B = 4096;  // patches per network pass (the last convolution: 256 tiles of 128 outputs)
  int rc = ensure_batch(c, B);
  if (rc) return rc;
  for (int r0 = 0; r0 < n; r0 += B) {
    const int nb = std::min(B, n - r0);
    // patches straight into the input activation
    const double *pb = pts_dev + (idx_dev ? 0 : (size_t)r0 * 3);
    const int *ib = idx_dev ? idx_dev + r0 : nullptr;
    if (bpv == 1)
      patch_kernel<uint8_t><<<nb, 256, 0, st>>>((const uint8_t *)ref, (const uint8_t *)cor, nx, ny, nz, pb,
                                                ib, c->act[0]);
    else
      patch_kernel<uint16_t><<<nb, 256, 0, st>>>((const uint16_t *)ref, (const uint16_t *)cor, nx, ny, nz,
                                                 pb, ib, c->act[0]);
    forward(c, nb, st, false);
    denorm_kernel<<<(nb * kF2 + 255) / 256, 256, 0, st>>>(c->act[kNL + 2], scales(),
                                                          idx_dev ? idx_dev + r0 : nullptr,
                                                          params_dev + (idx_dev ? 0 : (size_t)r0 * kF2), nb);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return dvc_internal_set_error(DVC_E_CUDA, cudaGetErrorString(e));
  return DVC_OK;
}

// The pointwise subgrid-stress network on the fifth-generation tensor cores.
//
// Every matrix product is a chain of tcgen05.mma (kind::f16: BF16 operands,
// FP32 accumulators in tensor memory) issued by one thread of the CTA, with
// both operands K-major in shared memory in the canonical no-swizzle layout
// (core matrices of 8 rows x 16 bytes, 128 contiguous bytes each; the next
// core matrix along K 128 bytes on, the next 8-row group K*16 bytes on).
// A CTA of 128 threads owns a tile of 128 points: thread p owns TMEM lane p,
// i.e. row p of every point-major accumulator, reads it with tcgen05.ld and
// writes its point's activations back as the BF16 operand of the next
// product.  Completion of each chain is signalled by tcgen05.commit on an
// mbarrier; every wait is bounded and a wait that runs out sets an error
// flag, after which the CTA drains, frees its tensor memory and returns.
//
//   k_mlp_pack  : FP32 parameters -> BF16 operand tiles W and W^T, FP32 biases
//   k_mlp_train : forward, loss and backward over a batch of 128-point tiles.
//                 Weight gradients dW^T = H^T dZ are products over the points
//                 (K = the tile's 128 points) and accumulate in tensor memory
//                 across the CTA's tiles; a row of ones under each H^T gives
//                 the bias gradients in the same products.  One atomic flush
//                 per CTA at the end.
//   k_mlp_infer : forward only, outputs in physical units
//   k_adam      : Adam step on the FP32 master parameters
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/chgpu_closure.h"
#include "async.cuh"
#include "chgpu_internal.h"
#include "mlp.cuh"

namespace chgpu {
namespace mlp {

// ---------------------------------------------------------------------------
// tensor-memory and tensor-core primitives (inline PTX, sm_100 family)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tm_alloc(unsigned* dst, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tm_dealloc(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tm_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tm_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy writes of shared memory made visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// shared-memory matrix descriptor: start address, leading (K-direction) and
// stride (M/N-direction) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(const void* p, unsigned lbo, unsigned sbo) {
  const unsigned a = smem_addr(p);
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr unsigned idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}
__device__ __forceinline__ void tm_mma(unsigned d, uint64_t a, uint64_t b, unsigned idesc, int accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tm_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}
// 16 consecutive FP32 columns of this thread's lane; the wait is inside the
// same statement so the registers are defined when it ends
__device__ __forceinline__ void tm_ld16(unsigned taddr, float (&v)[16]) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// one chain D (+)= A B^T over ksteps K-slices of 16: A [128 x 16*ksteps] and
// B [N x 16*ksteps], K-major; each slice is two core matrices along K
__device__ __forceinline__ void mma_chain(unsigned d, const unsigned char* a, unsigned a_sbo, const unsigned char* b,
                                          unsigned b_sbo, int ksteps, unsigned idesc, bool accumulate) {
  for (int s = 0; s < ksteps; ++s)
    tm_mma(d, sdesc(a + s * 256, 128, a_sbo), sdesc(b + s * 256, 128, b_sbo), idesc, (accumulate || s > 0) ? 1 : 0);
}

__device__ __forceinline__ unsigned short bf16_bits(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ unsigned pack2(float a, float b) {
  return (unsigned)bf16_bits(a) | ((unsigned)bf16_bits(b) << 16);
}
// 8 consecutive K elements of one row: one 16-byte store
__device__ __forceinline__ void store8(unsigned char* dst, const float* x) {
  *reinterpret_cast<uint4*>(dst) = make_uint4(pack2(x[0], x[1]), pack2(x[2], x[3]), pack2(x[4], x[5]), pack2(x[6], x[7]));
}
__device__ __forceinline__ void store1(unsigned char* dst, float x) {
  *reinterpret_cast<unsigned short*>(dst) = bf16_bits(x);
}

__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }

// ---------------------------------------------------------------------------
// operand packing
// ---------------------------------------------------------------------------
__global__ void k_mlp_pack(const float* __restrict__ theta, unsigned char* __restrict__ packed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  // regions in the order of the packed block: rows x K
  struct Reg { int off, rows, K; };
  const Reg regs[7] = {{P_W1, 64, 16}, {P_W2, 64, 64}, {P_W3, 64, 64}, {P_W4, 16, 64},
                       {P_W4T, 64, 16}, {P_W3T, 64, 64}, {P_W2T, 64, 64}};
  int e = i;
#pragma unroll
  for (int g = 0; g < 7; ++g) {
    const int cnt = regs[g].rows * regs[g].K;
    if (e >= 0 && e < cnt) {
      const int r = e / regs[g].K, k = e - r * regs[g].K;
      float v = 0.0f;
      switch (g) {
        case 0: v = theta[OFF_W1 + r * 16 + k]; break;       // W1[o=r][i=k]
        case 1: v = theta[OFF_W2 + r * 64 + k]; break;       // W2[o][i]
        case 2: v = theta[OFF_W3 + r * 64 + k]; break;
        case 3: v = r < NOUT ? theta[OFF_W4 + r * 64 + k] : 0.0f; break;
        case 4: v = k < NOUT ? theta[OFF_W4 + k * 64 + r] : 0.0f; break;  // W4^T: row i, K = o
        case 5: v = theta[OFF_W3 + k * 64 + r]; break;       // W3^T
        case 6: v = theta[OFF_W2 + k * 64 + r]; break;       // W2^T
      }
      store1(packed + regs[g].off + core_off(r, k, regs[g].K), v);
    }
    e -= cnt;
  }
  // biases b2, b3, b4 (padded to 16) as FP32
  if (e >= 0 && e < 144) {
    float v = 0.0f;
    if (e < 64) v = theta[OFF_B2 + e];
    else if (e < 128) v = theta[OFF_B3 + e - 64];
    else if (e - 128 < NOUT) v = theta[OFF_B4 + e - 128];
    reinterpret_cast<float*>(packed + P_BIAS)[e] = v;
  }
}
constexpr int kPackItems = 1024 + 4096 + 4096 + 1024 + 1024 + 4096 + 4096 + 144;

// ---------------------------------------------------------------------------
// shared pieces of the forward pass
// ---------------------------------------------------------------------------
// row p of the input tile: 10 normalised features, 1 (the bias column of
// W1), zeros; point-major [128 x 16] and, when xt is set, transposed
__device__ __forceinline__ void write_input_row(unsigned char* xp, unsigned char* xt, int p, const float (&f)[NIN]) {
  float x[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) x[k] = k < NIN ? f[k] : (k == NIN ? 1.0f : 0.0f);
  store8(xp + core_off(p, 0, 16), x);
  store8(xp + core_off(p, 8, 16), x + 8);
  if (xt) {
#pragma unroll
    for (int k = 0; k < 16; ++k) store1(xt + core_off(k, p, 128), x[k]);
  }
}

// hidden-layer epilogue: h = silu(acc + b) for the 64 columns of this lane,
// written point-major (next layer's A) and, when ht is set, transposed
__device__ __forceinline__ void hidden_epilogue(unsigned tz, const float* bias, unsigned char* hp, unsigned char* ht,
                                                int p) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    float v[16];
    tm_ld16(tz + 16 * j, v);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float z = v[q] + (bias ? bias[16 * j + q] : 0.0f);
      v[q] = z * sigmoid(z);
    }
    store8(hp + core_off(p, 16 * j, 64), v);
    store8(hp + core_off(p, 16 * j + 8, 64), v + 8);
    if (ht) {
#pragma unroll
      for (int q = 0; q < 16; ++q) store1(ht + core_off(16 * j + q, p, 128), v[q]);
    }
  }
}

// backward epilogue: dz = dh * silu'(z), z = acc + b; point-major (when dp
// is set) and transposed
__device__ __forceinline__ void grad_epilogue(unsigned tdh, unsigned tz, const float* bias, unsigned char* dp,
                                              unsigned char* dt, int p) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    float g[16], z[16];
    tm_ld16(tdh + 16 * j, g);
    tm_ld16(tz + 16 * j, z);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float zz = z[q] + (bias ? bias[16 * j + q] : 0.0f);
      const float s = sigmoid(zz);
      g[q] = g[q] * (s * (1.0f + zz * (1.0f - s)));
    }
    if (dp) {
      store8(dp + core_off(p, 16 * j, 64), g);
      store8(dp + core_off(p, 16 * j + 8, 64), g + 8);
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) store1(dt + core_off(16 * j + q, p, 128), g[q]);
  }
}

__device__ __forceinline__ void load_features(const float* __restrict__ feat, long long n, long long idx,
                                              const Norm& nm, float (&f)[NIN]) {
#pragma unroll
  for (int k = 0; k < NIN; ++k) f[k] = (feat[(long long)k * n + idx] - nm.mu_in[k]) * nm.isd_in[k];
}

// One chain of products and its completion: every thread's shared-memory
// writes are published to the tensor cores, one thread issues and commits,
// all wait (bounded).  Returns false, the same in every thread, when the
// wait ran out.
template <typename Issue>
__device__ __forceinline__ bool stage(unsigned long long* bar, unsigned& phase, Issue issue) {
  fence_async_smem();
  tm_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tm_fence_after();
    issue();
    tm_commit(bar);
  }
  const bool ok = mbar_wait(bar, phase, kBulkWaitPolls);
  phase ^= 1u;
  const bool all = __syncthreads_and(ok);
  tm_fence_after();
  return all;
}

// ---------------------------------------------------------------------------
// training: forward + loss + backward over tiles of 128 points
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 1) k_mlp_train(const unsigned char* __restrict__ packed,
                                                      const float* __restrict__ feat, const float* __restrict__ targ,
                                                      long long n, long long first, int tiles, Norm nm, float gscale,
                                                      float* __restrict__ grad, double* __restrict__ loss,
                                                      int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ unsigned tbase_s;
  const int p = threadIdx.x, warp = p >> 5;
  unsigned char* T = sm + S_T;
  if (p == 0) mbar_init(&bar, 1);
  if (warp == 0) tm_alloc(&tbase_s, kTrainCols);
  // rows of ones under H1^T, H2^T, H3^T (bias gradients)
  for (int w = p; w < 3 * 512; w += 128) {
    const int grp = w < 512 ? G_ONE1 : (w < 1024 ? G_ONE2 : G_ONE3);
    reinterpret_cast<unsigned*>(T + grp * 2048)[w & 511] = 0x3F803F80u;
  }
  tm_fence_before();
  __syncthreads();
  tm_fence_after();
  const unsigned tbase = tbase_s;
  const unsigned lane_off = (unsigned)(32 * warp) << 16;
  const unsigned tl = tbase + lane_off;  // this thread's lane
  unsigned phase = 0;
  if (p == 0) bulk_copy_g2s(sm, packed, PACKED_BYTES, &bar);
  bool ok = __syncthreads_and(mbar_wait(&bar, phase, kBulkWaitPolls));
  phase ^= 1u;
  const float* bias = reinterpret_cast<const float*>(sm + P_BIAS);
  const unsigned char *W1 = sm + P_W1, *W2 = sm + P_W2, *W3 = sm + P_W3, *W4 = sm + P_W4;
  const unsigned char *W4T = sm + P_W4T, *W3T = sm + P_W3T, *W2T = sm + P_W2T;
  unsigned char *X = sm + S_X, *PA = sm + S_PA, *PB = sm + S_PB, *DY = sm + S_DY;
  constexpr unsigned i64 = idesc_bf16(128, 64), i16 = idesc_bf16(128, 16);
  float lsum = 0.0f;
  int ntile = 0;
  for (int t = blockIdx.x; ok && t < tiles; t += gridDim.x, ++ntile) {
    const bool acc = ntile > 0;
    const long long idx = (first + (long long)t * 128 + p) % n;
    float f[NIN];
    load_features(feat, n, idx, nm, f);
    float tg[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; ++o) tg[o] = (targ[(long long)o * n + idx] - nm.mu_out[o]) * nm.isd_out[o];
    write_input_row(X, T + G_XT * 2048, p, f);
    // forward
    ok = stage(&bar, phase, [&] { mma_chain(tbase + C_Z1, X, 256, W1, 256, 1, i64, false); });
    if (!ok) break;
    hidden_epilogue(tl + C_Z1, nullptr, PA, T + G_H1T * 2048, p);
    ok = stage(&bar, phase, [&] { mma_chain(tbase + C_Z2, PA, 1024, W2, 1024, 4, i64, false); });
    if (!ok) break;
    hidden_epilogue(tl + C_Z2, bias, PB, T + G_H2T * 2048, p);
    ok = stage(&bar, phase, [&] { mma_chain(tbase + C_Z3, PB, 1024, W3, 1024, 4, i64, false); });
    if (!ok) break;
    hidden_epilogue(tl + C_Z3, bias + 64, PA, T + G_H3T * 2048, p);
    ok = stage(&bar, phase, [&] { mma_chain(tbase + C_Y4, PA, 1024, W4, 1024, 4, i16, false); });
    if (!ok) break;
    // loss and dL/dy
    {
      float v[16];
      tm_ld16(tl + C_Y4, v);
      float g[16];
#pragma unroll
      for (int o = 0; o < 16; ++o) {
        float d = 0.0f;
        if (o < NOUT) {
          d = v[o] + bias[128 + o] - tg[o];
          lsum += d * d;
        }
        g[o] = d * gscale;
      }
      store8(DY + core_off(p, 0, 16), g);
      store8(DY + core_off(p, 8, 16), g + 8);
#pragma unroll
      for (int o = 0; o < 16; ++o) store1(T + G_DYT * 2048 + core_off(o, p, 128), g[o]);
    }
    // backward
    ok = stage(&bar, phase, [&] {
      mma_chain(tbase + C_DW4, T + G_H3T * 2048, 2048, T + G_DYT * 2048, 2048, 8, i16, acc);
      mma_chain(tbase + C_DH, DY, 256, W4T, 256, 1, i64, false);
    });
    if (!ok) break;
    grad_epilogue(tl + C_DH, tl + C_Z3, bias + 64, PB, T + G_DZ3T * 2048, p);
    ok = stage(&bar, phase, [&] {
      mma_chain(tbase + C_DW3, T + G_H2T * 2048, 2048, T + G_DZ3T * 2048, 2048, 8, i64, acc);
      mma_chain(tbase + C_DH, PB, 1024, W3T, 1024, 4, i64, false);
    });
    if (!ok) break;
    grad_epilogue(tl + C_DH, tl + C_Z2, bias, PA, T + G_DZ2T * 2048, p);
    ok = stage(&bar, phase, [&] {
      mma_chain(tbase + C_DW2, T + G_H1T * 2048, 2048, T + G_DZ2T * 2048, 2048, 8, i64, acc);
      mma_chain(tbase + C_DH, PA, 1024, W2T, 1024, 4, i64, false);
    });
    if (!ok) break;
    grad_epilogue(tl + C_DH, tl + C_Z1, nullptr, nullptr, T + G_DZ1T * 2048, p);
    ok = stage(&bar, phase, [&] {
      mma_chain(tbase + C_DW1, T + G_XT * 2048, 2048, T + G_DZ1T * 2048, 2048, 8, i64, acc);
    });
  }
  if (!ok) {
    if (p == 0) atomicOr(err, 1);
    mbar_wait(&bar, phase ^ 1u, kBulkWaitPolls);  // the chain in flight, once more
  } else if (ntile > 0) {
    // flush: dW^T lanes are input features (lane 64: the ones row -> bias)
    if (warp < 3) {
      float v[16];
#pragma unroll 1
      for (int j = 0; j < 4; ++j) {  // W1: lanes 0..15, column o
        tm_ld16(tl + C_DW1 + 16 * j, v);
        if (p < 16)
          for (int q = 0; q < 16; ++q) atomicAdd(&grad[OFF_W1 + (16 * j + q) * 16 + p], v[q]);
      }
#pragma unroll 1
      for (int L = 0; L < 2; ++L) {  // W2/b2, W3/b3
        const unsigned col = L == 0 ? C_DW2 : C_DW3;
        const int ow = L == 0 ? OFF_W2 : OFF_W3, ob = L == 0 ? OFF_B2 : OFF_B3;
#pragma unroll 1
        for (int j = 0; j < 4; ++j) {
          tm_ld16(tl + col + 16 * j, v);
          if (p < 64)
            for (int q = 0; q < 16; ++q) atomicAdd(&grad[ow + (16 * j + q) * 64 + p], v[q]);
          else if (p == 64)
            for (int q = 0; q < 16; ++q) atomicAdd(&grad[ob + 16 * j + q], v[q]);
        }
      }
      tm_ld16(tl + C_DW4, v);
      if (p < 64)
        for (int o = 0; o < NOUT; ++o) atomicAdd(&grad[OFF_W4 + o * 64 + p], v[o]);
      else if (p == 64)
        for (int o = 0; o < NOUT; ++o) atomicAdd(&grad[OFF_B4 + o], v[o]);
    }
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((p & 31) == 0 && lsum != 0.0f) atomicAdd(loss, (double)lsum);
  tm_fence_before();
  __syncthreads();
  if (warp == 0) tm_dealloc(tbase, kTrainCols);
}

// ---------------------------------------------------------------------------
// inference
// ---------------------------------------------------------------------------
// point sources and sinks: structure-of-arrays feat[10][n] -> out[6][n] ...
struct SoaIO {
  const float* feat;
  float* out;
  long long n;
  __device__ long long count() const { return n; }
  __device__ void load(long long idx, const Norm& nm, float (&f)[NIN]) const { load_features(feat, n, idx, nm, f); }
  __device__ void store(long long idx, int o, float v) const { out[(long long)o * n + idx] = v; }
};
// ... or the closure points of a channel handle: the planes iy = 1..ny-1 of
// the physical gradient fields phys[9][plane][z][x] and the wall distance of
// each plane -> tau[6][plane][z][x] (the interior planes are contiguous)
struct PlaneIO {
  const float* phys;
  float* tau;
  const float* wd;
  long long plane_pts, comp_stride, n;
  __device__ long long count() const { return n; }
  __device__ void load(long long idx, const Norm& nm, float (&f)[NIN]) const {
    const long long off = idx + 2 * plane_pts;
#pragma unroll
    for (int k = 0; k < NIN - 1; ++k) f[k] = (phys[k * comp_stride + off] - nm.mu_in[k]) * nm.isd_in[k];
    f[NIN - 1] = (wd[off / plane_pts] - nm.mu_in[NIN - 1]) * nm.isd_in[NIN - 1];
  }
  __device__ void store(long long idx, int o, float v) const { tau[o * comp_stride + idx + 2 * plane_pts] = v; }
};

template <typename IO>
__global__ void __launch_bounds__(128) k_mlp_infer(const unsigned char* __restrict__ packed, IO io,
                                                   const Norm* __restrict__ nmp, int* __restrict__ err, int errbit) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  __shared__ unsigned tbase_s;
  const int p = threadIdx.x, warp = p >> 5;
  const Norm& nm = *nmp;  // read through the cache where used
  if (p == 0) mbar_init(&bar, 1);
  if (warp == 0) tm_alloc(&tbase_s, kInferCols);
  tm_fence_before();
  __syncthreads();
  tm_fence_after();
  const unsigned tbase = tbase_s;
  const unsigned tl = tbase + ((unsigned)(32 * warp) << 16);
  unsigned phase = 0;
  if (p == 0) {  // forward operands and biases: two bulk copies, one phase
    mbar_arrive_expect(&bar, P_W4T + (PACKED_BYTES - P_BIAS));
    bulk_copy_g2s_noarrive(sm, packed, P_W4T, &bar);
    bulk_copy_g2s_noarrive(sm + SI_BIAS, packed + P_BIAS, PACKED_BYTES - P_BIAS, &bar);
  }
  bool ok = __syncthreads_and(mbar_wait(&bar, phase, kBulkWaitPolls));
  phase ^= 1u;
  const float* bias = reinterpret_cast<const float*>(sm + SI_BIAS);
  unsigned char *X = sm + SI_X, *H = sm + SI_H;
  constexpr unsigned i64 = idesc_bf16(128, 64), i16 = idesc_bf16(128, 16);
  const long long n = io.count();
  const long long tiles = (n + 127) / 128;
  for (long long t = blockIdx.x; ok && t < tiles; t += gridDim.x) {
    const long long idx = t * 128 + p;
    float f[NIN];
    if (idx < n) io.load(idx, nm, f);
    else
      for (int k = 0; k < NIN; ++k) f[k] = 0.0f;
    write_input_row(X, nullptr, p, f);
    ok = stage(&bar, phase, [&] { mma_chain(tbase + I_Z, X, 256, sm + P_W1, 256, 1, i64, false); });
    if (!ok) break;
    hidden_epilogue(tl + I_Z, nullptr, H, nullptr, p);
    ok = stage(&bar, phase, [&] { mma_chain(tbase + I_Z, H, 1024, sm + P_W2, 1024, 4, i64, false); });
    if (!ok) break;
    hidden_epilogue(tl + I_Z, bias, H, nullptr, p);
    ok = stage(&bar, phase, [&] { mma_chain(tbase + I_Z, H, 1024, sm + P_W3, 1024, 4, i64, false); });
    if (!ok) break;
    hidden_epilogue(tl + I_Z, bias + 64, H, nullptr, p);
    ok = stage(&bar, phase, [&] { mma_chain(tbase + I_Z, H, 1024, sm + P_W4, 1024, 4, i16, false); });
    if (!ok) break;
    float v[16];
    tm_ld16(tl + I_Z, v);
    if (idx < n)
      for (int o = 0; o < NOUT; ++o) io.store(idx, o, (v[o] + bias[128 + o]) * nm.sd_out[o] + nm.mu_out[o]);
  }
  if (!ok) {
    if (p == 0) atomicOr(err, errbit);
    mbar_wait(&bar, phase ^ 1u, kBulkWaitPolls);
  }
  tm_fence_before();
  __syncthreads();
  if (warp == 0) tm_dealloc(tbase, kInferCols);
}

// ---------------------------------------------------------------------------
// Adam (FP32 master parameters); the gradient buffer is cleared for the next step
// ---------------------------------------------------------------------------
__global__ void k_adam(float* __restrict__ theta, float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.0f - b1) * gi;
  const float b = b2 * m2[i] + (1.0f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  theta[i] -= lr * (a * c1) / (sqrtf(b * c2) + eps);
  g[i] = 0.0f;
}

}  // namespace mlp

}  // namespace chgpu

struct chgpu_mlp {
  float *theta = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
  unsigned char* packed = nullptr;
  float *feat = nullptr, *targ = nullptr;
  long long n = 0, cursor = 0;
  double* loss = nullptr;  // per-step losses of the current train call
  int loss_cap = 0;
  int* err = nullptr;
  int adam_t = 0, nsm = 0;
  chgpu_mlp_norm user{};
  chgpu::mlp::Norm nm{};
  chgpu::mlp::Norm* nm_dev = nullptr;  // the same on the device (read by captured closure launches)
  cudaStream_t stream = nullptr;
  std::string msg;
};

namespace chgpu {

// ---------------------------------------------------------------------------
// launches (also used by the closure inside the coarse solver)
// ---------------------------------------------------------------------------
int mlp_set_smem_limits() {
  if (cudaFuncSetAttribute(mlp::k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::S_END) != cudaSuccess)
    return -1;
  if (cudaFuncSetAttribute(mlp::k_mlp_infer<mlp::SoaIO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           mlp::S_INFER_END) != cudaSuccess ||
      cudaFuncSetAttribute(mlp::k_mlp_infer<mlp::PlaneIO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           mlp::S_INFER_END) != cudaSuccess)
    return -1;
  return 0;
}
void launch_mlp_pack(const float* theta, unsigned char* packed, cudaStream_t s) {
  mlp::k_mlp_pack<<<(mlp::kPackItems + 255) / 256, 256, 0, s>>>(theta, packed);
}
void launch_mlp_train(const unsigned char* packed, const float* feat, const float* targ, long long n, long long first,
                      int tiles, const mlp::Norm& nm, float gscale, float* grad, double* loss, int* err, int nsm,
                      cudaStream_t s) {
  const int grid = tiles < nsm ? tiles : nsm;
  mlp::k_mlp_train<<<grid, 128, mlp::S_END, s>>>(packed, feat, targ, n, first, tiles, nm, gscale, grad, loss, err);
}
void launch_mlp_infer(const unsigned char* packed, const float* feat, long long n, const mlp::Norm* nm, float* out,
                      int* err, int nsm, cudaStream_t s) {
  const long long tiles = (n + 127) / 128;
  const int grid = (int)(tiles < 4LL * nsm ? tiles : 4LL * nsm);
  if (grid > 0) mlp::k_mlp_infer<<<grid, 128, mlp::S_INFER_END, s>>>(packed, mlp::SoaIO{feat, out, n}, nm, err, 1);
}
void launch_mlp_closure(const chgpu_mlp* m, const float* phys, float* tau, const float* wd, long long plane_pts,
                        int nplanes, int ny, int* err, int errbit, int nsm, cudaStream_t s) {
  const long long n = (long long)(ny - 1) * plane_pts;
  const long long tiles = (n + 127) / 128;
  const int grid = (int)(tiles < 4LL * nsm ? tiles : 4LL * nsm);
  mlp::PlaneIO io{phys, tau, wd, plane_pts, (long long)nplanes * plane_pts, n};
  if (grid > 0) mlp::k_mlp_infer<<<grid, 128, mlp::S_INFER_END, s>>>(m->packed, io, m->nm_dev, err, errbit);
}
void launch_adam(float* theta, float* g, float* m1, float* m2, int n, float lr, int t, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, t))), c2 = (float)(1.0 / (1.0 - std::pow(0.999, t)));
  mlp::k_adam<<<(n + 255) / 256, 256, 0, s>>>(theta, g, m1, m2, n, lr, b1, b2, 1e-8f, c1, c2);
}

}  // namespace chgpu

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace chgpu;

namespace {

std::string g_mlp_create_error;

int mfail(chgpu_mlp* m, int code, const std::string& msg) {
  if (m) m->msg = msg;
  else g_mlp_create_error = msg;
  return code;
}
int mcuda(chgpu_mlp* m, cudaError_t e, const char* where) {
  return mfail(m, CHGPU_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define MCK(m, call)                                  \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return mcuda((m), e_, #call); \
  } while (0)

// splitmix64 -> uniform in [-1, 1)
double uniform_pm1(unsigned long long& s) {
  s += 0x9E3779B97F4A7C15ull;
  unsigned long long z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

void set_norm(chgpu_mlp* m, const chgpu_mlp_norm& u) {
  m->user = u;
  for (int k = 0; k < mlp::NIN; ++k) {
    m->nm.mu_in[k] = u.mu_in[k];
    m->nm.isd_in[k] = 1.0f / u.sd_in[k];
  }
  for (int o = 0; o < mlp::NOUT; ++o) {
    m->nm.mu_out[o] = u.mu_out[o];
    m->nm.sd_out[o] = u.sd_out[o];
    m->nm.isd_out[o] = 1.0f / u.sd_out[o];
  }
}

int finish(chgpu_mlp* m) {
  MCK(m, cudaStreamSynchronize(m->stream));
  int e = 0;
  MCK(m, cudaMemcpy(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    cudaMemset(m->err, 0, sizeof(int));
    return mfail(m, CHGPU_E_CUDA, "a tensor-core completion wait ran out");
  }
  return 0;
}

}  // namespace

extern "C" {

const char* chgpu_mlp_last_error(const chgpu_mlp* m) { return m ? m->msg.c_str() : g_mlp_create_error.c_str(); }

int chgpu_mlp_create(unsigned long long seed, chgpu_mlp** out) {
  if (!out) return mfail(nullptr, CHGPU_E_PARAM, "chgpu_mlp_create: null argument");
  *out = nullptr;
  int dev = 0, major = 0, minor = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (e != cudaSuccess) return mcuda(nullptr, e, "chgpu_mlp_create");
  if (major != 10 || minor != 3)
    return mfail(nullptr, CHGPU_E_PARAM, "chgpu_mlp_create: needs a compute-capability 10.3 GPU (GB300)");
  if (mlp_set_smem_limits() != 0) return mfail(nullptr, CHGPU_E_CUDA, "chgpu_mlp_create: shared-memory limit refused");
  chgpu_mlp* m = new (std::nothrow) chgpu_mlp();
  if (!m) return mfail(nullptr, CHGPU_E_NOMEM, "chgpu_mlp_create: host allocation failed");
  cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t pb = CHGPU_MLP_NPARAMS * sizeof(float);
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&m->theta, pb) != cudaSuccess || cudaMalloc(&m->grad, pb) != cudaSuccess ||
      cudaMalloc(&m->m1, pb) != cudaSuccess || cudaMalloc(&m->m2, pb) != cudaSuccess ||
      cudaMalloc(&m->packed, mlp::PACKED_BYTES) != cudaSuccess || cudaMalloc(&m->err, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&m->nm_dev, sizeof(mlp::Norm)) != cudaSuccess) {
    chgpu_mlp_destroy(m);
    return mfail(nullptr, CHGPU_E_NOMEM, "chgpu_mlp_create: device allocation failed");
  }
  cudaMemset(m->grad, 0, pb);
  cudaMemset(m->m1, 0, pb);
  cudaMemset(m->m2, 0, pb);
  cudaMemset(m->err, 0, sizeof(int));
  std::vector<float> th(CHGPU_MLP_NPARAMS, 0.0f);
  unsigned long long s = seed;
  auto fill = [&](int off, int rows, int cols, int fan_in, int ncols_used, double gain) {
    const double a = std::sqrt(gain / fan_in);
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c) th[off + r * cols + c] = c < ncols_used ? (float)(a * uniform_pm1(s)) : 0.0f;
  };
  fill(mlp::OFF_W1, 64, 16, mlp::NIN, mlp::NIN, 6.0);
  fill(mlp::OFF_W2, 64, 64, 64, 64, 6.0);
  fill(mlp::OFF_W3, 64, 64, 64, 64, 6.0);
  fill(mlp::OFF_W4, mlp::NOUT, 64, 64, 64, 3.0);
  chgpu_mlp_norm id{};
  for (int k = 0; k < mlp::NIN; ++k) id.sd_in[k] = 1.0f;
  for (int o = 0; o < mlp::NOUT; ++o) id.sd_out[o] = 1.0f;
  set_norm(m, id);
  *out = m;
  if (int rc = chgpu_mlp_set_norm(m, &id)) return rc;
  return chgpu_mlp_set_params(m, th.data());
}

int chgpu_mlp_destroy(chgpu_mlp* m) {
  if (!m) return 0;
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->theta);
  cudaFree(m->grad);
  cudaFree(m->m1);
  cudaFree(m->m2);
  cudaFree(m->packed);
  cudaFree(m->feat);
  cudaFree(m->targ);
  cudaFree(m->loss);
  cudaFree(m->err);
  cudaFree(m->nm_dev);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return 0;
}

int chgpu_mlp_set_params(chgpu_mlp* m, const float* theta) {
  if (!m || !theta) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_set_params: null argument");
  MCK(m, cudaMemcpyAsync(m->theta, theta, CHGPU_MLP_NPARAMS * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  launch_mlp_pack(m->theta, m->packed, m->stream);
  MCK(m, cudaGetLastError());
  return finish(m);
}

int chgpu_mlp_get_params(chgpu_mlp* m, float* theta) {
  if (!m || !theta) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_get_params: null argument");
  MCK(m, cudaMemcpyAsync(theta, m->theta, CHGPU_MLP_NPARAMS * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  return finish(m);
}

int chgpu_mlp_set_norm(chgpu_mlp* m, const chgpu_mlp_norm* nm) {
  if (!m || !nm) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_set_norm: null argument");
  for (int k = 0; k < mlp::NIN; ++k)
    if (!(nm->sd_in[k] > 0.0f) || !std::isfinite(nm->mu_in[k]))
      return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_set_norm: sd_in must be positive and mu_in finite");
  for (int o = 0; o < mlp::NOUT; ++o)
    if (!(nm->sd_out[o] > 0.0f) || !std::isfinite(nm->mu_out[o]))
      return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_set_norm: sd_out must be positive and mu_out finite");
  set_norm(m, *nm);
  MCK(m, cudaMemcpyAsync(m->nm_dev, &m->nm, sizeof(mlp::Norm), cudaMemcpyHostToDevice, m->stream));
  return finish(m);
}

int chgpu_mlp_get_norm(chgpu_mlp* m, chgpu_mlp_norm* nm) {
  if (!m || !nm) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_get_norm: null argument");
  *nm = m->user;
  return 0;
}

int chgpu_mlp_set_data(chgpu_mlp* m, const float* feat, const float* targ, long long n) {
  if (!m || !feat || !targ || n < 128) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_set_data: need n >= 128 points");
  MCK(m, cudaStreamSynchronize(m->stream));
  cudaFree(m->feat);
  cudaFree(m->targ);
  m->feat = m->targ = nullptr;
  m->n = 0;
  if (cudaMalloc(&m->feat, (size_t)n * mlp::NIN * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m->targ, (size_t)n * mlp::NOUT * sizeof(float)) != cudaSuccess)
    return mfail(m, CHGPU_E_NOMEM, "chgpu_mlp_set_data: device allocation failed");
  MCK(m, cudaMemcpyAsync(m->feat, feat, (size_t)n * mlp::NIN * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(m, cudaMemcpyAsync(m->targ, targ, (size_t)n * mlp::NOUT * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  m->n = n;
  m->cursor = 0;
  return finish(m);
}

long long chgpu_mlp_data_size(const chgpu_mlp* m) { return m ? m->n : 0; }

int chgpu_mlp_gradient(chgpu_mlp* m, long long first, long long count, float* grad, double* loss) {
  if (!m) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_gradient: null handle");
  if (m->n == 0) return mfail(m, CHGPU_E_STATE, "chgpu_mlp_gradient: no training data");
  if (count < 128 || count % 128 || first < 0)
    return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_gradient: count must be a positive multiple of 128, first >= 0");
  if (count / 128 > (1LL << 30)) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_gradient: count too large");
  if (!m->loss || m->loss_cap < 1) {
    cudaFree(m->loss);
    if (cudaMalloc(&m->loss, sizeof(double)) != cudaSuccess) return mfail(m, CHGPU_E_NOMEM, "loss buffer");
    m->loss_cap = 1;
  }
  float* gbuf = nullptr;
  if (cudaMalloc(&gbuf, CHGPU_MLP_NPARAMS * sizeof(float)) != cudaSuccess)
    return mfail(m, CHGPU_E_NOMEM, "gradient buffer");
  cudaMemsetAsync(gbuf, 0, CHGPU_MLP_NPARAMS * sizeof(float), m->stream);
  cudaMemsetAsync(m->loss, 0, sizeof(double), m->stream);
  const float gscale = (float)(2.0 / ((double)count * mlp::NOUT));
  launch_mlp_train(m->packed, m->feat, m->targ, m->n, first % m->n, (int)(count / 128), m->nm, gscale, gbuf, m->loss,
                   m->err, m->nsm, m->stream);
  cudaError_t e = cudaGetLastError();
  double l = 0;
  if (e == cudaSuccess && grad)
    e = cudaMemcpyAsync(grad, gbuf, CHGPU_MLP_NPARAMS * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&l, m->loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream);
  int rc = e == cudaSuccess ? finish(m) : mcuda(m, e, "chgpu_mlp_gradient");
  cudaFree(gbuf);
  if (rc == 0 && loss) *loss = l / ((double)count * mlp::NOUT);
  return rc;
}

int chgpu_mlp_train(chgpu_mlp* m, int steps, long long batch, float lr, double* loss_out) {
  if (!m) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_train: null handle");
  if (m->n == 0) return mfail(m, CHGPU_E_STATE, "chgpu_mlp_train: no training data");
  if (steps < 0 || batch < 128 || batch % 128 || !(lr > 0.0f))
    return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_train: need steps >= 0, batch a positive multiple of 128, lr > 0");
  if (batch / 128 > (1LL << 30)) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_train: batch too large");
  if (steps == 0) return 0;
  if (m->loss_cap < steps) {
    cudaFree(m->loss);
    m->loss = nullptr;
    m->loss_cap = 0;
    if (cudaMalloc(&m->loss, (size_t)steps * sizeof(double)) != cudaSuccess)
      return mfail(m, CHGPU_E_NOMEM, "loss buffer");
    m->loss_cap = steps;
  }
  MCK(m, cudaMemsetAsync(m->loss, 0, (size_t)steps * sizeof(double), m->stream));
  const float gscale = (float)(2.0 / ((double)batch * mlp::NOUT));
  for (int s = 0; s < steps; ++s) {
    launch_mlp_train(m->packed, m->feat, m->targ, m->n, m->cursor, (int)(batch / 128), m->nm, gscale, m->grad,
                     m->loss + s, m->err, m->nsm, m->stream);
    launch_adam(m->theta, m->grad, m->m1, m->m2, CHGPU_MLP_NPARAMS, lr, ++m->adam_t, m->stream);
    launch_mlp_pack(m->theta, m->packed, m->stream);
    m->cursor = (m->cursor + batch) % m->n;
  }
  MCK(m, cudaGetLastError());
  std::vector<double> l(steps);
  MCK(m, cudaMemcpyAsync(l.data(), m->loss, (size_t)steps * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  if (int rc = finish(m)) return rc;
  if (loss_out)
    for (int s = 0; s < steps; ++s) loss_out[s] = l[s] / ((double)batch * mlp::NOUT);
  return 0;
}

int chgpu_mlp_predict(chgpu_mlp* m, const float* feat, long long n, float* out) {
  if (!m || !feat || !out || n < 1) return mfail(m, CHGPU_E_PARAM, "chgpu_mlp_predict: null argument or n < 1");
  float *df = nullptr, *dout = nullptr;
  if (cudaMalloc(&df, (size_t)n * mlp::NIN * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&dout, (size_t)n * mlp::NOUT * sizeof(float)) != cudaSuccess) {
    cudaFree(df);
    return mfail(m, CHGPU_E_NOMEM, "chgpu_mlp_predict: device allocation failed");
  }
  cudaError_t e = cudaMemcpyAsync(df, feat, (size_t)n * mlp::NIN * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) {
    launch_mlp_infer(m->packed, df, n, m->nm_dev, dout, m->err, m->nsm, m->stream);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, dout, (size_t)n * mlp::NOUT * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
  const int rc = e == cudaSuccess ? finish(m) : mcuda(m, e, "chgpu_mlp_predict");
  cudaFree(df);
  cudaFree(dout);
  return rc;
}

}  // extern "C"

// Layout of the subgrid-stress network's parameters, operand tiles, shared
// memory and tensor memory (mlp.cu), and its launches.
#pragma once

#include <cuda_runtime.h>

struct chgpu_mlp;

namespace chgpu {
namespace mlp {

constexpr int NIN = 10, NH = 64, NOUT = 6;
// FP32 parameter vector (the order of chgpu_closure.h)
constexpr int OFF_W1 = 0, OFF_W2 = 1024, OFF_B2 = 5120, OFF_W3 = 5184, OFF_B3 = 9280, OFF_W4 = 9344, OFF_B4 = 9728;
constexpr int NPARAMS = 9734;

// Byte offset of element (r, k) of a [rows x K] BF16 operand, K-major, in
// the canonical no-swizzle layout: 8x8 core matrices of 128 contiguous
// bytes, adjacent along K 128 bytes apart, 8-row groups K*16 bytes apart.
__host__ __device__ constexpr int core_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// packed operand block (bytes): B operands of the forward products (W, rows =
// outputs), of the backward data products (W^T, rows = inputs), FP32 biases
constexpr int P_W1 = 0;       // [64 x 16]
constexpr int P_W2 = 2048;    // [64 x 64]
constexpr int P_W3 = 10240;   // [64 x 64]
constexpr int P_W4 = 18432;   // [16 x 64], rows 6..15 zero
constexpr int P_W4T = 20480;  // [64 x 16], columns 6..15 zero
constexpr int P_W3T = 22528;  // [64 x 64]
constexpr int P_W2T = 30720;  // [64 x 64]
constexpr int P_BIAS = 38912; // b2[64], b3[64], b4[16]
constexpr int PACKED_BYTES = 39488;

// shared memory of the training kernel
constexpr int S_X = 39936;          // input tile [128 x 16], point-major
constexpr int S_PA = S_X + 4096;    // [128 x 64] ping
constexpr int S_PB = S_PA + 16384;  // [128 x 64] pong
constexpr int S_DY = S_PB + 16384;  // dL/dy [128 x 16]
constexpr int S_T = S_DY + 4096;    // transposed operands: rows x 128 points, 2048 bytes per 8 rows
// 8-row groups of the transposed region.  A weight-gradient product reads
// 128 rows from the start of an H^T: its 64 (16) rows, then the group of
// ones (lane 64 -> the bias gradient), then rows whose lanes are unused.
constexpr int G_XT = 0, G_H1T = 2, G_ONE1 = 10, G_H2T = 11, G_ONE2 = 19, G_H3T = 20, G_ONE3 = 28;
constexpr int G_DYT = 29, G_DZ3T = 31, G_DZ2T = 39, G_DZ1T = 47, G_END = 55;
constexpr int S_END = S_T + G_END * 2048;  // 193 536 bytes
// shared memory of the inference kernel: the forward operands W1..W4 (the
// first P_W4T bytes of the packed block), the biases, the input tile and one
// activation tile (each layer's epilogue overwrites the operand its product
// has finished reading)
constexpr int SI_BIAS = P_W4T;                 // 20480
constexpr int SI_X = 21504;                    // [128 x 16]
constexpr int SI_H = SI_X + 4096;              // [128 x 64]
constexpr int S_INFER_END = SI_H + 16384;      // 41 984 bytes

// tensor-memory columns (FP32, 128 lanes)
constexpr unsigned C_Z1 = 0, C_Z2 = 64, C_Z3 = 128, C_Y4 = 192, C_DH = 208;
constexpr unsigned C_DW1 = 272, C_DW2 = 336, C_DW3 = 400, C_DW4 = 464;
constexpr unsigned kTrainCols = 512;
constexpr unsigned I_Z = 0, kInferCols = 64;  // every layer's accumulator in the same 64 columns

struct Norm {
  float mu_in[NIN], isd_in[NIN];
  float mu_out[NOUT], sd_out[NOUT], isd_out[NOUT];
};

}  // namespace mlp

int mlp_set_smem_limits();
void launch_mlp_pack(const float* theta, unsigned char* packed, cudaStream_t s);
void launch_mlp_train(const unsigned char* packed, const float* feat, const float* targ, long long n, long long first,
                      int tiles, const mlp::Norm& nm, float gscale, float* grad, double* loss, int* err, int nsm,
                      cudaStream_t s);
void launch_mlp_infer(const unsigned char* packed, const float* feat, long long n, const mlp::Norm* nm, float* out,
                      int* err, int nsm, cudaStream_t s);
// tau at the closure points (planes iy = 1..ny-1) of phys[9][plane][plane_pts]
// -> tau[6][plane][plane_pts]; a wait that runs out ors errbit into *err
void launch_mlp_closure(const chgpu_mlp* m, const float* phys, float* tau, const float* wd, long long plane_pts,
                        int nplanes, int ny, int* err, int errbit, int nsm, cudaStream_t s);
void launch_adam(float* theta, float* g, float* m1, float* m2, int n, float lr, int t, cudaStream_t s);

}  // namespace chgpu

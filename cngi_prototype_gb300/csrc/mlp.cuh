// Parameter layout of the learned-GCF network (see mlp.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ngg.h"

namespace ngg {

constexpr int MLP_OFF_W[4] = {0, 4160, 8320, 12480};       // W1..W4 [64][64]
constexpr int MLP_OFF_b[4] = {4096, 8256, 12416, 16576};   // b1..b4 [64]
constexpr int MLP_LAYER = 4160;                           // W_k + b_k
constexpr int MLP_OFF_WO = 16640;                          // Wo [64]
constexpr int MLP_OFF_BO = 16704;                          // bo
constexpr int MLP_OFF_B = 16705;                           // B [32][4], fixed
constexpr int MLP_N_TRAINED = 16705;
static_assert(MLP_OFF_B + 128 == NGG_MLP_NPARAM, "parameter layout");
static_assert(MLP_N_TRAINED == NGG_MLP_NTRAINED, "parameter layout");

constexpr int SP_TABLE = 32;   // columns per tap row of the mosaic gridder's table

// the mosaic gridder's reorganised table ckt[c][oui][ovi][2S][32] for every
// channel from the network (mlp_tc.cu)
int mlp_synth_table(const float *params, const NggMlpScale *scale, const double *freq, int64_t C, int os0, int os1,
                    int S, const int32_t *support, float *ckt, cudaStream_t s);

}  // namespace ngg

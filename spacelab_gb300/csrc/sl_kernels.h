// sl_kernels.h -- host-side launch interface of the step kernels.
#pragma once
#include "sl_device.cuh"

namespace sl {

constexpr int kRedBlocks = 64;  // energy reduction partial blocks

// Optional per-kernel CUDA events recorded between the launches of a step:
// ev[0] after the drift, ev[1] after the pair tiles, ev[2] after the row sums.
struct StepTimers {
    cudaEvent_t ev[3];
};

void launch_derive(const System& s, cudaStream_t st);
void launch_step(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm);
int pair_grid_blocks(const System& s, int num_sms);

}  // namespace sl

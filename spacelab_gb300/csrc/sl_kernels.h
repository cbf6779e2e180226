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

constexpr int kPairPhases = 5;

// A side stream and events that let the row sums of one pair phase run
// while the next phases' pair tiles are computed.  NULL: one pair launch,
// then one row-sum launch, on the main stream only.
struct StepOverlap {
    cudaStream_t side;
    cudaEvent_t phase[kPairPhases];
    cudaEvent_t join;
};

void launch_derive(const System& s, cudaStream_t st);
void launch_step(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm,
                 const StepOverlap* ov = nullptr);
void launch_step_mixed(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm);
void launch_drift(const System& s, cudaStream_t st);
void launch_energy(const System& s, cudaStream_t st);
int pair_grid_blocks(long long tiles, int num_sms);
// Block-column bounds cb[0..np] of the pipelined step's pair phases; returns np.
int phase_bounds(int nb, int* cb);

}  // namespace sl

// sl_kernels.h -- host-side launch interface of the step kernels.
#pragma once
#include <cuda.h>

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
// vec3[n] AoS arrays src[k] / dst[k] (device-accessible: device staging,
// or host memory the GPU reads and writes directly) <-> the SoA arrays
// arr[k]: in, for the arrays whose bit is set in `present` (others: arr[5],
// the previous positions, takes the positions; the rest zero); out, for the
// arrays whose bit is set in `want`.  check: arrays of `present` whose
// non-finite values set kStatusInputNonFiniteBit; guard: stage_out writes
// nothing once that bit is set.
void launch_stage_in(const System& s, const double* const src[6], Vec3Soa* const arr[6], unsigned present,
                     cudaStream_t st, unsigned check = 0);
void launch_stage_out(const System& s, double* const dst[6], Vec3Soa* const arr[6], unsigned want, cudaStream_t st,
                      bool guard = false);
// map: a tensor map of the pair-term buffer (make_pair_map) selects the
// TMA-streamed row sums; NULL the plain-load form.
void launch_step(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm,
                 const StepOverlap* ov = nullptr, const CUtensorMap* map = nullptr, bool int_adds = true);
// Prepares the TMA row sums of the exact form: the tensor map of the
// pair-term buffer (FP64) and the kernels' shared-memory limits; false if
// that fails (the plain-load row sums are used then).
bool make_pair_map(const System& s, CUtensorMap* map);
// The TMA-streamed ordered row sums over partner blocks [b0, b1) with terms
// of type T (double); first/last as for the plain row sums.  int_adds: each
// FP64 addition on the integer pipe (rowsum_int_kernel), else on the FP64
// unit (rowsum_tma_kernel); the sums are identical.
template <typename T>
void launch_rowsum_tma(const System& s, const CUtensorMap& map, int b0, int b1, int first, int last, int num_sms,
                       bool int_adds, cudaStream_t st);
// Status bit set by a kernel whose bounded wait for a TMA copy ran out.
constexpr unsigned kStatusWaitTimeoutBit = 2u;
// Status bit set by stage_in for a non-finite value of a checked input array
// (launch_stage_in's `check` mask); a guarded stage_out then writes nothing.
constexpr unsigned kStatusInputNonFiniteBit = 0x40000000u;
// The double-float mixed form (SL_MODE_MIXED_DF, sl_step_mixed.cu).
void launch_step_mixed(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm);
// The mixed form with FP64 displacements, overlaps and accumulation
// (SL_MODE_MIXED, sl_step_mixed64.cu).
void launch_step_mixed64(const System& s, bool write, int num_sms, cudaStream_t st, StepTimers* tm);
// Whether the mixed pair kernel takes two column blocks per item (mixed_pair_items)
// for nb row blocks on num_sms SMs: where each warp takes many items.
bool mixed_pair_double(int nb, int num_sms);
void launch_drift(const System& s, cudaStream_t st);
void launch_energy(const System& s, cudaStream_t st);
int pair_grid_blocks(long long tiles, int num_sms);
// Block-column bounds cb[0..np] of the pipelined step's pair phases; returns np.
int phase_bounds(int nb, int* cb);

}  // namespace sl

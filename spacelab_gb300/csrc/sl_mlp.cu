// sl_mlp.cu -- the collision-outcome surrogate: an MLP (n_in -> H x L hidden
// layers with GELU -> n_out) with BF16 weights and activations and FP32
// accumulation, trained and evaluated on the GPU by this file's kernels
// (include/spacelab_mlp.h).
//
// Every matrix product is one kernel, gemm_nt_tc: C[M][N] = A[M][K] . B[N][K]^T
// with A and B bf16 row-major (K contiguous) on the fifth-generation tensor
// cores: TMA copies of 128-byte-swizzled K chunks into shared memory,
// tcgen05.mma (M = 128, N <= 128, K = 16, bf16 x bf16 -> f32) into a tensor
// memory accumulator, tcgen05.ld back to registers for the epilogue, which
// adds the bias and writes the FP32 pre-activation and/or the BF16
// activation (GELU or identity).
//   forward   Z_l = X_l W_l^T + b_l,  X_{l+1} = bf16(GELU(Z_l))
//   backward  dW_l = dZ_l^T X_l   (A = dZ^T, B = X^T: transposed copies)
//             dX_l = dZ_l W_l     (B = W^T: a transposed copy of W)
//             dZ_{l-1} = bf16(dX_l * GELU'(Z_{l-1}))
// Widths are padded to multiples of 32 with zero weights that stay zero
// (their gradients are zero).  FP32 master weights are updated with Adam;
// bf16 copies feed the GEMMs.  An mma.sync m16n8k16 kernel (gemm_nt_kernel)
// is kept only as the second opinion of sl_diag_gemm_bf16.
#include "../../include/spacelab_mlp.h"
#include "../../include/spacelab_gpu.h"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include "sl_tma.cuh"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <random>
#include <string>
#include <vector>

int sl_record_error(int code, const char* msg);

namespace {

using bf16 = __nv_bfloat16;

constexpr int kTM = 64, kTN = 64, kTK = 32, kPadK = 8;  // CTA tile; smem row pad (bank spread)

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm_x2(uint32_t& r0, uint32_t& r1, const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float z)
{
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
    return cdf + z * pdf;
}

// C = A . B^T for bf16 A[M][K] (lda), B[N][K] (ldb); K % 32 == 0; any M, N.
// act: 0 identity, 1 GELU (applied to the bf16 output only).
__global__ void __launch_bounds__(128) gemm_nt_kernel(const bf16* __restrict__ A, int lda, const bf16* __restrict__ B,
                                                      int ldb, const float* __restrict__ bias, float* Cf, bf16* Cb,
                                                      int ldc, int M, int N, int K, int act)
{
    __shared__ __align__(16) bf16 As[kTM][kTK + kPadK];
    __shared__ __align__(16) bf16 Bs[kTN][kTK + kPadK];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
    float acc[2][4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kTK) {
        // 64 rows x 32 bf16 = 4 16-byte chunks per row; 128 threads x 2 chunks per matrix
        for (int q = tid; q < kTM * 4; q += 128) {
            const int r = q >> 2, c = (q & 3) * 8;
            uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
            if (m0 + r < M) va = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * lda + k0 + c);
            if (n0 + r < N) vb = *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * ldb + k0 + c);
            *reinterpret_cast<uint4*>(&As[r][c]) = va;
            *reinterpret_cast<uint4*>(&Bs[r][c]) = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTK; kk += 16) {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
                ldsm_x4(a[mt][0], a[mt][1], a[mt][2], a[mt][3], &As[wm + mt * 16 + (lane & 15)][kk + (lane >> 4) * 8]);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
                ldsm_x2(b[nt][0], b[nt][1], &Bs[wn + nt * 8 + (lane & 7)][kk + ((lane >> 3) & 1) * 8]);
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt)
                    mma_bf16(acc[mt][nt], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b[nt][0], b[nt][1]);
        }
        __syncthreads();
    }
    const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = m0 + wm + mt * 16 + g + h * 8;
                const int col = n0 + wn + nt * 8 + t4 * 2;
                if (row >= M) continue;
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    if (col + e >= N) continue;
                    float v = acc[mt][nt][2 * h + e] + (bias ? bias[col + e] : 0.0f);
                    if (Cf) Cf[(size_t)row * ldc + col + e] = v;
                    if (Cb) Cb[(size_t)row * ldc + col + e] = __float2bfloat16(act ? gelu(v) : v);
                }
            }
}

// ------------------------------------------------------------- tcgen05 --
// C[M][N] = A[M][K] . B[N][K]^T on the fifth-generation tensor cores.  One
// CTA (4 warps) per 128-row block of C and BN columns; its accumulator is
// BN f32 columns x 128 lanes of tensor memory (TMEM).  K is taken in chunks
// of 64 elements (128 bytes): TMA copies the A and B chunks into shared
// memory with the 128-byte swizzle -- the K-major layout the MMA's shared-
// memory descriptors describe (8-row groups 1024 bytes apart) -- into one of
// two stages, and one thread issues four tcgen05.mma (M=128, N=BN, K=16)
// per chunk, then tcgen05.commit to the stage's barrier so that the next
// copy into that stage waits for the MMAs reading it.  Boxes past M, N or K
// are zero-filled by the copy engine.  The epilogue: warp w reads TMEM
// lanes 32w..32w+31 (rows m0 + 32w + lane) 32 columns at a time with
// tcgen05.ld, adds the bias and writes the FP32 and/or BF16 (GELU or
// identity) outputs.  Every wait is bounded (sl_tma.cuh); a wait that runs
// out sets *err, the CTA waits (bounded) for its MMAs, frees its TMEM and
// returns.
constexpr int kTcM = 128, kTcK = 64, kTcStages = 2;
constexpr int kTcThreads = 128;

template <int BN>
struct TcSmem {
    static constexpr int kABytes = kTcM * kTcK * 2;  // 16 KB
    static constexpr int kBBytes = BN * kTcK * 2;
    static constexpr int kBytes = kTcStages * (kABytes + kBBytes) + 1024 /* barriers etc. */ + 1024 /* alignment */;
};

// Shared-memory matrix descriptor of a K-major tile with the 128-byte
// swizzle: start address >> 4 (bits 0-13), leading byte offset (unused for
// this layout; 16 bytes, bits 16-29), stride byte offset 1024 = 8 rows x 128
// bytes (bits 32-45), descriptor version 1 (bits 46-47), base offset 0 (the
// tile is 1024-byte aligned), layout SWIZZLE_128B = 2 (bits 61-63).  The
// K = 16 sub-steps within a 128-byte row advance the start address by 32
// bytes.
__device__ __forceinline__ uint64_t tc_desc_sw128(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3fffu) | ((uint64_t)(16 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (bits
// 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives on `bar` once every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void tc_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(sl::tma::smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive f32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

template <int BN>
__global__ void __launch_bounds__(kTcThreads) gemm_nt_tc_kernel(const __grid_constant__ CUtensorMap mapA,
                                                                 const __grid_constant__ CUtensorMap mapB,
                                                                 const float* __restrict__ bias, float* Cf, bf16* Cb,
                                                                 int ldc, int M, int N, int K, int act, int* err)
{
    using Sm = TcSmem<BN>;
    extern __shared__ unsigned char tc_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) &
                                                           ~static_cast<uintptr_t>(1023));
    unsigned char* sa = base;                                  // [stage][128 rows][128 B]
    unsigned char* sb = base + kTcStages * Sm::kABytes;        // [stage][BN rows][128 B]
    uint64_t* full = reinterpret_cast<uint64_t*>(sb + kTcStages * Sm::kBBytes);
    uint64_t* empty = full + kTcStages;
    uint64_t* done = empty + kTcStages;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    int* failed = reinterpret_cast<int*>(tmem_slot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * BN;
    const int nk = (K + kTcK - 1) / kTcK;

    if (tid == 0) {
        for (int st = 0; st < kTcStages; ++st) {
            sl::tma::mbar_init(&full[st], 1);
            sl::tma::mbar_init(&empty[st], 1);
        }
        sl::tma::mbar_init(done, 1);
        *failed = 0;
        sl::tma::fence_barrier_init();
    }
    if (warp == 0) {  // BN f32 columns of TMEM (a power of two >= 32)
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(sl::tma::smem_addr(tmem_slot)), "r"(BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (tid == 0) {
        constexpr uint32_t idesc = tc_idesc_bf16(kTcM, BN);
        const uint32_t bytes = Sm::kABytes + Sm::kBBytes;
        auto issue = [&](int kc) {
            const int st = kc % kTcStages;
            sl::tma::mbar_arrive_expect_tx(&full[st], bytes);
            sl::tma::load_2d(sa + st * Sm::kABytes, &mapA, kc * kTcK, m0, &full[st]);
            sl::tma::load_2d(sb + st * Sm::kBBytes, &mapB, kc * kTcK, n0, &full[st]);
        };
        int issued = 0;
        for (; issued < nk && issued < kTcStages; ++issued) issue(issued);
        bool ok = true;
        int kc = 0;
        for (; kc < nk && ok; ++kc) {
            const int st = kc % kTcStages;
            const uint32_t par = (uint32_t)(kc / kTcStages) & 1u;
            if (!sl::tma::mbar_wait(&full[st], par)) { ok = false; break; }
            tc_fence_after();
            const uint32_t a0 = sl::tma::smem_addr(sa + st * Sm::kABytes);
            const uint32_t b0 = sl::tma::smem_addr(sb + st * Sm::kBBytes);
#pragma unroll
            for (int k = 0; k < kTcK / 16; ++k)
                tc_mma(tmem, tc_desc_sw128(a0 + 32 * k), tc_desc_sw128(b0 + 32 * k), idesc, (kc | k) != 0);
            tc_commit(&empty[st]);
            if (kc + kTcStages < nk) {
                // the stage's next copy waits for the MMAs that read it
                if (!sl::tma::mbar_wait(&empty[st], par)) { ok = false; ++kc; break; }
                issue(kc + kTcStages);
                ++issued;
            }
        }
        tc_commit(done);  // arrives when every MMA issued above has completed
        if (!ok) {
            *failed = 1;
            // let the copies in flight land before the CTA's memory is reused
            for (int q = kc; q < issued; ++q)
                sl::tma::mbar_wait(&full[q % kTcStages], (uint32_t)(q / kTcStages) & 1u);
        }
    }
    __syncwarp();
    if (!sl::tma::mbar_wait(done, 0)) *failed = 1;
    tc_fence_after();
    __syncthreads();
    // the same decision in every thread (tcgen05.ld is warp-collective)
    if (*failed) {
        if (tid == 0) atomicExch(err, 1);
    } else {
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int cg = 0; cg < BN / 32; ++cg) {
            float v[32];
            tc_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cg * 32), v);
            if (row < M) {
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int col = n0 + cg * 32 + i;
                    if (col >= N) break;
                    const float z = v[i] + (bias ? bias[col] : 0.0f);
                    if (Cf) Cf[(size_t)row * ldc + col] = z;
                    if (Cb) Cb[(size_t)row * ldc + col] = __float2bfloat16(act ? gelu(z) : z);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}

// out[c][r] = in[r][c]
__global__ void transpose_kernel(const bf16* __restrict__ in, int rows, int cols, int ldi, bf16* out, int ldo)
{
    __shared__ bf16 t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = by + y, c = bx + threadIdx.x;
        t[y][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * ldi + c] : __float2bfloat16(0.0f);
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = bx + y, r = by + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * ldo + r] = t[threadIdx.x][y];
    }
}

// float -> bf16 rows (input features, zero padding beyond n)
__global__ void pack_input_kernel(const float* __restrict__ x, int M, int n, int ld, bf16* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * ld) return;
    const int r = i / ld, c = i - r * ld;
    out[i] = __float2bfloat16(c < n ? x[(size_t)r * n + c] : 0.0f);
}

// MSE over the first n_out columns: dZ = 2 (z - y) / (M n_out), loss partials
__global__ void mse_grad_kernel(const float* __restrict__ z, int ldz, const float* __restrict__ y, int M, int n_out,
                                bf16* dz, int ld, float* loss_partial)
{
    __shared__ float red[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < M * ld) {
        const int r = i / ld, c = i - r * ld;
        float g = 0.0f;
        if (c < n_out) {
            const float e = z[(size_t)r * ldz + c] - y[(size_t)r * n_out + c];
            l = e * e;
            g = 2.0f * e / (float)(M * n_out);
        }
        dz[i] = __float2bfloat16(g);
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_partial[blockIdx.x] = red[0];
}

// dZ = bf16(dX * GELU'(Z)) elementwise
__global__ void gelu_back_kernel(const float* __restrict__ dx, const float* __restrict__ z, int n, bf16* dz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dz[i] = __float2bfloat16(dx[i] * gelu_grad(z[i]));
}

// db[c] = sum_r dZ[r][c]  (dZ bf16 [M][ld])
__global__ void bias_grad_kernel(const bf16* __restrict__ dz, int M, int ld, int n, float* db)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    float s = 0.0f;
    for (int r = 0; r < M; ++r) s += __bfloat162float(dz[(size_t)r * ld + c]);
    db[c] = s;
}

// Adam on fp32 master parameters; refreshes the bf16 copy.  mask: the
// parameter is live (padding stays 0).
__global__ void adam_kernel(float* p, const float* g, float* m, float* v, bf16* pb, const uint8_t* mask, int n, float lr,
                            float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (mask && !mask[i]) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    if (pb) pb[i] = __float2bfloat16(pi);
}

__global__ void to_bf16_kernel(const float* __restrict__ in, bf16* out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16(in[i]);
}

int pad32(int x) { return (x + 31) / 32 * 32; }

}  // namespace

struct sl_mlp {
    int n_in = 0, hidden = 0, layers = 0, n_out = 0, max_batch = 0;
    int nl = 0;                          // linear layers = hidden layers + 1
    std::vector<int> din, dout;          // padded widths of each linear layer
    std::vector<size_t> w_off, b_off;    // offsets into the parameter vector
    size_t nparam = 0;
    float *P = nullptr, *G = nullptr, *Mom = nullptr, *Var = nullptr;  // fp32 params, grads, Adam moments
    bf16* Pb = nullptr;                  // bf16 copy of params (weights used by the GEMMs)
    uint8_t* mask = nullptr;             // live parameters
    bf16 *Wt = nullptr;                  // transposed weights scratch (max din x dout)
    std::vector<bf16*> X;                // bf16 activations per layer input [max_batch][din]
    std::vector<float*> Z;               // fp32 pre-activations per layer [max_batch][dout]
    bf16 *dZ = nullptr, *dZt = nullptr, *Xt = nullptr;
    float* dX = nullptr;
    float *xin = nullptr, *yin = nullptr, *loss_part = nullptr;
    int step = 0;
    int* d_err = nullptr;         // set by a tcgen05 GEMM whose bounded wait ran out
    bool tc_setup_failed = false; // a GEMM's tensor maps or launch attributes could not be set up
    void* arena = nullptr;
};

namespace {

void gemm_mma_sync(cudaStream_t st, const bf16* A, int lda, const bf16* B, int ldb, const float* bias, float* Cf,
                   bf16* Cb, int ldc, int M, int N, int K, int act)
{
    dim3 grid((N + kTN - 1) / kTN, (M + kTM - 1) / kTM);
    gemm_nt_kernel<<<grid, 128, 0, st>>>(A, lda, B, ldb, bias, Cf, Cb, ldc, M, N, K, act);
}

PFN_cuTensorMapEncodeTiled_v12000 mlp_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    return encode;
}

// A row-major bf16 matrix [rows][k] with leading dimension ld (elements) as a
// 2D tensor map: boxes of 64 elements (128 bytes) of k x box_rows rows, the
// 128-byte swizzle, zero fill outside the matrix.
bool make_tc_map(CUtensorMap* map, const bf16* base, int rows, int k, int ld, int box_rows)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = mlp_map_encoder();
    if (!encode || !base || (reinterpret_cast<uintptr_t>(base) & 15u) || (ld * 2) % 16) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
bool launch_tc(cudaStream_t st, const CUtensorMap& ma, const bf16* B, int ldb, const float* bias, float* Cf, bf16* Cb,
               int ldc, int M, int N, int K, int act, int* err)
{
    // set on every call: the attribute belongs to the current device's
    // context, and the call is a host-side table update
    if (cudaFuncSetAttribute(gemm_nt_tc_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcSmem<BN>::kBytes) !=
        cudaSuccess)
        return false;
    CUtensorMap mb;
    if (!make_tc_map(&mb, B, N, K, ldb, BN)) return false;
    dim3 grid((N + BN - 1) / BN, (M + kTcM - 1) / kTcM);
    gemm_nt_tc_kernel<BN><<<grid, kTcThreads, TcSmem<BN>::kBytes, st>>>(ma, mb, bias, Cf, Cb, ldc, M, N, K, act, err);
    return true;
}

// The tcgen05 GEMM; false if its tensor maps or launch attributes cannot be
// set up (the caller reports the error; nothing is launched then).
bool gemm_tc(cudaStream_t st, const bf16* A, int lda, const bf16* B, int ldb, const float* bias, float* Cf, bf16* Cb,
             int ldc, int M, int N, int K, int act, int* err)
{
    CUtensorMap ma;
    if (!make_tc_map(&ma, A, M, K, lda, kTcM)) return false;
    // at most 128 columns per CTA: the products are small (M of a few
    // hundred rows), so more, narrower CTAs spread them over more SMs
    if (N <= 32) return launch_tc<32>(st, ma, B, ldb, bias, Cf, Cb, ldc, M, N, K, act, err);
    if (N <= 64) return launch_tc<64>(st, ma, B, ldb, bias, Cf, Cb, ldc, M, N, K, act, err);
    return launch_tc<128>(st, ma, B, ldb, bias, Cf, Cb, ldc, M, N, K, act, err);
}

// Every product of the network runs on the tcgen05 GEMM.
void gemm(sl_mlp* h, cudaStream_t st, const bf16* A, int lda, const bf16* B, int ldb, const float* bias, float* Cf,
          bf16* Cb, int ldc, int M, int N, int K, int act)
{
    if (h->tc_setup_failed) return;
    if (!gemm_tc(st, A, lda, B, ldb, bias, Cf, Cb, ldc, M, N, K, act, h->d_err)) h->tc_setup_failed = true;
}

// After a synchronisation: the GEMMs' setup and bounded waits.
int mlp_status(sl_mlp* h, const char* what)
{
    if (h->tc_setup_failed)
        return sl_record_error(SL_ERR_CUDA, (std::string(what) + ": tcgen05 GEMM setup (tensor maps) failed").c_str());
    int err = 0;
    if (cudaMemcpy(&err, h->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return sl_record_error(SL_ERR_CUDA, (std::string(what) + ": reading the GEMM status failed").c_str());
    if (err)
        return sl_record_error(SL_ERR_TIMEOUT,
                               (std::string(what) + ": a bounded wait in the tcgen05 GEMM ran out").c_str());
    return SL_OK;
}

void transpose(cudaStream_t st, const bf16* in, int rows, int cols, int ldi, bf16* out, int ldo)
{
    dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
    transpose_kernel<<<grid, block, 0, st>>>(in, rows, cols, ldi, out, ldo);
}

// forward over M rows of xin (already on device); the output pre-activation
// of the last layer is Z[nl-1] ([M][dout_last], fp32)
void forward(sl_mlp* h, int M, cudaStream_t st)
{
    const int ld0 = h->din[0];
    pack_input_kernel<<<(M * ld0 + 255) / 256, 256, 0, st>>>(h->xin, M, h->n_in, ld0, h->X[0]);
    for (int l = 0; l < h->nl; ++l) {
        const bool last = l == h->nl - 1;
        gemm(h, st, h->X[l], h->din[l], h->Pb + h->w_off[l], h->din[l], h->P + h->b_off[l], h->Z[l],
             last ? nullptr : h->X[l + 1], h->dout[l], M, h->dout[l], h->din[l], last ? 0 : 1);
    }
}

// backward for M rows with targets yin; fills G
void backward(sl_mlp* h, int M, cudaStream_t st)
{
    const int L = h->nl;
    const int ldo = h->dout[L - 1];
    const int nb = (M * ldo + 255) / 256;
    mse_grad_kernel<<<nb, 256, 0, st>>>(h->Z[L - 1], ldo, h->yin, M, h->n_out, h->dZ, ldo, h->loss_part);
    for (int l = L - 1; l >= 0; --l) {
        const int K = h->din[l], N = h->dout[l];
        // dW = dZ^T X : A = dZ^T [N][M], B = X^T [K][M]
        transpose(st, h->dZ, M, N, N, h->dZt, M);
        transpose(st, h->X[l], M, K, K, h->Xt, M);
        gemm(h, st, h->dZt, M, h->Xt, M, nullptr, h->G + h->w_off[l], nullptr, K, N, K, M, 0);
        bias_grad_kernel<<<(N + 127) / 128, 128, 0, st>>>(h->dZ, M, N, N, h->G + h->b_off[l]);
        if (l == 0) break;
        // dX = dZ W : A = dZ [M][N], B = W^T [K][N]
        transpose(st, h->Pb + h->w_off[l], N, K, K, h->Wt, N);
        gemm(h, st, h->dZ, N, h->Wt, N, nullptr, h->dX, nullptr, K, M, K, N, 0);
        gelu_back_kernel<<<(M * K + 255) / 256, 256, 0, st>>>(h->dX, h->Z[l - 1], M * K, h->dZ);
    }
}

}  // namespace

extern "C" {

int sl_mlp_create(int n_in, int hidden, int hidden_layers, int n_out, int max_batch, uint64_t seed, sl_mlp** out)
{
    if (!out) return sl_record_error(SL_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n_in < 1 || hidden < 1 || hidden_layers < 1 || n_out < 1 || max_batch < 32 || max_batch % 32)
        return sl_record_error(SL_ERR_ARG, "need n_in, hidden, layers, n_out >= 1 and max_batch a multiple of 32");
    sl_mlp* h = new (std::nothrow) sl_mlp();
    if (!h) return sl_record_error(SL_ERR_ALLOC, "host allocation failed");
    h->n_in = n_in; h->hidden = hidden; h->layers = hidden_layers; h->n_out = n_out; h->max_batch = max_batch;
    h->nl = hidden_layers + 1;
    for (int l = 0; l < h->nl; ++l) {
        h->din.push_back(pad32(l == 0 ? n_in : hidden));
        h->dout.push_back(pad32(l == h->nl - 1 ? n_out : hidden));
    }
    size_t off = 0;
    for (int l = 0; l < h->nl; ++l) {
        h->w_off.push_back(off); off += (size_t)h->din[l] * h->dout[l];
        h->b_off.push_back(off); off += (size_t)h->dout[l];
    }
    h->nparam = off;
    int maxw = 0;
    for (int l = 0; l < h->nl; ++l) maxw = std::max(maxw, std::max(h->din[l], h->dout[l]));
    // one arena
    size_t bytes = 0;
    auto take = [&](size_t b) { size_t o = bytes; bytes = (bytes + b + 255) / 256 * 256; return o; };
    const size_t oP = take(off * 4), oG = take(off * 4), oM = take(off * 4), oV = take(off * 4), oPb = take(off * 2),
                 oMask = take(off), oWt = take((size_t)maxw * maxw * 2);
    std::vector<size_t> oX, oZ;
    for (int l = 0; l < h->nl; ++l) {
        oX.push_back(take((size_t)max_batch * h->din[l] * 2));
        oZ.push_back(take((size_t)max_batch * h->dout[l] * 4));
    }
    const size_t odZ = take((size_t)max_batch * maxw * 2), odZt = take((size_t)max_batch * maxw * 2),
                 oXt = take((size_t)max_batch * maxw * 2), odX = take((size_t)max_batch * maxw * 4),
                 oxin = take((size_t)max_batch * n_in * 4), oyin = take((size_t)max_batch * n_out * 4),
                 oloss = take(((size_t)max_batch * maxw / 256 + 1) * 4), oerr = take(sizeof(int));
    if (cudaMalloc(&h->arena, bytes) != cudaSuccess) {
        delete h;
        return sl_record_error(SL_ERR_ALLOC, "cudaMalloc of the MLP arena failed");
    }
    char* b = static_cast<char*>(h->arena);
    h->P = (float*)(b + oP); h->G = (float*)(b + oG); h->Mom = (float*)(b + oM); h->Var = (float*)(b + oV);
    h->Pb = (bf16*)(b + oPb); h->mask = (uint8_t*)(b + oMask); h->Wt = (bf16*)(b + oWt);
    for (int l = 0; l < h->nl; ++l) { h->X.push_back((bf16*)(b + oX[l])); h->Z.push_back((float*)(b + oZ[l])); }
    h->dZ = (bf16*)(b + odZ); h->dZt = (bf16*)(b + odZt); h->Xt = (bf16*)(b + oXt); h->dX = (float*)(b + odX);
    h->xin = (float*)(b + oxin); h->yin = (float*)(b + oyin); h->loss_part = (float*)(b + oloss);
    h->d_err = (int*)(b + oerr);
    cudaMemset(h->arena, 0, bytes);
    // He-style init of live weights, zero biases and padding
    std::vector<float> p(off, 0.0f);
    std::vector<uint8_t> mk(off, 0);
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.0f, 1.0f);
    for (int l = 0; l < h->nl; ++l) {
        const int kin = l == 0 ? n_in : hidden, nout = l == h->nl - 1 ? n_out : hidden;
        const float sd = std::sqrt(2.0f / (float)kin);
        for (int r = 0; r < nout; ++r)
            for (int c = 0; c < kin; ++c) {
                const size_t i = h->w_off[l] + (size_t)r * h->din[l] + c;
                p[i] = sd * nd(rng);
                mk[i] = 1;
            }
        for (int r = 0; r < nout; ++r) mk[h->b_off[l] + r] = 1;
    }
    cudaMemcpy(h->P, p.data(), off * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(h->mask, mk.data(), off, cudaMemcpyHostToDevice);
    to_bf16_kernel<<<(int)((off + 255) / 256), 256>>>(h->P, h->Pb, (int)off);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        sl_mlp_destroy(h);
        return sl_record_error(SL_ERR_CUDA, "MLP initialisation failed");
    }
    *out = h;
    return SL_OK;
}

int sl_mlp_destroy(sl_mlp* h)
{
    if (!h) return SL_OK;
    if (h->arena) cudaFree(h->arena);
    delete h;
    return SL_OK;
}

int sl_mlp_num_params(const sl_mlp* h, int64_t* n)
{
    if (!h || !n) return sl_record_error(SL_ERR_ARG, "null argument");
    *n = (int64_t)h->nparam;
    return SL_OK;
}

int sl_mlp_get_params(sl_mlp* h, float* params)
{
    if (!h || !params) return sl_record_error(SL_ERR_ARG, "null argument");
    if (cudaMemcpy(params, h->P, h->nparam * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return sl_record_error(SL_ERR_CUDA, "copy failed");
    return SL_OK;
}

int sl_mlp_set_params(sl_mlp* h, const float* params)
{
    if (!h || !params) return sl_record_error(SL_ERR_ARG, "null argument");
    if (cudaMemcpy(h->P, params, h->nparam * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        return sl_record_error(SL_ERR_CUDA, "copy failed");
    to_bf16_kernel<<<(int)((h->nparam + 255) / 256), 256>>>(h->P, h->Pb, (int)h->nparam);
    if (cudaDeviceSynchronize() != cudaSuccess) return sl_record_error(SL_ERR_CUDA, "bf16 refresh failed");
    return SL_OK;
}

int sl_mlp_gradients(sl_mlp* h, const float* x, const float* y, int M, float* grads, float* loss)
{
    if (!h || !x || !y || M < 32 || M % 32 || M > h->max_batch)
        return sl_record_error(SL_ERR_ARG, "M must be a multiple of 32 up to max_batch");
    cudaMemcpy(h->xin, x, (size_t)M * h->n_in * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(h->yin, y, (size_t)M * h->n_out * 4, cudaMemcpyHostToDevice);
    forward(h, M, nullptr);
    backward(h, M, nullptr);
    if (cudaDeviceSynchronize() != cudaSuccess) return sl_record_error(SL_ERR_CUDA, "MLP step failed");
    if (int r = mlp_status(h, "sl_mlp_gradients")) return r;
    if (grads) cudaMemcpy(grads, h->G, h->nparam * 4, cudaMemcpyDeviceToHost);
    if (loss) {
        const int ldo = h->dout[h->nl - 1];
        const int nb = (M * ldo + 255) / 256;
        std::vector<float> part(nb);
        cudaMemcpy(part.data(), h->loss_part, nb * 4, cudaMemcpyDeviceToHost);
        double s = 0;
        for (float v : part) s += v;
        *loss = (float)(s / ((double)M * h->n_out));
    }
    return SL_OK;
}

int sl_mlp_train(sl_mlp* h, const float* x, const float* y, int n, int epochs, int batch, float lr, uint64_t seed,
                 float* loss_per_epoch)
{
    if (!h || !x || !y || n < batch || batch < 32 || batch % 32 || batch > h->max_batch || epochs < 1)
        return sl_record_error(SL_ERR_ARG, "bad training arguments");
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::mt19937_64 rng(seed);
    std::vector<float> xb((size_t)batch * h->n_in), yb((size_t)batch * h->n_out);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const int ldo = h->dout[h->nl - 1];
    const int nb = (batch * ldo + 255) / 256;
    std::vector<float> part(nb);
    int rc = SL_OK;
    for (int ep = 0; ep < epochs && rc == SL_OK; ++ep) {
        std::shuffle(idx.begin(), idx.end(), rng);
        double ls = 0;
        int steps = 0;
        for (int s0 = 0; s0 + batch <= n; s0 += batch) {
            for (int r = 0; r < batch; ++r) {
                std::memcpy(&xb[(size_t)r * h->n_in], &x[(size_t)idx[s0 + r] * h->n_in], h->n_in * 4);
                std::memcpy(&yb[(size_t)r * h->n_out], &y[(size_t)idx[s0 + r] * h->n_out], h->n_out * 4);
            }
            cudaMemcpyAsync(h->xin, xb.data(), xb.size() * 4, cudaMemcpyHostToDevice, nullptr);
            cudaMemcpyAsync(h->yin, yb.data(), yb.size() * 4, cudaMemcpyHostToDevice, nullptr);
            forward(h, batch, nullptr);
            backward(h, batch, nullptr);
            ++h->step;
            const float c1 = 1.0f - std::pow(b1, (float)h->step), c2 = 1.0f - std::pow(b2, (float)h->step);
            adam_kernel<<<(int)((h->nparam + 255) / 256), 256>>>(h->P, h->G, h->Mom, h->Var, h->Pb, h->mask,
                                                                 (int)h->nparam, lr, b1, b2, eps, c1, c2);
            cudaMemcpy(part.data(), h->loss_part, nb * 4, cudaMemcpyDeviceToHost);
            double s = 0;
            for (float v : part) s += v;
            ls += s / ((double)batch * h->n_out);
            ++steps;
        }
        if (cudaGetLastError() != cudaSuccess) rc = sl_record_error(SL_ERR_CUDA, "training kernel failed");
        if (loss_per_epoch) loss_per_epoch[ep] = (float)(ls / std::max(1, steps));
    }
    if (cudaDeviceSynchronize() != cudaSuccess && rc == SL_OK) rc = sl_record_error(SL_ERR_CUDA, "training failed");
    if (rc == SL_OK) rc = mlp_status(h, "sl_mlp_train");
    return rc;
}

int sl_mlp_predict(sl_mlp* h, const float* x, int n, float* y)
{
    if (!h || !x || !y || n < 1) return sl_record_error(SL_ERR_ARG, "bad arguments");
    const int B = h->max_batch, L = h->nl, ldo = h->dout[L - 1];
    std::vector<float> zb((size_t)B * ldo);
    for (int s0 = 0; s0 < n; s0 += B) {
        const int M = std::min(B, n - s0);
        const int Mp = (M + 31) / 32 * 32;
        cudaMemset(h->xin, 0, (size_t)Mp * h->n_in * 4);
        cudaMemcpy(h->xin, x + (size_t)s0 * h->n_in, (size_t)M * h->n_in * 4, cudaMemcpyHostToDevice);
        forward(h, Mp, nullptr);
        if (cudaMemcpy(zb.data(), h->Z[L - 1], (size_t)M * ldo * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return sl_record_error(SL_ERR_CUDA, "prediction failed");
        if (int r = mlp_status(h, "sl_mlp_predict")) return r;
        for (int r = 0; r < M; ++r)
            for (int c = 0; c < h->n_out; ++c) y[(size_t)(s0 + r) * h->n_out + c] = zb[(size_t)r * ldo + c];
    }
    return SL_OK;
}

}  // extern "C"

extern "C" int sl_diag_gemm_bf16(int M, int N, int K, const uint16_t* A, const uint16_t* B, const float* bias,
                                 int act, int kernel, float* C, uint16_t* Cb)
{
    if (M < 1 || N < 1 || K < 1 || K % 8 || !A || !B || !C || (kernel != 0 && kernel != 1))
        return sl_record_error(SL_ERR_ARG, "sl_diag_gemm_bf16: need M, N >= 1, K a multiple of 8, kernel 0 or 1");
    if (kernel == 0 && K % kTK)
        return sl_record_error(SL_ERR_ARG, "sl_diag_gemm_bf16: the mma.sync kernel needs K a multiple of 32");
    const size_t na = (size_t)M * K, nbb = (size_t)N * K, nc = (size_t)M * N;
    size_t off = 0;
    auto take = [&](size_t b) { size_t o = off; off = (off + b + 255) / 256 * 256; return o; };
    const size_t oA = take(na * 2), oB = take(nbb * 2), oBias = take((size_t)N * 4), oC = take(nc * 4),
                 oCb = take(nc * 2), oErr = take(sizeof(int));
    void* arena = nullptr;
    if (cudaMalloc(&arena, off) != cudaSuccess) return sl_record_error(SL_ERR_ALLOC, "sl_diag_gemm_bf16: cudaMalloc");
    char* b = static_cast<char*>(arena);
    bf16* dA = (bf16*)(b + oA);
    bf16* dB = (bf16*)(b + oB);
    float* dBias = bias ? (float*)(b + oBias) : nullptr;
    float* dC = (float*)(b + oC);
    bf16* dCb = Cb ? (bf16*)(b + oCb) : nullptr;
    int* dErr = (int*)(b + oErr);
    int rc = SL_OK;
    cudaMemcpy(dA, A, na * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, nbb * 2, cudaMemcpyHostToDevice);
    if (bias) cudaMemcpy(dBias, bias, (size_t)N * 4, cudaMemcpyHostToDevice);
    cudaMemset(dErr, 0, sizeof(int));
    if (kernel == 0) {
        gemm_mma_sync(nullptr, dA, K, dB, K, dBias, dC, dCb, N, M, N, K, act);
    } else if (!gemm_tc(nullptr, dA, K, dB, K, dBias, dC, dCb, N, M, N, K, act, dErr)) {
        rc = sl_record_error(SL_ERR_CUDA, "sl_diag_gemm_bf16: tensor map or launch setup failed");
    }
    if (rc == SL_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) rc = sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
    }
    int herr = 0;
    if (rc == SL_OK) {
        cudaMemcpy(&herr, dErr, sizeof(int), cudaMemcpyDeviceToHost);
        if (herr) rc = sl_record_error(SL_ERR_TIMEOUT, "sl_diag_gemm_bf16: a bounded wait in the tcgen05 GEMM ran out");
    }
    if (rc == SL_OK) {
        cudaMemcpy(C, dC, nc * 4, cudaMemcpyDeviceToHost);
        if (Cb) cudaMemcpy(Cb, dCb, nc * 2, cudaMemcpyDeviceToHost);
    }
    cudaFree(arena);
    return rc;
}

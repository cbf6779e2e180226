// sl_static.cu -- the force pass on caller-owned device buffers, with all of
// its working memory in one file-scope device array (sl_forces_static in
// include/spacelab_gpu.h).  It allocates nothing: no cudaMalloc, cudaFree,
// pinned host memory, stream or event is created here.
//
// The working memory is the same set of arrays a handle holds (structure-of-
// arrays state, per-sphere constants, pair and torque term buffers, contact
// masks, reduction partials), laid out for at most kStaticMaxSpheres spheres,
// and the kernels are the step kernels of sl_step.cu, launched through their
// existing launchers with a System that points into the array.
#include "../../include/spacelab_gpu.h"
#include "sl_device.cuh"
#include "sl_kernels.h"

#include <cuda.h>  // CUcontext, for the driver entry points below

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

int sl_record_error(int code, const char* msg);

namespace {

constexpr int kStaticMaxSpheres = SL_STATIC_MAX_SPHERES;
static_assert(kStaticMaxSpheres % sl::kBlock == 0, "static capacity must be whole 32-sphere blocks");
constexpr int kNp = kStaticMaxSpheres;
constexpr int kNb = kNp / sl::kBlock;
constexpr long long kTiles = (long long)kNb * (kNb + 1) / 2;

// offsets in doubles, each rounded up to 32 doubles (256 bytes)
constexpr size_t up32(size_t x) { return (x + 31) / 32 * 32; }
constexpr size_t kVec = up32(kNp);                       // one SoA row
constexpr size_t kOffVec = 0;                            // 8 vec3 x 3 rows
constexpr size_t kOffScal = kOffVec + 24 * kVec;         // 8 per-sphere scalars
constexpr size_t kOffPair = kOffScal + 8 * kVec;
constexpr size_t kOffTorq = kOffPair + up32(3ull * kNp * kNp);
constexpr size_t kOffMask = kOffTorq + up32(3ull * kNp * kNp);
constexpr size_t kOffPe = kOffMask + up32((size_t)kNp * kNb / 2 + 1);
constexpr size_t kOffRed = kOffPe + up32(kTiles);
constexpr size_t kOffEnergy = kOffRed + up32(sl::kRedBlocks * 8);
constexpr size_t kOffStatus = kOffEnergy + 32;
constexpr size_t kOffScalars = kOffStatus + 32;
constexpr size_t kScratchDoubles = kOffScalars + 32;

// The working memory.  Every GPU that loads the library holds it (about
// 3.2 MB for 256 spheres) until the process exits.
__device__ __align__(256) double g_static_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
// A real sphere's R, m or moi is not finite and > 0 (set by the load kernel).
constexpr unsigned kStatusBadInputBit = 0x80000000u;

struct DeviceSlot {
    double* scratch = nullptr;
    int num_sms = 0;
    unsigned long long ctx_id = 0;  // context the address belongs to (0 = none yet)
};
std::mutex g_mutex;
DeviceSlot g_slots[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the context current on this thread (0 if none is current or
// the driver does not offer the query).  Ids are never reused within a
// process, so a context rebuilt by cudaDeviceReset gets a new one.
unsigned long long current_context_id()
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
        fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(fn);
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_static_scratch in the current device's current
// context.  It is looked up (cudaGetSymbolAddress) once per device and
// looked up again whenever the current context is not the one the cached
// address came from: after cudaDeviceReset the primary context and its copy
// of the array are rebuilt, and a driver-API context of its own holds
// another copy.  Host code may not use the symbol itself as a pointer: on
// the host it names a stand-in object, not device memory.
int scratch_for_current_device(double** base, int* num_sms)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return sl_record_error(SL_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    DeviceSlot& slot = g_slots[dev];
    const unsigned long long ctx = current_context_id();
    if (!slot.scratch || ctx == 0 || ctx != slot.ctx_id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return sl_record_error(SL_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
        slot.scratch = static_cast<double*>(p);
        slot.num_sms = sms;
        // the lookup made the runtime's context current if none was
        slot.ctx_id = ctx ? ctx : current_context_id();
    }
    *base = slot.scratch;
    *num_sms = slot.num_sms;
    return SL_OK;
}

sl::System static_system(double* base, int n, const sl_material& mat)
{
    sl::System s{};
    s.n = n;
    s.npad = (n + sl::kBlock - 1) / sl::kBlock * sl::kBlock;
    s.nb = s.npad / sl::kBlock;
    s.ntiles = (long long)s.nb * (s.nb + 1) / 2;
    s.nitems = s.ntiles;
    // pairbuf/torqbuf rows are s.npad long; they fit the kNp x kNp capacity
    sl::Vec3Soa* vecs[8] = {&s.pos, &s.prev, &s.vel, &s.velh, &s.w, &s.wh, &s.acc, &s.aacc};
    for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 3; ++c) vecs[v]->c[c] = base + kOffVec + (size_t)(3 * v + c) * kVec;
    double* inv_m_slot = nullptr;  // 8 bytes per sphere, holds the mass reciprocals rm
    double** scal[8] = {&s.R, &s.m, &s.moi, &s.twoR, &s.fourR, &s.cR3, &inv_m_slot, &s.inv_moi};
    for (int k = 0; k < 8; ++k) *scal[k] = base + kOffScal + (size_t)k * kVec;
    s.rm = reinterpret_cast<unsigned long long*>(inv_m_slot);
    s.pairbuf = base + kOffPair;
    s.torqbuf = base + kOffTorq;
    s.cmask = reinterpret_cast<uint32_t*>(base + kOffMask);
    s.pe_tile = base + kOffPe;
    s.red = base + kOffRed;
    s.energy = base + kOffEnergy;
    s.status = reinterpret_cast<unsigned int*>(base + kOffStatus);
    s.sc = reinterpret_cast<const sl::Scalars*>(base + kOffScalars);
    s.mat = sl::Material{mat.G, mat.Ha, mat.u_s, mat.u_r, mat.h_min};
    return s;
}

// Caller's vec3[n] device arrays -> the scratch's SoA rows; R/m/moi with
// padding 1; acc/aacc cleared (the scratch keeps the previous call's
// contents; the error word is cleared before this kernel runs); scalars
// dt = 0 (a force pass), kin, kout.
// A real sphere whose R, m or moi is not finite and > 0 sets
// kStatusBadInputBit, as sl_upload rejects such values on the handle path.
__global__ void static_load_kernel(const __grid_constant__ sl::System s, const double* pos, const double* vel,
                                   const double* w, const double* R, const double* m, const double* moi,
                                   double kin, double kout)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        sl::Scalars* sc = const_cast<sl::Scalars*>(s.sc);
        sc->dt = 0.0;
        sc->kin = kin;
        sc->kout = kout;
    }
    if (i >= s.npad) return;
    const bool real = i < s.n;
    for (int c = 0; c < 3; ++c) {
        s.pos.c[c][i] = real ? pos[3 * (size_t)i + c] : 0.0;
        s.vel.c[c][i] = real ? vel[3 * (size_t)i + c] : 0.0;
        s.w.c[c][i] = real ? w[3 * (size_t)i + c] : 0.0;
        s.acc.c[c][i] = 0.0;
        s.aacc.c[c][i] = 0.0;
    }
    double r = real ? R[i] : 1.0, mi = real ? m[i] : 1.0, mo = real ? moi[i] : 1.0;
    // written so that NaN fails too; a rejected sphere is given 1.0 so that
    // the rest of the pass runs on ordinary numbers before the call fails
    if (!(r > 0.0 && r < INFINITY) || !(mi > 0.0 && mi < INFINITY) || !(mo > 0.0 && mo < INFINITY)) {
        atomicOr(s.status, kStatusBadInputBit);
        r = mi = mo = 1.0;
    }
    s.R[i] = r;
    s.m[i] = mi;
    s.moi[i] = mo;
}

__global__ void static_store_kernel(const __grid_constant__ sl::System s, double* acc, double* aacc,
                                    double* energy)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (energy && i < 8) energy[i] = s.energy[i];
    if (i >= s.n) return;
    for (int c = 0; c < 3; ++c) {
        acc[3 * (size_t)i + c] = s.acc.c[c][i];
        aacc[3 * (size_t)i + c] = s.aacc.c[c][i];
    }
}

}  // namespace

extern "C" int sl_forces_static(int n, const double* pos, const double* vel, const double* w, const double* R,
                                const double* m, const double* moi, const sl_material* mat, double kin,
                                double kout, double* acc, double* aacc, double* energy, void* stream)
{
    if (n < 1 || n > kStaticMaxSpheres)
        return sl_record_error(SL_ERR_ARG, ("sl_forces_static: n = " + std::to_string(n) +
                                            " is outside 1.." + std::to_string(kStaticMaxSpheres) +
                                            " (the capacity of its static working memory)").c_str());
    if (!pos || !vel || !w || !R || !m || !moi || !acc || !aacc || !mat)
        return sl_record_error(SL_ERR_ARG, "sl_forces_static: NULL input or output pointer");
    if (!(mat->h_min > 0) || !std::isfinite(kin) || !std::isfinite(kout) || kin < 0 || kout < 0)
        return sl_record_error(SL_ERR_ARG, "sl_forces_static: need h_min > 0 and finite kin, kout >= 0");
    double* base = nullptr;
    int num_sms = 0;
    if (int rc = scratch_for_current_device(&base, &num_sms)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const sl::System s = static_system(base, n, *mat);
    const int threads = 128;
    cudaError_t e = cudaMemsetAsync(s.status, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
    static_load_kernel<<<(s.npad + threads - 1) / threads, threads, 0, st>>>(s, pos, vel, w, R, m, moi, kin, kout);
    sl::launch_derive(s, st);
    sl::launch_step(s, true, num_sms, st, nullptr);
    static_store_kernel<<<(s.npad + threads - 1) / threads, threads, 0, st>>>(s, acc, aacc, energy);
    e = cudaGetLastError();
    if (e != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
    unsigned int status = 0;
    e = cudaMemcpyAsync(&status, s.status, sizeof(status), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
    if (status & kStatusBadInputBit)
        return sl_record_error(SL_ERR_ARG, "sl_forces_static: a radius, mass or moment of inertia is not finite and > 0");
    if (status & sl::kStatusWaitTimeoutBit)
        return sl_record_error(SL_ERR_TIMEOUT, "sl_forces_static: a bounded wait for asynchronous copies ran out");
    if (status) return sl_record_error(SL_ERR_NONFINITE, "sl_forces_static: non-finite forces or state");
    return SL_OK;
}

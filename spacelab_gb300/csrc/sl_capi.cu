// sl_capi.cu -- the extern "C" handle API of include/spacelab_gpu.h.
//
// A handle owns one device arena holding the structure-of-arrays state of
// one system, the per-pair scratch (pairbuf/torqbuf/cmask; the mixed form's
// per-tile partials instead of pairbuf) and the energy reduction buffers,
// plus a CUDA stream and, for sl_run, an instantiated CUDA graph of one write
// interval.  A kernel transposes the caller's vec3[n] (AoS) arrays to or from
// the SoA state, reading and writing them in place where the GPU can reach
// them, otherwise through a device staging area and one copy per array.
#include "../../include/spacelab_gpu.h"
#include "sl_device.cuh"
#include "sl_kernels.h"
#include "sl_pair_mixed.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace {

thread_local std::string g_last_error = "";

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
    return fail(SL_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SL_CUDA(call)                                  \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr int kTimerPool = 8192;

}  // namespace

// Records `msg` as this thread's sl_last_error() text; used by entry points
// in other translation units of the library.
int sl_record_error(int code, const char* msg)
{
    return fail(code, msg ? std::string(msg) : std::string());
}

struct sl_handle {
    sl::System sys{};
    sl::Scalars host_sc{0, 0, 0};
    sl::Scalars* d_sc = nullptr;
    int mode = SL_MODE_EXACT;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // exact mode: side stream + events overlapping row sums with pair phases
    sl::StepOverlap ov{};
    CUtensorMap pair_map{};  // exact form: the pair-term buffer for the TMA row sums
    bool has_map = false;     // the TMA row sums are ready (exact form)
    bool has_ov = false;   // ov's stream and events exist
    bool overlap = false;  // steps use them
    bool rowsum_int = false;  // exact row sums: FP64 additions on the integer pipe (else the FP64 unit)
    void* arena = nullptr;
    size_t arena_bytes = 0;
    double* staging = nullptr;  // pinned, 18 * npad doubles (per-sphere scalars at upload)
    double* d_stage = nullptr;  // device, 6 x 3 npad doubles: AoS copies of the vec3 arrays
    double* h_energy = nullptr; // pinned, 8 doubles
    unsigned int* h_status = nullptr;
    bool uploaded = false;
    bool forces_ready = false;
    // the GPU reads and writes pageable host memory directly (cudaDevAttr-
    // PageableMemoryAccess: coherent CPU-GPU systems such as Grace-Blackwell)
    bool host_direct = false;
    // graph of one write interval for sl_run
    cudaGraphExec_t interval_exec = nullptr;
    int interval_skip = 0;
    // kernel timing
    bool timing = false;
    std::vector<sl::StepTimers> timers;
    int timers_used = 0;
    double pair_ms = 0, rowsum_ms = 0;
    long launches = 0;
};

namespace {

int check_handle(const sl_handle* h)
{
    if (!h) return fail(SL_ERR_ARG, "null handle");
    return SL_OK;
}

void launch_mode_step(sl_handle* h, bool write, sl::StepTimers* tm)
{
    if (h->mode == SL_MODE_MIXED)
        sl::launch_step_mixed64(h->sys, write, h->num_sms, h->stream, tm);
    else if (h->mode == SL_MODE_MIXED_DF)
        sl::launch_step_mixed(h->sys, write, h->num_sms, h->stream, tm);
    else
        sl::launch_step(h->sys, write, h->num_sms, h->stream, tm, h->overlap ? &h->ov : nullptr,
                        h->has_map ? &h->pair_map : nullptr, h->rowsum_int);
}

// One step on the handle's stream, with optional timing events.
int enqueue_step(sl_handle* h, bool write)
{
    sl::StepTimers* tm = nullptr;
    if (h->timing) {
        if (h->timers_used >= (int)h->timers.size()) {
            sl::StepTimers t;
            for (int k = 0; k < 3; ++k) SL_CUDA(cudaEventCreate(&t.ev[k]));
            if ((int)h->timers.size() >= kTimerPool) return fail(SL_ERR_STATE, "timer pool exhausted; read sl_kernel_times");
            h->timers.push_back(t);
        }
        tm = &h->timers[h->timers_used++];
    }
    launch_mode_step(h, write, tm);
    SL_CUDA(cudaGetLastError());
    return SL_OK;
}

int fetch_energy_and_status(sl_handle* h, sl_energy* out, bool want_energy)
{
    if (want_energy)
        SL_CUDA(cudaMemcpyAsync(h->h_energy, h->sys.energy, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SL_CUDA(cudaMemcpyAsync(h->h_status, h->sys.status, sizeof(unsigned int), cudaMemcpyDeviceToHost, h->stream));
    SL_CUDA(cudaStreamSynchronize(h->stream));
    if (want_energy && out) {
        out->PE = h->h_energy[0];
        out->KE = h->h_energy[1];
        for (int k = 0; k < 3; ++k) {
            out->mom[k] = h->h_energy[2 + k];
            out->ang_mom[k] = h->h_energy[5 + k];
        }
    }
    if (*h->h_status & sl::kStatusInputNonFiniteBit)
        return fail(SL_ERR_ARG, "non-finite position, velocity or spin in input");
    if (*h->h_status & sl::kStatusWaitTimeoutBit)
        return fail(SL_ERR_TIMEOUT, "a row-sum kernel's bounded wait for its TMA copies ran out");
    if (*h->h_status) return fail(SL_ERR_NONFINITE, "state became non-finite (NaN/Inf position, velocity or spin)");
    return SL_OK;
}

// True if no element is Inf or NaN (exponent field all ones); a branch-free
// loop over the bit patterns, which the compiler vectorises.
bool all_finite(const double* a, size_t count)
{
    const uint64_t* u = reinterpret_cast<const uint64_t*>(a);
    uint64_t bad = 0;
    for (size_t i = 0; i < count; ++i) bad |= ((u[i] & 0x7ff0000000000000ull) == 0x7ff0000000000000ull) ? 1u : 0u;
    return bad == 0;
}

// A device-accessible view of the caller's array p, or NULL where the GPU
// cannot reach it (plain pageable memory without pageable access): then the
// exchange goes through the device staging buffer and a copy.
const double* device_view(const sl_handle* h, const double* p)
{
    if (h->host_direct) return p;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clear the failed lookup's error
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return static_cast<const double*>(a.devicePointer);
    return nullptr;
}

// The six vec3 arrays a handle exchanges with its caller, in staging order.
void stage_arrays(sl_handle* h, sl::Vec3Soa* out[6])
{
    sl::System& s = h->sys;
    sl::Vec3Soa* a[6] = {&s.pos, &s.vel, &s.w, &s.acc, &s.aacc, &s.prev};
    for (int k = 0; k < 6; ++k) out[k] = a[k];
}

void drop_graph(sl_handle* h)
{
    if (h->interval_exec) cudaGraphExecDestroy(h->interval_exec);
    h->interval_exec = nullptr;
    h->interval_skip = 0;
}

}  // namespace

extern "C" {

int sl_version(void) { return SL_API_VERSION; }

const char* sl_last_error(void) { return g_last_error.c_str(); }

int sl_create(int n, const sl_material* mat, int mode, sl_handle** out)
{
    if (!out) return fail(SL_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (n < 1) return fail(SL_ERR_ARG, "n must be >= 1");
    if (n > 46340) return fail(SL_ERR_ARG, "n > 46340 exceeds the reference's pair index range");
    if (!mat) return fail(SL_ERR_ARG, "material is NULL");
    if (mode != SL_MODE_EXACT && mode != SL_MODE_MIXED && mode != SL_MODE_MIXED_DF)
        return fail(SL_ERR_UNSUPPORTED, "unknown mode");
    if (!(mat->h_min > 0)) return fail(SL_ERR_ARG, "h_min must be > 0");

    sl_handle* h = new (std::nothrow) sl_handle();
    if (!h) return fail(SL_ERR_ALLOC, "host allocation failed");
    h->mode = mode;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaGetDevice"); }
    e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaDeviceGetAttribute"); }
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, h->device) == cudaSuccess)
        h->host_direct = pageable != 0;
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaStreamCreate"); }
    if (mode == SL_MODE_EXACT) {
        h->has_ov = true;  // destroy releases whatever was created
        e = cudaStreamCreateWithFlags(&h->ov.side, cudaStreamNonBlocking);
        for (int p = 0; p < sl::kPairPhases && e == cudaSuccess; ++p)
            e = cudaEventCreateWithFlags(&h->ov.phase[p], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ov.join, cudaEventDisableTiming);
        if (e != cudaSuccess) { sl_destroy(h); return cuda_fail(e, "side stream / event creation"); }
    }

    sl::System& s = h->sys;
    s.n = n;
    s.npad = (n + sl::kBlock - 1) / sl::kBlock * sl::kBlock;
    s.nb = s.npad / sl::kBlock;
    s.ntiles = (long long)s.nb * (s.nb + 1) / 2;
    s.pair_double = mode == SL_MODE_MIXED_DF && sl::mixed_pair_double(s.nb, h->num_sms);
    s.nitems = s.pair_double ? sl::mixed_pair_items(s.nb) : s.ntiles;
    s.mat = sl::Material{mat->G, mat->Ha, mat->u_s, mat->u_r, mat->h_min};
    const size_t np = s.npad;
    const size_t A = 256;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, A); return o; };
    size_t o_vec[8][3];
    for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 3; ++c) o_vec[v][c] = take(np * sizeof(double));
    size_t o_sc[8];
    for (int k = 0; k < 8; ++k) o_sc[k] = take(np * sizeof(double));
    // FP32 per-sphere constants (both mixed forms) and the double-float
    // positions (SL_MODE_MIXED_DF only)
    const bool mixed = mode != SL_MODE_EXACT;
    const bool mixed_df = mode == SL_MODE_MIXED_DF;
    size_t o_f[10] = {};
    for (int k = 0; k < 10; ++k) o_f[k] = take(mixed && (k < 4 || mixed_df) ? np * sizeof(float) : 0);
    // the mixed forms keep per-tile partial sums instead of pair terms (FP64
    // in SL_MODE_MIXED, FP32 in SL_MODE_MIXED_DF), and torque terms in the
    // same type
    const size_t part_elem = mixed_df ? sizeof(float) : sizeof(double);
    const size_t o_pair = take(mixed ? 3 * (size_t)s.nb * np * part_elem : 3 * np * np * sizeof(double));
    const size_t o_torq = take(3 * np * np * (mixed_df ? sizeof(float) : sizeof(double)));
    const size_t o_mask = take(np * s.nb * sizeof(uint32_t));
    const size_t o_pe = take((size_t)s.nitems * sizeof(double));
    const size_t o_red = take(sl::kRedBlocks * 8 * sizeof(double));
    const size_t o_en = take(8 * sizeof(double));
    const size_t o_st = take(sizeof(unsigned int));
    const size_t o_tc = take(sl::kPairPhases * sizeof(int));  // the pair kernels' work queues
    const size_t o_cf = take(mixed ? np * sizeof(int) : 0);
    const size_t o_scl = take(sizeof(sl::Scalars));
    const size_t o_dstage = take(6 * 3 * np * sizeof(double));
    h->arena_bytes = off;
    e = cudaMalloc(&h->arena, h->arena_bytes);
    if (e != cudaSuccess) { sl_destroy(h); return fail(SL_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e)); }
    char* base = static_cast<char*>(h->arena);
    sl::Vec3Soa* vecs[8] = {&s.pos, &s.prev, &s.vel, &s.velh, &s.w, &s.wh, &s.acc, &s.aacc};
    for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 3; ++c) vecs[v]->c[c] = reinterpret_cast<double*>(base + o_vec[v][c]);
    double* inv_m_slot = nullptr;  // 8 bytes per sphere, holds the mass reciprocals rm
    double** scal[8] = {&s.R, &s.m, &s.moi, &s.twoR, &s.fourR, &s.cR3, &inv_m_slot, &s.inv_moi};
    for (int k = 0; k < 8; ++k) *scal[k] = reinterpret_cast<double*>(base + o_sc[k]);
    s.rm = reinterpret_cast<unsigned long long*>(inv_m_slot);
    if (mixed) {
        s.f_R = reinterpret_cast<float*>(base + o_f[0]);
        s.f_inv_m = reinterpret_cast<float*>(base + o_f[1]);
        s.f_inv_moi = reinterpret_cast<float*>(base + o_f[2]);
        s.f_Rlo = reinterpret_cast<float*>(base + o_f[3]);
    }
    if (mixed_df)
        for (int k = 0; k < 6; ++k) s.f_pos[k] = reinterpret_cast<float*>(base + o_f[4 + k]);
    if (mixed_df)
        s.f_part = reinterpret_cast<float*>(base + o_pair);
    else if (mixed)
        s.part64 = reinterpret_cast<double*>(base + o_pair);
    else
        s.pairbuf = reinterpret_cast<double*>(base + o_pair);
    s.torqbuf = reinterpret_cast<double*>(base + o_torq);
    s.cmask = reinterpret_cast<uint32_t*>(base + o_mask);
    s.pe_tile = reinterpret_cast<double*>(base + o_pe);
    s.red = reinterpret_cast<double*>(base + o_red);
    s.energy = reinterpret_cast<double*>(base + o_en);
    s.status = reinterpret_cast<unsigned int*>(base + o_st);
    s.tile_counter = reinterpret_cast<int*>(base + o_tc);
    if (mixed) s.contact_flag = reinterpret_cast<int*>(base + o_cf);
    h->d_sc = reinterpret_cast<sl::Scalars*>(base + o_scl);
    h->d_stage = reinterpret_cast<double*>(base + o_dstage);
    s.sc = h->d_sc;
    h->has_map = !mixed && sl::make_pair_map(s, &h->pair_map);
    e = cudaMemsetAsync(h->arena, 0, h->arena_bytes, h->stream);
    if (e != cudaSuccess) { sl_destroy(h); return cuda_fail(e, "cudaMemset"); }
    e = cudaMallocHost(&h->staging, 18 * np * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_energy, 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_status, sizeof(unsigned int));
    if (e != cudaSuccess) { sl_destroy(h); return fail(SL_ERR_ALLOC, "pinned host allocation failed"); }
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) { sl_destroy(h); return cuda_fail(e, "cudaStreamSynchronize"); }
    *out = h;
    return SL_OK;
}

int sl_destroy(sl_handle* h)
{
    if (!h) return SL_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graph(h);
    for (auto& t : h->timers)
        for (int k = 0; k < 3; ++k) cudaEventDestroy(t.ev[k]);
    if (h->arena) cudaFree(h->arena);
    if (h->staging) cudaFreeHost(h->staging);
    if (h->h_energy) cudaFreeHost(h->h_energy);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->has_ov) {
        if (h->ov.side) cudaStreamDestroy(h->ov.side);
        for (int p = 0; p < sl::kPairPhases; ++p)
            if (h->ov.phase[p]) cudaEventDestroy(h->ov.phase[p]);
        if (h->ov.join) cudaEventDestroy(h->ov.join);
    }
    delete h;
    return SL_OK;
}

int sl_num_particles(const sl_handle* h, int* n)
{
    if (int r = check_handle(h)) return r;
    if (!n) return fail(SL_ERR_ARG, "n is NULL");
    *n = h->sys.n;
    return SL_OK;
}

int sl_upload(sl_handle* h, const double* pos, const double* vel, const double* w, const double* R,
              const double* m, const double* moi)
{
    if (int r = check_handle(h)) return r;
    if (!R || !m || !moi) return fail(SL_ERR_ARG, "R, m or moi is NULL");
    const int n = h->sys.n, np = h->sys.npad;
    for (int i = 0; i < n; ++i) {
        if (!(R[i] > 0) || !(m[i] > 0) || !(moi[i] > 0) || !std::isfinite(R[i]) || !std::isfinite(m[i]) ||
            !std::isfinite(moi[i]))
            return fail(SL_ERR_ARG, "R, m and moi must be finite and > 0 (sphere " + std::to_string(i) + ")");
    }
    if (int r = sl_upload_resume(h, pos, vel, w, nullptr, nullptr, nullptr)) return r;
    // length scale of the mixed form: 2^len_shift within a factor 2 of max R
    double rmax = 0, rmin = R[0];
    for (int i = 0; i < n; ++i) {
        rmax = R[i] > rmax ? R[i] : rmax;
        rmin = R[i] < rmin ? R[i] : rmin;
    }
    int ex = 0;
    std::frexp(rmax, &ex);
    h->sys.len_shift = ex - 1;
    h->sys.far_sq = sl::far_threshold_sq(h->sys.mat.h_min, rmin);
    // padded spheres get R = m = moi = 1 (they are never paired)
    const double* src[3] = {R, m, moi};
    double* dst[3] = {h->sys.R, h->sys.m, h->sys.moi};
    for (int k = 0; k < 3; ++k) {
        double* row = h->staging + (size_t)k * np;
        for (int i = 0; i < n; ++i) row[i] = src[k][i];
        for (int i = n; i < np; ++i) row[i] = 1.0;
        SL_CUDA(cudaMemcpyAsync(dst[k], row, np * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    }
    sl::launch_derive(h->sys, h->stream);
    SL_CUDA(cudaGetLastError());
    SL_CUDA(cudaStreamSynchronize(h->stream));
    h->uploaded = true;
    h->forces_ready = false;
    return SL_OK;
}

namespace {

// The exchange of sl_upload_resume, enqueued on the handle's stream without
// waiting: the status word cleared, then the staging kernel (reading each
// array in place where the GPU can reach it, else through a copy).  The
// finite check of pos, vel and w runs on the host before anything is
// enqueued, or, with device_check, in the staging kernel itself
// (kStatusInputNonFiniteBit, read by the caller after its wait).
int enqueue_resume(sl_handle* h, const double* pos, const double* vel, const double* w, const double* acc,
                   const double* aacc, const double* pos_prev, bool device_check)
{
    if (!pos || !vel || !w) return fail(SL_ERR_ARG, "pos, vel or w is NULL");
    const int n = h->sys.n;
    if (!device_check &&
        (!all_finite(pos, 3 * (size_t)n) || !all_finite(vel, 3 * (size_t)n) || !all_finite(w, 3 * (size_t)n)))
        return fail(SL_ERR_ARG, "non-finite position, velocity or spin in input");
    SL_CUDA(cudaMemsetAsync(h->sys.status, 0, sizeof(unsigned int), h->stream));
    const size_t np = h->sys.npad;
    // the staging kernel reads each array where the GPU can reach it, else
    // from a copy in the device staging area; absent acc/aacc are zero, an
    // absent previous position is the position
    const double* srcs[6] = {pos, vel, w, acc, aacc, pos_prev};
    const double* views[6] = {};
    unsigned present = 0;
    for (int k = 0; k < 6; ++k)
        if (srcs[k]) {
            views[k] = device_view(h, srcs[k]);
            if (!views[k]) {
                double* stage = h->d_stage + (size_t)k * 3 * np;
                SL_CUDA(cudaMemcpyAsync(stage, srcs[k], 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                                        h->stream));
                views[k] = stage;
            }
            present |= 1u << k;
        }
    sl::Vec3Soa* dst[6];
    stage_arrays(h, dst);
    sl::launch_stage_in(h->sys, views, dst, present, h->stream, device_check ? 7u : 0u);
    SL_CUDA(cudaGetLastError());
    return SL_OK;
}

// The exchange of sl_download, enqueued without waiting.  outs[k] that the
// GPU cannot reach are written through the staging area and a copy, which
// the caller's stream synchronisation completes.  guard (only where the GPU
// reaches every array, so that nothing goes through a copy): nothing is
// written once the staging kernel found a non-finite input.
int enqueue_download(sl_handle* h, double* pos, double* vel, double* w, double* acc, double* aacc,
                     bool guard = false)
{
    double* outs[5] = {pos, vel, w, acc, aacc};
    const size_t np = h->sys.npad;
    const int n = h->sys.n;
    unsigned want = 0;
    for (int k = 0; k < 5; ++k)
        if (outs[k]) want |= 1u << k;
    sl::Vec3Soa* src[6];
    stage_arrays(h, src);
    double* views[6] = {};
    bool staged[5] = {};
    for (int k = 0; k < 5; ++k)
        if (outs[k]) {
            views[k] = const_cast<double*>(device_view(h, outs[k]));
            if (!views[k]) {
                views[k] = h->d_stage + (size_t)k * 3 * np;
                staged[k] = true;
            }
        }
    sl::launch_stage_out(h->sys, views, src, want, h->stream, guard);
    SL_CUDA(cudaGetLastError());
    for (int k = 0; k < 5; ++k)
        if (staged[k])
            SL_CUDA(cudaMemcpyAsync(outs[k], views[k], 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                                    h->stream));
    return SL_OK;
}

}  // namespace

int sl_upload_resume(sl_handle* h, const double* pos, const double* vel, const double* w, const double* acc,
                     const double* aacc, const double* pos_prev)
{
    if (int r = check_handle(h)) return r;
    if (int r = enqueue_resume(h, pos, vel, w, acc, aacc, pos_prev, false)) return r;
    SL_CUDA(cudaStreamSynchronize(h->stream));
    h->forces_ready = (acc != nullptr && aacc != nullptr);
    return SL_OK;
}

int sl_set_scalars(sl_handle* h, double dt, double kin, double kout)
{
    if (int r = check_handle(h)) return r;
    if (!std::isfinite(dt) || !std::isfinite(kin) || !std::isfinite(kout) || dt < 0 || kin < 0 || kout < 0)
        return fail(SL_ERR_ARG, "dt, kin, kout must be finite and >= 0");
    h->host_sc = sl::Scalars{dt, kin, kout};
    SL_CUDA(cudaMemcpyAsync(h->d_sc, &h->host_sc, sizeof(sl::Scalars), cudaMemcpyHostToDevice, h->stream));
    SL_CUDA(cudaStreamSynchronize(h->stream));
    return SL_OK;
}

int sl_init_forces(sl_handle* h, sl_energy* out)
{
    if (int r = check_handle(h)) return r;
    if (!h->uploaded) return fail(SL_ERR_STATE, "sl_upload first");
    // A step with dt = 0 leaves pos/vel/w unchanged, sets prev = pos and
    // evaluates the pair terms of init_conditions, with the energy totals.
    const sl::Scalars zero{0.0, h->host_sc.kin, h->host_sc.kout};
    SL_CUDA(cudaMemcpyAsync(h->d_sc, &zero, sizeof(sl::Scalars), cudaMemcpyHostToDevice, h->stream));
    for (int c = 0; c < 3; ++c) {
        SL_CUDA(cudaMemsetAsync(h->sys.acc.c[c], 0, h->sys.npad * sizeof(double), h->stream));
        SL_CUDA(cudaMemsetAsync(h->sys.aacc.c[c], 0, h->sys.npad * sizeof(double), h->stream));
    }
    if (int r = enqueue_step(h, true)) return r;
    SL_CUDA(cudaMemcpyAsync(h->d_sc, &h->host_sc, sizeof(sl::Scalars), cudaMemcpyHostToDevice, h->stream));
    const int r = fetch_energy_and_status(h, out, true);
    h->forces_ready = (r == SL_OK);
    return r;
}

int sl_step(sl_handle* h, int nsteps, int write_last, sl_energy* out)
{
    if (int r = check_handle(h)) return r;
    if (!h->uploaded) return fail(SL_ERR_STATE, "sl_upload first");
    if (nsteps < 0) return fail(SL_ERR_ARG, "nsteps < 0");
    for (int k = 0; k < nsteps; ++k)
        if (int r = enqueue_step(h, write_last && k == nsteps - 1)) return r;
    return fetch_energy_and_status(h, out, write_last && nsteps > 0);
}

int sl_run(sl_handle* h, int first_step, int last_step, int skip, sl_energy* rows, int max_rows, int* nrows)
{
    if (int r = check_handle(h)) return r;
    if (!h->uploaded) return fail(SL_ERR_STATE, "sl_upload first");
    if (skip < 1) return fail(SL_ERR_ARG, "skip must be >= 1 (ColliderSingleCore.cpp:402-405)");
    if (first_step < 1 || last_step < first_step) return fail(SL_ERR_ARG, "need 1 <= first_step <= last_step");
    if (nrows) *nrows = 0;
    int written = 0;
    int step = first_step;
    const bool use_graph = !h->timing;
    while (step < last_step) {
        if (use_graph && skip > 1 && (step - 1) % skip == 0 && step + skip - 1 < last_step) {
            // a whole interval: skip-1 plain steps then one write step
            if (h->interval_skip != skip) {
                drop_graph(h);
                cudaGraph_t g;
                SL_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
                for (int k = 0; k < skip; ++k) launch_mode_step(h, k == skip - 1, nullptr);
                SL_CUDA(cudaStreamEndCapture(h->stream, &g));
                const cudaError_t e = cudaGraphInstantiate(&h->interval_exec, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
                h->interval_skip = skip;
            }
            SL_CUDA(cudaGraphLaunch(h->interval_exec, h->stream));
            step += skip;
            const int r = fetch_energy_and_status(h, written < max_rows && rows ? &rows[written] : nullptr, true);
            if (r) { if (nrows) *nrows = written; return r; }
            if (written < max_rows) ++written;
        } else {
            const bool write = (step % skip == 0);
            if (int r = enqueue_step(h, write)) return r;
            if (write) {
                const int r = fetch_energy_and_status(h, written < max_rows && rows ? &rows[written] : nullptr, true);
                if (r) { if (nrows) *nrows = written; return r; }
                if (written < max_rows) ++written;
            }
            ++step;
        }
    }
    if (nrows) *nrows = written;
    return fetch_energy_and_status(h, nullptr, false);
}

int sl_download(sl_handle* h, double* pos, double* vel, double* w, double* acc, double* aacc)
{
    if (int r = check_handle(h)) return r;
    if (int r = enqueue_download(h, pos, vel, w, acc, aacc)) return r;
    SL_CUDA(cudaStreamSynchronize(h->stream));
    return SL_OK;
}

int sl_step_host(sl_handle* h, double* pos, double* vel, double* w, double* acc, double* aacc, int write,
                 sl_energy* out)
{
    if (int r = check_handle(h)) return r;
    if (!h->uploaded) return fail(SL_ERR_STATE, "sl_upload first");
    if (!acc || !aacc) return fail(SL_ERR_ARG, "acc or aacc is NULL");
    // The arrays hold the state at the end of the caller's previous step:
    // the previous-step positions are the current ones (pos_prev NULL), as
    // the reference's `distances` hold the current positions' pair distances
    // between steps.  Where the GPU reaches all five arrays, the finite check
    // of the input runs in the staging kernel and a rejected input is never
    // written back; otherwise it runs on the host first.
    bool reach = true;
    for (const double* p : {static_cast<const double*>(pos), static_cast<const double*>(vel),
                            static_cast<const double*>(w), static_cast<const double*>(acc),
                            static_cast<const double*>(aacc)})
        reach = reach && p && device_view(h, p) != nullptr;
    if (int r = enqueue_resume(h, pos, vel, w, acc, aacc, nullptr, reach)) return r;
    h->forces_ready = true;
    if (int r = enqueue_step(h, write != 0)) return r;
    if (int r = enqueue_download(h, pos, vel, w, acc, aacc, reach)) return r;
    const int r = fetch_energy_and_status(h, out, write != 0);
    if (r == SL_ERR_ARG) h->forces_ready = false;  // the device copy holds the rejected input
    return r;
}

int sl_contacts(sl_handle* h, int* pairs, long max_pairs, long* count)
{
    if (int r = check_handle(h)) return r;
    if (!count) return fail(SL_ERR_ARG, "count is NULL");
    if (!h->forces_ready) return fail(SL_ERR_STATE, "no force pass has run");
    const sl::System& s = h->sys;
    std::vector<uint32_t> mask((size_t)s.npad * s.nb);
    SL_CUDA(cudaMemcpyAsync(mask.data(), s.cmask, mask.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    SL_CUDA(cudaStreamSynchronize(h->stream));
    long c = 0;
    for (int A = 0; A < s.n; ++A) {
        for (int Y = 0; Y <= A / sl::kBlock; ++Y) {
            // [npad][nb] in the exact form, [nb][npad] in the mixed form
            uint32_t wd = h->mode != SL_MODE_EXACT ? mask[(size_t)Y * s.npad + A] : mask[(size_t)A * s.nb + Y];
            while (wd) {
                const int b = __builtin_ctz(wd);
                wd &= wd - 1;
                const int B = Y * sl::kBlock + b;
                if (B >= A) break;
                if (pairs && c < max_pairs) { pairs[2 * c] = A; pairs[2 * c + 1] = B; }
                ++c;
            }
        }
    }
    *count = c;
    return SL_OK;
}

void* sl_stream(sl_handle* h) { return h ? static_cast<void*>(h->stream) : nullptr; }

int sl_set_overlap(sl_handle* h, int enable)
{
    if (int r = check_handle(h)) return r;
    if (enable && !h->has_ov) return fail(SL_ERR_UNSUPPORTED, "the pipelined step exists in exact mode only");
    SL_CUDA(cudaStreamSynchronize(h->stream));
    if (h->overlap != (enable != 0)) drop_graph(h);
    h->overlap = enable != 0;
    return SL_OK;
}

int sl_set_rowsum(sl_handle* h, int method)
{
    if (int r = check_handle(h)) return r;
    if (method != SL_ROWSUM_INT && method != SL_ROWSUM_FP64) return fail(SL_ERR_ARG, "unknown row-sum method");
    if (h->mode != SL_MODE_EXACT) return fail(SL_ERR_UNSUPPORTED, "the row-sum method applies to exact mode only");
    SL_CUDA(cudaStreamSynchronize(h->stream));
    const bool want = method == SL_ROWSUM_INT;
    if (h->rowsum_int != want) drop_graph(h);
    h->rowsum_int = want;
    return SL_OK;
}

int sl_step_launches(const sl_handle* h, int write, int* count)
{
    if (int r = check_handle(h)) return r;
    if (!count) return fail(SL_ERR_ARG, "count is NULL");
    int np = 1;
    if (h->mode == SL_MODE_EXACT && h->overlap) {
        int cb[sl::kPairPhases + 1];
        np = sl::phase_bounds(h->sys.nb, cb);
    }
    *count = 1 + 2 * np + (write ? 2 : 0);  // drift, pair + row-sum per phase, energy
    return SL_OK;
}

int sl_pair_kernel(const sl_handle* h, const char** name)
{
    if (int r = check_handle(h)) return r;
    if (!name) return fail(SL_ERR_ARG, "name is NULL");
    *name = h->mode == SL_MODE_EXACT ? "pair_tile_kernel"
            : h->mode == SL_MODE_MIXED ? "mixed64_pair_kernel"
            : h->sys.pair_double       ? "mixed_pair2_kernel"
                                       : "mixed_pair_kernel";
    return SL_OK;
}

int sl_kernel_timing(sl_handle* h, int enable)
{
    if (int r = check_handle(h)) return r;
    SL_CUDA(cudaStreamSynchronize(h->stream));
    h->timing = enable != 0;
    h->timers_used = 0;
    h->pair_ms = h->rowsum_ms = 0;
    h->launches = 0;
    return SL_OK;
}

int sl_kernel_times(sl_handle* h, double* pair_ms, double* rowsum_ms, long* launches, int reset)
{
    if (int r = check_handle(h)) return r;
    SL_CUDA(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < h->timers_used; ++k) {
        float a = 0, b = 0;
        SL_CUDA(cudaEventElapsedTime(&a, h->timers[k].ev[0], h->timers[k].ev[1]));
        SL_CUDA(cudaEventElapsedTime(&b, h->timers[k].ev[1], h->timers[k].ev[2]));
        h->pair_ms += a;
        h->rowsum_ms += b;
        h->launches += 1;
    }
    h->timers_used = 0;
    if (pair_ms) *pair_ms = h->pair_ms;
    if (rowsum_ms) *rowsum_ms = h->rowsum_ms;
    if (launches) *launches = h->launches;
    if (reset) { h->pair_ms = h->rowsum_ms = 0; h->launches = 0; }
    return SL_OK;
}

int sl_device_bytes(const sl_handle* h, uint64_t* bytes)
{
    if (int r = check_handle(h)) return r;
    if (!bytes) return fail(SL_ERR_ARG, "bytes is NULL");
    *bytes = h->arena_bytes;
    return SL_OK;
}

}  // extern "C"

// sl_batch_capi.cu -- extern "C" API of the batched solver
// (include/spacelab_batch.h): a batch of independent systems in one device
// arena, advanced by one persistent, graph-captured launch, with a
// project-written autotuner for the j-tile size and threads per instance.
#include "../../include/spacelab_batch.h"
#include "../../include/spacelab_gpu.h"
#include "sl_batch.h"
#include "sl_pair_mixed.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

int sl_record_error(int code, const char* msg);

namespace {

#define SLB_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return sl_record_error(SL_ERR_CUDA, (std::string(#call) + ": " +     \
                                                                    cudaGetErrorString(e_)).c_str()); \
    } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

const int kTiles[4] = {32, 64, 128, 0};  // 0: the mixed form's pair-tile pass
const int kThreads[3] = {64, 128, 256};
const int kThreadsTiles[3] = {128, 256, 512};  // the mixed pair-tile pass's candidates
// device memory the exact pair-tile pass's per-CTA buffers may take: at
// most this, and at most a third of the free memory at creation
constexpr size_t kExactTileScratchBytes = size_t(48) << 30;

}  // namespace

struct sl_batch {
    sl::Batch b{};
    int mode = SL_MODE_EXACT;
    int steps = 0, skip = 0;
    int num_sms = 0;
    int tile = 64, threads = 128;
    cudaStream_t stream = nullptr;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    double* snapshot = nullptr;  // initial state for the autotuner (device)
    bool uploaded = false;
    std::vector<int> counts, offsets;
};

namespace {

int blocks_for(const sl_batch* h, int tile, int threads)
{
    int per_sm = sl::batch_max_blocks_per_sm(tile, threads, h->mode == SL_MODE_MIXED_DF);
    if (per_sm < 1) per_sm = 1;
    long long blocks = (long long)per_sm * h->num_sms;
    if (tile == 0 && blocks > h->b.part_ctas) blocks = h->b.part_ctas;  // one scratch region per CTA
    if (blocks > h->b.ninst) blocks = h->b.ninst;
    return (int)blocks;
}

// One persistent launch over all instances, captured as a CUDA graph
// (queue reset + kernel) and launched.
int launch_run(sl_batch* h, int tile, int threads, int first_step, int nsteps, int do_init, int skip)
{
    const int blocks = blocks_for(h, tile, threads);
    cudaGraph_t g;
    SLB_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(h->b.counter, 0, sizeof(int), h->stream);
    if (h->mode == SL_MODE_MIXED_DF)
        sl::launch_batch_mixed(h->b, tile, threads, blocks, first_step, nsteps, skip, do_init, h->stream);
    else
        sl::launch_batch_exact(h->b, tile, threads, blocks, first_step, nsteps, skip, do_init, h->stream);
    SLB_CUDA(cudaStreamEndCapture(h->stream, &g));
    cudaGraphExec_t ge;
    const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
    const cudaError_t e2 = cudaGraphLaunch(ge, h->stream);
    const cudaError_t e3 = cudaStreamSynchronize(h->stream);
    cudaGraphExecDestroy(ge);
    if (e2 != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e2));
    if (e3 != cudaSuccess) return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e3));
    return SL_OK;
}

// device-to-device copy of the 5 vec3 state arrays to/from the snapshot
int snapshot_copy(sl_batch* h, bool save)
{
    const sl::Vec3Soa* v[5] = {&h->b.pos, &h->b.vel, &h->b.w, &h->b.acc, &h->b.aacc};
    const size_t bytes = (size_t)h->b.total * sizeof(double);
    for (int k = 0; k < 5; ++k)
        for (int c = 0; c < 3; ++c) {
            double* snap = h->snapshot + (size_t)(3 * k + c) * h->b.total;
            if (save)
                SLB_CUDA(cudaMemcpyAsync(snap, v[k]->c[c], bytes, cudaMemcpyDeviceToDevice, h->stream));
            else
                SLB_CUDA(cudaMemcpyAsync(v[k]->c[c], snap, bytes, cudaMemcpyDeviceToDevice, h->stream));
        }
    SLB_CUDA(cudaStreamSynchronize(h->stream));
    return SL_OK;
}

}  // namespace

namespace {

// Spreads the low 10 bits of x to every third bit (bits 0, 3, ..., 27).
uint32_t spread3(uint32_t x)
{
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// Per instance, its spheres' global indices sorted by the Z-order (Morton)
// code of their positions quantised to 10 bits per axis over the instance's
// bounding box; ties keep index order.
std::vector<int> zorder_perm(const std::vector<int>& offsets, const std::vector<int>& counts, const double* pos)
{
    std::vector<int> perm;
    perm.reserve(offsets.empty() ? 0 : offsets.back() + counts.back());
    std::vector<std::pair<uint32_t, int>> key;
    for (size_t inst = 0; inst < offsets.size(); ++inst) {
        const int off = offsets[inst], n = counts[inst];
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int i = off; i < off + n; ++i)
            for (int c = 0; c < 3; ++c) {
                lo[c] = std::min(lo[c], pos[3 * (size_t)i + c]);
                hi[c] = std::max(hi[c], pos[3 * (size_t)i + c]);
            }
        key.clear();
        for (int i = off; i < off + n; ++i) {
            uint32_t code = 0;
            for (int c = 0; c < 3; ++c) {
                const double ext = hi[c] - lo[c];
                const double q = ext > 0 ? (pos[3 * (size_t)i + c] - lo[c]) / ext * 1023.0 : 0.0;
                code |= spread3((uint32_t)std::min(1023.0, std::max(0.0, q))) << c;
            }
            key.emplace_back(code, i);
        }
        std::stable_sort(key.begin(), key.end(),
                         [](const std::pair<uint32_t, int>& a, const std::pair<uint32_t, int>& c) { return a.first < c.first; });
        for (const auto& k : key) perm.push_back(k.second);
    }
    return perm;
}

}  // namespace

extern "C" {

int sl_batch_create(int ninst, const int* counts, const sl_material* mat, int mode, int steps, int skip,
                    sl_batch** out)
{
    if (!out) return sl_record_error(SL_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (ninst < 1 || !counts || !mat) return sl_record_error(SL_ERR_ARG, "need ninst >= 1, counts and material");
    if (mode != SL_MODE_EXACT && mode != SL_MODE_MIXED_DF)
        return sl_record_error(SL_ERR_UNSUPPORTED, "the batched solver runs SL_MODE_EXACT or SL_MODE_MIXED_DF");
    if (steps < 0 || skip < 1) return sl_record_error(SL_ERR_ARG, "need steps >= 0 and skip >= 1");
    if (!(mat->h_min > 0)) return sl_record_error(SL_ERR_ARG, "h_min must be > 0");
    long long total = 0;
    for (int i = 0; i < ninst; ++i) {
        if (counts[i] < 1) return sl_record_error(SL_ERR_ARG, "every instance needs >= 1 sphere");
        total += counts[i];
    }
    if (total > (1ll << 30)) return sl_record_error(SL_ERR_ARG, "batch too large");
    sl_batch* h = new (std::nothrow) sl_batch();
    if (!h) return sl_record_error(SL_ERR_ALLOC, "host allocation failed");
    h->mode = mode;
    h->steps = steps;
    h->skip = skip;
    h->counts.assign(counts, counts + ninst);
    h->offsets.resize(ninst);
    std::exclusive_scan(h->counts.begin(), h->counts.end(), h->offsets.begin(), 0);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return sl_record_error(SL_ERR_CUDA, "cudaStreamCreate failed");
    }
    sl::Batch& b = h->b;
    b.ninst = ninst;
    b.total = (int)total;
    b.nrec = steps / skip + 1;
    b.mat = sl::Material{mat->G, mat->Ha, mat->u_s, mat->u_r, mat->h_min};
    const size_t T = (size_t)total;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    size_t o_vec[8][3], o_sc[8], o_f[10];
    for (auto& v : o_vec)
        for (auto& c : v) c = take(T * sizeof(double));
    for (auto& s : o_sc) s = take(T * sizeof(double));
    for (auto& f : o_f) f = take(mode == SL_MODE_MIXED_DF ? T * sizeof(float) : 0);
    const size_t o_order = take(ninst * sizeof(int)), o_off = take(ninst * sizeof(int)),
                 o_cnt = take(ninst * sizeof(int)), o_counter = take(sizeof(int));
    const size_t o_par = take(4 * (size_t)ninst * sizeof(double));
    const size_t o_en = take((size_t)ninst * b.nrec * 8 * sizeof(double));
    const size_t o_st = take(ninst * sizeof(unsigned));
    const size_t o_snap = take(15 * T * sizeof(double));
    const size_t o_perm = take(mode == SL_MODE_MIXED_DF ? T * sizeof(int) : 0);
    // mixed: the pair-tile pass's per-CTA partials, sized for the largest instance
    const int max_n = *std::max_element(counts, counts + ninst);
    b.part_nb = (max_n + sl::kBlock - 1) / sl::kBlock;
    b.part_np = b.part_nb * sl::kBlock;
    b.part_cta = 6 * (size_t)b.part_nb * b.part_np;
    // no more CTAs than instances ever run at once
    const long long max_ctas = std::min<long long>((long long)h->num_sms * sl::kTileCtasPerSm, ninst);
    b.part_ctas = (int)max_ctas;
    const size_t o_part = take(mode == SL_MODE_MIXED_DF ? b.part_cta * b.part_ctas * sizeof(float) : 0);
    // exact: the pair-tile pass's per-CTA pair terms, torques and contact
    // words at the largest instance's padded size, where that fits the
    // budget for at least one CTA per SM
    b.x_nb = b.part_nb;
    b.x_np = b.part_np;
    b.xpair_cta = 3 * (size_t)b.x_np * b.x_np;
    b.xmask_cta = (size_t)b.x_np * b.x_nb;
    size_t o_xpair = 0, o_xtorq = 0, o_xmask = 0;
    bool exact_tiles = false;
    if (mode == SL_MODE_EXACT) {
        const size_t per_cta = 2 * b.xpair_cta * sizeof(double) + b.xmask_cta * sizeof(uint32_t);
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
        const long long fit = (long long)(std::min(kExactTileScratchBytes, free_b / 3) / per_cta);
        const long long ctas = std::min<long long>(max_ctas, fit);
        if (ctas >= std::min<long long>(h->num_sms, ninst)) {
            exact_tiles = true;
            b.part_ctas = (int)ctas;
            o_xpair = take(b.xpair_cta * ctas * sizeof(double));
            o_xtorq = take(b.xpair_cta * ctas * sizeof(double));
            o_xmask = take(b.xmask_cta * ctas * sizeof(uint32_t));
        }
    }
    const size_t o_isc = take((size_t)ninst * sizeof(sl::Scalars));
    h->arena_bytes = off;
    if (cudaMalloc(&h->arena, off) != cudaSuccess) {
        sl_batch_destroy(h);
        return sl_record_error(SL_ERR_ALLOC, "cudaMalloc of the batch arena failed");
    }
    char* base = static_cast<char*>(h->arena);
    sl::Vec3Soa* vecs[8] = {&b.pos, &b.prev, &b.vel, &b.velh, &b.w, &b.wh, &b.acc, &b.aacc};
    for (int v = 0; v < 8; ++v)
        for (int c = 0; c < 3; ++c) vecs[v]->c[c] = reinterpret_cast<double*>(base + o_vec[v][c]);
    double* inv_m_slot = nullptr;  // 8 bytes per sphere, holds the mass reciprocals rm
    double** scal[8] = {&b.R, &b.m, &b.moi, &b.twoR, &b.fourR, &b.cR3, &inv_m_slot, &b.inv_moi};
    for (int k = 0; k < 8; ++k) *scal[k] = reinterpret_cast<double*>(base + o_sc[k]);
    b.rm = reinterpret_cast<unsigned long long*>(inv_m_slot);
    if (mode == SL_MODE_MIXED_DF) {
        b.f_R = reinterpret_cast<float*>(base + o_f[0]);
        b.f_inv_m = reinterpret_cast<float*>(base + o_f[1]);
        b.f_inv_moi = reinterpret_cast<float*>(base + o_f[2]);
        b.f_Rlo = reinterpret_cast<float*>(base + o_f[3]);
        for (int k = 0; k < 6; ++k) b.f_pos[k] = reinterpret_cast<float*>(base + o_f[4 + k]);
        b.perm = reinterpret_cast<const int*>(base + o_perm);
        b.part = reinterpret_cast<float*>(base + o_part);
    }
    int* order = reinterpret_cast<int*>(base + o_order);
    int* doff = reinterpret_cast<int*>(base + o_off);
    int* dcnt = reinterpret_cast<int*>(base + o_cnt);
    b.order = order; b.off = doff; b.cnt = dcnt;
    b.counter = reinterpret_cast<int*>(base + o_counter);
    double* par = reinterpret_cast<double*>(base + o_par);
    b.dt = par; b.kin = par + ninst; b.kout = par + 2 * ninst; b.u_s = par + 3 * ninst;
    b.energy = reinterpret_cast<double*>(base + o_en);
    if (exact_tiles) {
        b.xpair = reinterpret_cast<double*>(base + o_xpair);
        b.xtorq = reinterpret_cast<double*>(base + o_xtorq);
        b.xmask = reinterpret_cast<uint32_t*>(base + o_xmask);
    }
    b.isc = reinterpret_cast<sl::Scalars*>(base + o_isc);
    b.status = reinterpret_cast<unsigned*>(base + o_st);
    h->snapshot = reinterpret_cast<double*>(base + o_snap);
    // largest instances first: the work queue then balances like LPT scheduling
    std::vector<int> ord(ninst);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) { return counts[a] > counts[c]; });
    cudaError_t e = cudaMemsetAsync(h->arena, 0, off, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(order, ord.data(), ninst * sizeof(int), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(doff, h->offsets.data(), ninst * sizeof(int), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dcnt, counts, ninst * sizeof(int), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        sl_batch_destroy(h);
        return sl_record_error(SL_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = h;
    return SL_OK;
}

int sl_batch_destroy(sl_batch* h)
{
    if (!h) return SL_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->arena) cudaFree(h->arena);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SL_OK;
}

int sl_batch_upload(sl_batch* h, const double* pos, const double* vel, const double* w, const double* R,
                    const double* m, const double* moi, const double* dt, const double* kin, const double* kout,
                    const double* u_s)
{
    if (!h) return sl_record_error(SL_ERR_ARG, "null batch");
    if (!pos || !vel || !w || !R || !m || !moi || !dt || !kin || !kout || !u_s)
        return sl_record_error(SL_ERR_ARG, "NULL input array");
    sl::Batch& b = h->b;
    const size_t T = (size_t)b.total;
    double rmax = 0;
    for (size_t i = 0; i < T; ++i) {
        if (!(R[i] > 0) || !(m[i] > 0) || !(moi[i] > 0)) return sl_record_error(SL_ERR_ARG, "R, m, moi must be > 0");
        rmax = std::max(rmax, R[i]);
    }
    for (size_t i = 0; i < 3 * T; ++i)
        if (!std::isfinite(pos[i]) || !std::isfinite(vel[i]) || !std::isfinite(w[i]))
            return sl_record_error(SL_ERR_ARG, "non-finite position, velocity or spin");
    for (int i = 0; i < b.ninst; ++i)
        if (!(dt[i] >= 0) || !(kin[i] >= 0) || !(kout[i] >= 0) || !(u_s[i] >= 0))
            return sl_record_error(SL_ERR_ARG, "per-instance dt, kin, kout, u_s must be >= 0");
    int ex = 0;
    std::frexp(rmax, &ex);
    b.len_shift = ex - 1;
    double rmin = R[0];
    for (size_t i = 0; i < T; ++i) rmin = std::min(rmin, R[i]);
    b.far_sq = sl::far_threshold_sq(b.mat.h_min, rmin);
    std::vector<double> tmp(T);
    const double* v3[3] = {pos, vel, w};
    sl::Vec3Soa* dv[3] = {&b.pos, &b.vel, &b.w};
    for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c) {
            for (size_t i = 0; i < T; ++i) tmp[i] = v3[k][3 * i + c];
            SLB_CUDA(cudaMemcpy(dv[k]->c[c], tmp.data(), T * sizeof(double), cudaMemcpyHostToDevice));
        }
    for (int c = 0; c < 3; ++c) {
        SLB_CUDA(cudaMemset(b.acc.c[c], 0, T * sizeof(double)));
        SLB_CUDA(cudaMemset(b.aacc.c[c], 0, T * sizeof(double)));
    }
    SLB_CUDA(cudaMemcpy(b.R, R, T * sizeof(double), cudaMemcpyHostToDevice));
    SLB_CUDA(cudaMemcpy(b.m, m, T * sizeof(double), cudaMemcpyHostToDevice));
    SLB_CUDA(cudaMemcpy(b.moi, moi, T * sizeof(double), cudaMemcpyHostToDevice));
    const double* par[4] = {dt, kin, kout, u_s};
    double* dpar = const_cast<double*>(b.dt);
    for (int k = 0; k < 4; ++k)
        SLB_CUDA(cudaMemcpy(dpar + (size_t)k * b.ninst, par[k], b.ninst * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<sl::Scalars> isc(b.ninst);
    for (int i = 0; i < b.ninst; ++i) isc[i] = sl::Scalars{dt[i], kin[i], kout[i]};
    SLB_CUDA(cudaMemcpy(b.isc, isc.data(), b.ninst * sizeof(sl::Scalars), cudaMemcpyHostToDevice));
    if (b.perm) {
        const std::vector<int> perm = zorder_perm(h->offsets, h->counts, pos);
        SLB_CUDA(cudaMemcpy(const_cast<int*>(b.perm), perm.data(), T * sizeof(int), cudaMemcpyHostToDevice));
    }
    SLB_CUDA(cudaMemset(b.status, 0, b.ninst * sizeof(unsigned)));
    sl::launch_batch_derive(b, h->stream);
    SLB_CUDA(cudaGetLastError());
    SLB_CUDA(cudaStreamSynchronize(h->stream));
    h->uploaded = true;
    return SL_OK;
}

int sl_batch_set_shape(sl_batch* h, int tile, int threads)
{
    if (!h) return sl_record_error(SL_ERR_ARG, "null batch");
    const bool mixed = h->mode == SL_MODE_MIXED_DF;
    const bool threads_ok = threads == 64 || threads == 128 || threads == 256 || (tile == 0 && mixed && threads == 512);
    if ((tile != 32 && tile != 64 && tile != 128 && tile != 0) || !threads_ok)
        return sl_record_error(SL_ERR_ARG,
                               "tile must be 32/64/128 (or 0) and threads 64/128/256 (or 512 with tile 0, mixed)");
    if (tile == 0 && !mixed && !h->b.xpair)
        return sl_record_error(SL_ERR_UNSUPPORTED, "the exact pair-tile pass's buffers do not fit for this batch");
    h->tile = tile;
    h->threads = threads;
    return SL_OK;
}

int sl_batch_autotune(sl_batch* h, int sample_steps, int* tile, int* threads, double* times_ms)
{
    if (!h || !h->uploaded) return sl_record_error(SL_ERR_STATE, "upload the batch first");
    if (sample_steps < 1) return sl_record_error(SL_ERR_ARG, "sample_steps must be >= 1");
    if (int r = snapshot_copy(h, true)) return r;
    cudaEvent_t e0, e1;
    SLB_CUDA(cudaEventCreate(&e0));
    SLB_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int bt = h->tile, bth = h->threads, k = 0;
    for (int ti = 0; ti < 4; ++ti)
        for (int hi = 0; hi < 3; ++hi, ++k) {
            const bool mixed = h->mode == SL_MODE_MIXED_DF;
            if (kTiles[ti] == 0 && !mixed && !h->b.xpair) {
                if (times_ms) times_ms[k] = -1.0;
                continue;
            }
            if (int r = snapshot_copy(h, false)) return r;
            const int thr = kTiles[ti] == 0 && mixed ? kThreadsTiles[hi] : kThreads[hi];
            // first launch compiles nothing but warms the caches; time the second
            if (int r = launch_run(h, kTiles[ti], thr, 1, 1, 0, 0)) return r;
            cudaEventRecord(e0, h->stream);
            if (int r = launch_run(h, kTiles[ti], thr, 2, sample_steps, 0, 0)) return r;
            cudaEventRecord(e1, h->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (times_ms) times_ms[k] = ms;
            if (ms < best) { best = ms; bt = kTiles[ti]; bth = thr; }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (int r = snapshot_copy(h, false)) return r;
    SLB_CUDA(cudaMemset(h->b.status, 0, h->b.ninst * sizeof(unsigned)));
    h->tile = bt;
    h->threads = bth;
    if (tile) *tile = bt;
    if (threads) *threads = bth;
    return SL_OK;
}

int sl_batch_run(sl_batch* h, int first_step, int nsteps, int do_init)
{
    if (!h || !h->uploaded) return sl_record_error(SL_ERR_STATE, "upload the batch first");
    if (first_step < 1 || nsteps < 0) return sl_record_error(SL_ERR_ARG, "need first_step >= 1, nsteps >= 0");
    return launch_run(h, h->tile, h->threads, first_step, nsteps, do_init, h->skip);
}

int sl_batch_download(sl_batch* h, double* pos, double* vel, double* w, double* acc, double* aacc)
{
    if (!h) return sl_record_error(SL_ERR_ARG, "null batch");
    const size_t T = (size_t)h->b.total;
    std::vector<double> tmp(T);
    double* outs[5] = {pos, vel, w, acc, aacc};
    const sl::Vec3Soa* src[5] = {&h->b.pos, &h->b.vel, &h->b.w, &h->b.acc, &h->b.aacc};
    for (int k = 0; k < 5; ++k) {
        if (!outs[k]) continue;
        for (int c = 0; c < 3; ++c) {
            SLB_CUDA(cudaMemcpy(tmp.data(), src[k]->c[c], T * sizeof(double), cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < T; ++i) outs[k][3 * i + c] = tmp[i];
        }
    }
    return SL_OK;
}

int sl_batch_energy(sl_batch* h, double* energy, int* nrec)
{
    if (!h) return sl_record_error(SL_ERR_ARG, "null batch");
    if (nrec) *nrec = h->b.nrec;
    if (energy)
        SLB_CUDA(cudaMemcpy(energy, h->b.energy, (size_t)h->b.ninst * h->b.nrec * 8 * sizeof(double),
                            cudaMemcpyDeviceToHost));
    return SL_OK;
}

int sl_batch_status(sl_batch* h, unsigned* status)
{
    if (!h || !status) return sl_record_error(SL_ERR_ARG, "null argument");
    SLB_CUDA(cudaMemcpy(status, h->b.status, h->b.ninst * sizeof(unsigned), cudaMemcpyDeviceToHost));
    return SL_OK;
}

int sl_batch_shape(const sl_batch* h, int* tile, int* threads, int* blocks)
{
    if (!h) return sl_record_error(SL_ERR_ARG, "null batch");
    if (tile) *tile = h->tile;
    if (threads) *threads = h->threads;
    if (blocks) *blocks = blocks_for(h, h->tile, h->threads);
    return SL_OK;
}

}  // extern "C"

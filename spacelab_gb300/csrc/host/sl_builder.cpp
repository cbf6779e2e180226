// sl_builder.cpp -- seeded, platform-independent cluster builder and setup
// helpers (include/spacelab_host.h).  Compiled with -ffp-contract=off so the
// same seed gives the same bits on x86-64 and aarch64.
#include "../../../include/spacelab_host.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr double kPi = 3.141592653589793;
constexpr double kLn2 = 0.6931471805599453;           // RN(ln 2)
constexpr double kLn2Hi = 0.693147180369123816490;    // ln 2 split for exp's
constexpr double kLn2Lo = 1.90821492927058770002e-10; // range reduction

uint64_t splitmix64(uint64_t& x)
{
    uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

// xoshiro256** (Blackman & Vigna, 2018).
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed)
    {
        uint64_t x = seed;
        for (auto& v : s) v = splitmix64(x);
    }
    uint64_t next()
    {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform in [0, 1) with 53 random bits
    double uniform() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }
    // Marsaglia polar method; the second deviate is kept for the next call.
    bool have_spare = false;
    double spare = 0;
    double gauss()
    {
        if (have_spare) { have_spare = false; return spare; }
        double u, v, q;
        do {
            u = 2 * uniform() - 1;
            v = 2 * uniform() - 1;
            q = u * u + v * v;
        } while (q >= 1 || q == 0);
        const double f = std::sqrt(-2 * slh_log(q) / q);
        spare = v * f;
        have_spare = true;
        return u * f;
    }
};

// cube root by Newton's method from an exp/log start, basic operations only
double det_cbrt(double x)
{
    if (!(x > 0)) return 0;
    double y = slh_exp(slh_log(x) / 3);
    for (int k = 0; k < 4; ++k) y = y - (y * y * y - x) / (3 * y * y);
    return y;
}

int place_cluster(Rng& rng, int n, const double* R, double Rc, double* pos)
{
    double rmax = 0;
    for (int i = 0; i < n; ++i) rmax = std::max(rmax, R[i]);
    const double cell = 2 * rmax;
    const int G = static_cast<int>(std::ceil(2 * Rc / cell)) + 1;
    std::vector<int> head((size_t)G * G * G, -1), next(n, -1);
    auto cell_of = [&](double v) {
        int c = static_cast<int>((v + Rc) / cell);
        return c < 0 ? 0 : (c >= G ? G - 1 : c);
    };
    const long long max_attempts = 20000000LL;
    for (int i = 0; i < n; ++i) {
        long long attempts = 0;
        for (;;) {
            if (++attempts > max_attempts) return 2;
            const double x = (2 * rng.uniform() - 1) * Rc;
            const double y = (2 * rng.uniform() - 1) * Rc;
            const double z = (2 * rng.uniform() - 1) * Rc;
            if (x * x + y * y + z * z > Rc * Rc) continue;
            const int cx = cell_of(x), cy = cell_of(y), cz = cell_of(z);
            bool ok = true;
            for (int dx = -1; dx <= 1 && ok; ++dx)
                for (int dy = -1; dy <= 1 && ok; ++dy)
                    for (int dz = -1; dz <= 1 && ok; ++dz) {
                        const int gx = cx + dx, gy = cy + dy, gz = cz + dz;
                        if (gx < 0 || gy < 0 || gz < 0 || gx >= G || gy >= G || gz >= G) continue;
                        for (int j = head[((size_t)gx * G + gy) * G + gz]; j >= 0; j = next[j]) {
                            const double ex = x - pos[3 * j], ey = y - pos[3 * j + 1], ez = z - pos[3 * j + 2];
                            const double lim = (R[i] + R[j]) * (1 + 1e-9);
                            if (ex * ex + ey * ey + ez * ez <= lim * lim) { ok = false; break; }
                        }
                    }
            if (!ok) continue;
            pos[3 * i] = x; pos[3 * i + 1] = y; pos[3 * i + 2] = z;
            const size_t c = ((size_t)cx * G + cy) * G + cz;
            next[i] = head[c];
            head[c] = i;
            break;
        }
    }
    return 0;
}

}  // namespace

extern "C" {

double slh_log(double x)
{
    if (!(x > 0)) return -HUGE_VAL;
    int e = 0;
    double m = std::frexp(x, &e);  // exact: x = m 2^e, m in [0.5, 1)
    if (m < 0.70710678118654752) { m *= 2; e -= 1; }
    const double s = (m - 1) / (m + 1);  // |s| <= 0.1716
    const double s2 = s * s;
    double p = 1.0 / 31;
    for (int k = 14; k >= 0; --k) p = p * s2 + 1.0 / (2 * k + 1);  // atanh series
    return 2 * s * p + e * kLn2;
}

double slh_exp(double x)
{
    if (x > 709) return HUGE_VAL;
    if (x < -745) return 0;
    const double k = std::nearbyint(x / kLn2);
    const double r = (x - k * kLn2Hi) - k * kLn2Lo;  // |r| <= 0.35
    double p = 1.0;
    for (int i = 22; i >= 1; --i) p = 1.0 + p * r / i;
    return std::ldexp(p, static_cast<int>(k));
}

uint64_t slh_rng_next(uint64_t* state4)
{
    Rng r(0);
    std::memcpy(r.s, state4, sizeof(r.s));
    const uint64_t v = r.next();
    std::memcpy(state4, r.s, sizeof(r.s));
    return v;
}

int slh_to_origin(int n, double* pos, const double* m)
{
    if (n < 1 || !pos || !m) return 1;
    double mt = 0;
    for (int i = 0; i < n; ++i) mt += m[i];
    double cx = 0, cy = 0, cz = 0;
    for (int i = 0; i < n; ++i) {
        cx += m[i] * pos[3 * i]; cy += m[i] * pos[3 * i + 1]; cz += m[i] * pos[3 * i + 2];
    }
    cx = cx / mt; cy = cy / mt; cz = cz / mt;
    for (int i = 0; i < n; ++i) { pos[3 * i] -= cx; pos[3 * i + 1] -= cy; pos[3 * i + 2] -= cz; }
    return 0;
}

int slh_build_cluster(int n, double median_radius, double sigma_ln, double clip_lo, double clip_hi,
                      double rho, double phi, double sigma_v, uint64_t seed, double* pos, double* vel,
                      double* w, double* R, double* m, double* moi)
{
    if (n < 1 || !(median_radius > 0) || !(rho > 0) || !(phi > 0) || !(phi < 0.5) || sigma_ln < 0 ||
        sigma_v < 0 || !pos || !vel || !w || !R || !m || !moi)
        return 1;
    if (sigma_ln > 0 && !(clip_lo > 0 && clip_hi >= clip_lo)) return 1;
    Rng rng(seed);
    for (int i = 0; i < n; ++i) {
        double f = 1.0;
        if (sigma_ln > 0) {
            f = slh_exp(sigma_ln * rng.gauss());
            f = std::min(std::max(f, clip_lo), clip_hi);
        }
        R[i] = median_radius * f;
    }
    std::sort(R, R + n, [](double a, double b) { return a > b; });  // place large spheres first
    double vol = 0;
    for (int i = 0; i < n; ++i) vol += R[i] * R[i] * R[i];
    const double Rc = det_cbrt(vol / phi);
    if (int r = place_cluster(rng, n, R, Rc, pos)) return r;
    for (int i = 0; i < 3 * n; ++i) vel[i] = sigma_v * rng.gauss();
    for (int i = 0; i < 3 * n; ++i) w[i] = 0;
    for (int i = 0; i < n; ++i) {
        m[i] = rho * 4.0 / 3.0 * kPi * (R[i] * R[i] * R[i]);
        moi[i] = .4 * m[i] * R[i] * R[i];
    }
    return slh_to_origin(n, pos, m);
}

int slh_build_collision(int n_t, int n_p, double radius, double rho, double phi, double sigma_v,
                        double speed, double off_x, double off_y, uint64_t seed_t, uint64_t seed_p,
                        double* pos, double* vel, double* w, double* R, double* m, double* moi)
{
    if (n_t < 1 || n_p < 1 || !pos || !vel || !w || !R || !m || !moi) return 1;
    const int n = n_t + n_p;
    // target in [0, n_t), projectile in [n_t, n)
    if (int r = slh_build_cluster(n_t, radius, 0, 1, 1, rho, phi, sigma_v, seed_t, pos, vel, w, R, m, moi))
        return r;
    if (int r = slh_build_cluster(n_p, radius, 0, 1, 1, rho, phi, sigma_v, seed_p, pos + 3 * n_t,
                                  vel + 3 * n_t, w + 3 * n_t, R + n_t, m + n_t, moi + n_t))
        return r;
    const double Rt = radius * det_cbrt(n_t / phi);
    const double Rp = radius * det_cbrt(n_p / phi);
    double mt = 0, mp = 0;
    for (int i = 0; i < n_t; ++i) mt += m[i];
    for (int i = n_t; i < n; ++i) mp += m[i];
    const double vSmall = -speed;             // ball_group.hpp:1415
    const double vBig = -(mp / mt) * vSmall;  // ball_group.hpp:1416
    for (int i = n_t; i < n; ++i) {
        pos[3 * i] += off_x * (Rt + Rp);
        pos[3 * i + 1] += off_y * (Rt + Rp);
        vel[3 * i] += vSmall;
    }
    for (int i = 0; i < n_t; ++i) vel[3 * i] += vBig;
    return slh_to_origin(n, pos, m);
}

int slh_cluster_rg(int count, const int* n, const uint64_t* seed, double radius, double rho, double phi,
                   int threads, double* rg)
{
    if (count < 0 || (count > 0 && (!n || !seed || !rg)) || !(radius > 0)) return 1;
    if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    threads = std::min(threads, std::max(1, count));
    std::atomic<int> next{0};
    std::atomic<int> failed{0};
    auto work = [&]() {
        std::vector<double> pos, vel, w, R, m, moi;
        for (int k = next.fetch_add(1); k < count; k = next.fetch_add(1)) {
            const int nk = n[k];
            if (nk < 1) { failed.store(1); rg[k] = -1.0; continue; }
            pos.resize(3 * (size_t)nk); vel.resize(3 * (size_t)nk); w.resize(3 * (size_t)nk);
            R.resize(nk); m.resize(nk); moi.resize(nk);
            // the same call slh_build_collision makes for each of its clusters
            if (slh_build_cluster(nk, radius, 0, 1, 1, rho, phi, 1e-3, seed[k], pos.data(), vel.data(), w.data(),
                                  R.data(), m.data(), moi.data())) {
                failed.store(1);
                rg[k] = -1.0;
                continue;
            }
            if (slh_radius_of_gyration(nk, pos.data(), m.data(), &rg[k])) {
                failed.store(1);
                rg[k] = -1.0;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    return failed.load() ? 2 : 0;
}

int slh_spring_and_dt(double r_max, double m_min, double speed, double rho, double cor,
                      double steps_per_contact, double* kin, double* kout, double* dt)
{
    if (!(r_max > 0) || !(m_min > 0) || !(speed > 0) || !(rho > 0) || !(cor > 0) || !(steps_per_contact > 0) ||
        !kin || !kout || !dt)
        return 1;
    const double maxOverlap = .1;
    const double fourThirdsPiRho = 4. / 3. * kPi * rho;
    const double kConsts = 3e3 * fourThirdsPiRho / (maxOverlap * maxOverlap);
    *kin = kConsts * r_max * speed * speed;
    *kout = cor * *kin;
    *dt = kPi * std::sqrt(m_min / (2 * *kin)) / steps_per_contact;
    return 0;
}

}  // extern "C"

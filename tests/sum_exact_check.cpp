// Host check of the integer-pipe FP64 running sum (spacelab_gb300/csrc/
// sl_sum_exact.cuh) against the host's own IEEE double additions.  The same
// header is compiled into the GPU row-sum kernel; here it runs as plain C++.
//
//   pairs:     one addition s + t for random, cancelling, tie-making, few-bit
//              and special (0, -0, subnormal, Inf, NaN) operands, in the frame
//              of the true binade and of wrong ones: whenever the fast path
//              accepts, its result must be RN(s + t) bit for bit;
//   sequences: row-like sums in 16-term chunks with the shadow's predictions
//              and the FP64 repeat of failed chunks, as the kernel runs them;
//              every chunk's result must equal the sequential FP64 sum.
// Prints "pairs P fast F" / "chunks C repeated R" and exits 1 on a mismatch.
#include "sl_sum_exact.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

using namespace sl::xs;

static unsigned long long n_pairs = 0, n_fast = 0, n_bad = 0;

static void check_pair(double s, double t, int qn)
{
    Run r = from_double(s);
    if (r.q == kNoFrame) return;
    uint32_t bad = 0;
    step_in(r, qn, bad, d2u(t));
    ++n_pairs;
    if (bad) return;
    ++n_fast;
    const double e = s + t, g = to_double(r);
    if (d2u(e) != d2u(g) && ++n_bad <= 10)
        std::printf("pair mismatch: s=%a t=%a qn=%d want %a got %a\n", s, t, qn, e, g);
}

static int binade_q(double x) { return (int)((d2u(x) >> 52) & 0x7ff) - kBiasShift; }

static void pairs(std::mt19937_64& rng, long count)
{
    std::uniform_real_distribution<double> U(0, 1);
    for (long i = 0; i < count; ++i) {
        const int es = (int)(U(rng) * 80) - 40, et = es + (int)(U(rng) * 140) - 70;
        double s = std::ldexp(1.0 + U(rng), es) * (U(rng) < .5 ? -1 : 1);
        double t = std::ldexp(1.0 + U(rng), et) * (U(rng) < .5 ? -1 : 1);
        if (i % 7 == 0) t = -s * (1 + std::ldexp(U(rng) - .5, -(int)(U(rng) * 55)));  // cancellation
        if (i % 11 == 0) t = u2d(d2u(t) & ~((1ull << (int)(U(rng) * 52)) - 1));        // few significant bits
        if (i % 13 == 0) s = u2d(d2u(s) & ~((1ull << (int)(U(rng) * 52)) - 1));
        if (i % 17 == 0) t = std::ldexp(1.0, std::ilogb(s) - 53) * ((i & 1) ? 1 : -1) * (1 + (i % 3));  // ties
        const int q0 = binade_q(s + t);
        for (int dq = -3; dq <= 3; ++dq) check_pair(s, t, q0 + dq);
        check_pair(s, t, (int)(U(rng) * 256));
    }
    // halfway cases around powers of two: s = (1 + k ulp) 2^sc, t = j/4 ulp
    for (int k = -40; k < 40; ++k)
        for (int j = -300; j <= 300; ++j)
            for (int sc = -3; sc <= 3; ++sc) {
                const double s = std::ldexp(1.0 + k * 0x1p-52, sc), t = std::ldexp(j * 0x1p-54, sc);
                for (int dq = -2; dq <= 2; ++dq) check_pair(s, t, binade_q(s + t) + dq);
                check_pair(-s, t, binade_q(-s + t));
                check_pair(-s, -t, binade_q(-s - t));
            }
    const double specials[] = {0.0, -0.0, 0x1p-1074, -0x1p-1074, 0x1.8p-1030, 0x1p-1022, INFINITY, -INFINITY, NAN};
    for (double t : specials)
        for (long i = 0; i < 20000; ++i) {
            const double s = std::ldexp(1.0 + U(rng), (int)(U(rng) * 200) - 100) * (U(rng) < .5 ? -1 : 1);
            for (int dq = -2; dq <= 2; ++dq) check_pair(s, t, binade_q(s) + dq);
        }
}

// One row: n terms, summed sequentially in FP64 and in chunks of 16 as the
// kernel does (frame form + shadow, FP64 repeat of a failed chunk).
static unsigned long long n_chunks = 0, n_repeat = 0;

static void row(std::mt19937_64& rng, int n, int kind)
{
    std::uniform_real_distribution<double> U(0, 1);
    std::vector<double> t(n);
    for (int j = 0; j < n; ++j) {
        double mag;
        if (kind == 0) mag = std::ldexp(1.0, -(int)(U(rng) * 60));                       // log-uniform spread
        else if (kind == 1) mag = U(rng) < 0.003 ? std::ldexp(1.0, (int)(U(rng) * 30)) : std::ldexp(1.0, -30 - (int)(U(rng) * 30));
        else mag = std::ldexp(1.0, -(int)(U(rng) * 8));                                  // comparable terms
        t[j] = mag * (1 + U(rng)) * (U(rng) < .5 ? -1 : 1);
        if (kind == 2 && j > 0 && U(rng) < 0.05) t[j] = -t[j - 1];                      // exact cancellations
        if (U(rng) < 0.01) t[j] = U(rng) < .5 ? 0.0 : -0.0;
    }
    double seq = 0.0, slow = 0.0;
    Run run = from_double(0.0);
    for (int j0 = 0; j0 < n; j0 += 16) {
        const int j1 = j0 + 16 < n ? j0 + 16 : n;
        const Run r0 = run;
        float s32 = shadow_of(run);
        uint32_t bad = 0;
        for (int j = j0; j < j1; ++j) step(run, s32, bad, d2u(t[j]));
        ++n_chunks;
        if (bad) {
            ++n_repeat;
            double v = r0.q == kNoFrame ? slow : to_double(r0);
            for (int j = j0; j < j1; ++j) v += t[j];
            slow = v;
            run = from_double(v);
        }
        for (int j = j0; j < j1; ++j) seq += t[j];
        const double got = run.q == kNoFrame ? slow : to_double(run);
        if (d2u(got) != d2u(seq) && ++n_bad <= 10)
            std::printf("row mismatch (kind %d) at term %d: want %a got %a\n", kind, j1, seq, got);
    }
}

int main(int argc, char** argv)
{
    const long npairs = argc > 1 ? std::atol(argv[1]) : 2000000;
    const int nrows = argc > 2 ? std::atoi(argv[2]) : 300;
    std::mt19937_64 rng(20261204);
    pairs(rng, npairs);
    for (int r = 0; r < nrows; ++r) row(rng, 5000, r % 3);
    std::printf("pairs %llu fast %llu\n", n_pairs, n_fast);
    std::printf("chunks %llu repeated %llu\n", n_chunks, n_repeat);
    std::printf("mismatches %llu\n", n_bad);
    return n_bad != 0;
}

// sl_outcome.cpp -- outcome of one projectile-target collision from its final
// state (include/spacelab_host.h, slh_collision_outcome).
//
// The reference records no outcome (its `bound` column is always written as
// 0, ball_group.hpp:496,502, and get_radius is a maximum distance,
// ball_group.hpp:377-391), so the definitions are this project's:
//   remnants      connected components of the graph linking spheres whose
//                 surface gap R_i + R_j - |r_ij| > -bond_gap (touching, or
//                 within bond_gap of touching);
//   largest       the component of largest mass; largest_fraction = its
//                 mass / total mass;
//   stuck         projectile mass (spheres [n_t, n)) in the largest
//                 component / projectile mass;
//   rg            radius of gyration of the largest component,
//                 sqrt(sum m |r - r_cm|^2 / sum m);
// Components are found with a uniform cell grid (cell = 2 max R + bond_gap)
// and union-find, O(n) for bounded density.
#include "../../../include/spacelab_host.h"

#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <vector>

namespace {

struct DSU {
    std::vector<int> p;
    explicit DSU(int n) : p(n) { for (int i = 0; i < n; ++i) p[i] = i; }
    int find(int x)
    {
        while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
        return x;
    }
    void unite(int a, int b)
    {
        a = find(a); b = find(b);
        if (a != b) p[a < b ? b : a] = a < b ? a : b;
    }
};

}  // namespace

extern "C" int slh_collision_outcome(int n, int n_t, const double* pos, const double* R, const double* m,
                                     double bond_gap, double* largest_fraction, double* stuck_fraction, double* rg,
                                     int* n_components)
{
    if (n < 1 || n_t < 0 || n_t > n || !pos || !R || !m || bond_gap < 0) return 1;
    double rmax = 0, lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL};
    for (int i = 0; i < n; ++i) {
        rmax = std::max(rmax, R[i]);
        for (int c = 0; c < 3; ++c) lo[c] = std::min(lo[c], pos[3 * i + c]);
    }
    const double cell = 2 * rmax + bond_gap;
    auto key = [&](long long x, long long y, long long z) { return (x * 73856093LL) ^ (y * 19349663LL) ^ (z * 83492791LL); };
    std::unordered_map<long long, std::vector<int>> grid;
    grid.reserve(n * 2);
    std::vector<long long> cx(n), cy(n), cz(n);
    for (int i = 0; i < n; ++i) {
        cx[i] = (long long)std::floor((pos[3 * i] - lo[0]) / cell);
        cy[i] = (long long)std::floor((pos[3 * i + 1] - lo[1]) / cell);
        cz[i] = (long long)std::floor((pos[3 * i + 2] - lo[2]) / cell);
        grid[key(cx[i], cy[i], cz[i])].push_back(i);
    }
    DSU d(n);
    for (int i = 0; i < n; ++i)
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    auto it = grid.find(key(cx[i] + dx, cy[i] + dy, cz[i] + dz));
                    if (it == grid.end()) continue;
                    for (int j : it->second) {
                        if (j <= i || cx[j] != cx[i] + dx || cy[j] != cy[i] + dy || cz[j] != cz[i] + dz) continue;
                        const double ex = pos[3 * j] - pos[3 * i], ey = pos[3 * j + 1] - pos[3 * i + 1],
                                     ez = pos[3 * j + 2] - pos[3 * i + 2];
                        const double lim = R[i] + R[j] + bond_gap;
                        if (ex * ex + ey * ey + ez * ez < lim * lim) d.unite(i, j);
                    }
                }
    std::vector<double> mass(n, 0.0);
    double mt = 0, mp = 0;
    int comps = 0;
    for (int i = 0; i < n; ++i) {
        const int r = d.find(i);
        if (r == i) ++comps;
        mass[r] += m[i];
        mt += m[i];
        if (i >= n_t) mp += m[i];
    }
    int big = 0;
    for (int i = 0; i < n; ++i)
        if (mass[i] > mass[big]) big = i;
    double stuck = 0, cm[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
        if (d.find(i) == big) {
            if (i >= n_t) stuck += m[i];
            for (int c = 0; c < 3; ++c) cm[c] += m[i] * pos[3 * i + c];
        }
    for (double& c : cm) c /= mass[big];
    double s2 = 0;
    for (int i = 0; i < n; ++i)
        if (d.find(i) == big)
            for (int c = 0; c < 3; ++c) {
                const double e = pos[3 * i + c] - cm[c];
                s2 += m[i] * e * e;
            }
    if (largest_fraction) *largest_fraction = mass[big] / mt;
    if (stuck_fraction) *stuck_fraction = mp > 0 ? stuck / mp : 0.0;
    if (rg) *rg = std::sqrt(s2 / mass[big]);
    if (n_components) *n_components = comps;
    return 0;
}

extern "C" int slh_radius_of_gyration(int n, const double* pos, const double* m, double* rg)
{
    if (n < 1 || !pos || !m || !rg) return 1;
    double mt = 0, cm[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
        mt += m[i];
        for (int c = 0; c < 3; ++c) cm[c] += m[i] * pos[3 * i + c];
    }
    for (double& c : cm) c /= mt;
    double s2 = 0;
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            const double e = pos[3 * i + c] - cm[c];
            s2 += m[i] * e * e;
        }
    *rg = std::sqrt(s2 / mt);
    return 0;
}

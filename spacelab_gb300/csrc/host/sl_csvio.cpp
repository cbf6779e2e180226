// sl_csvio.cpp -- the reference's output/continue file formats and an exact
// binary checkpoint (include/spacelab_host.h).
//
// Formats (reference files, paths inside the SpaceLab project):
//   <prefix>simData.csv    header x0,y0,z0,wx0,wy0,wz0,wmag0,vx0,vy0,vz0,bound0,
//                          x1,... (ball_group.hpp:463-472), then one row per
//                          write step, each row preceded by '\n' and holding
//                          11 values per sphere: pos, w, |w|, vel, bound = 0
//                          (ColliderSingleCore.cpp:259,268-280)
//   <prefix>energy.csv     header Time,PE,KE,E,p,L (ball_group.hpp:462), rows
//                          '\n' + time,PE,KE,PE+KE,|mom|,|ang_mom| written at
//                          12 significant digits (ColliderSingleCore.cpp:42,
//                          335-338)
//   <prefix>constants.csv  R,m,moi per sphere, one line each
//                          (ball_group.hpp:475-477)
// Values are written as an ostream with the given precision writes them
// (printf %.*g); the reference uses the default precision 6 for simData and
// constants, so its files do not round-trip exactly -- pass 17 for files that
// do.  Continue semantics follow getLastLine / parseSimData / loadConsts
// (ball_group.hpp:979-1077): the state is the LAST row of simData, the sphere
// count is (commas / 11) + 1.  Unlike the reference, a trailing newline after
// the last row is accepted.
#include "../../../include/spacelab_host.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr int kProperties = 11;  // columns per sphere (dust_const.hpp:44)

void put_num(std::string& s, double x, int precision)
{
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.*g", precision, x);
    s += buf;
}

int append_text(const char* path, const std::string& text, const char* mode)
{
    FILE* f = std::fopen(path, mode);
    if (!f) return 3;
    const size_t w = std::fwrite(text.data(), 1, text.size(), f);
    const int rc = std::fclose(f);
    return (w == text.size() && rc == 0) ? 0 : 3;
}

int read_file(const char* path, std::string& out)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return 3;
    std::vector<char> buf(1 << 16);
    out.clear();
    size_t r;
    while ((r = std::fread(buf.data(), 1, buf.size(), f)) > 0) out.append(buf.data(), r);
    std::fclose(f);
    return 0;
}

// Last non-empty line (trailing '\n' and '\r' tolerated).
std::string last_line(const std::string& text)
{
    size_t end = text.size();
    while (end > 0 && (text[end - 1] == '\n' || text[end - 1] == '\r')) --end;
    const size_t beg = text.rfind('\n', end == 0 ? 0 : end - 1);
    return text.substr(beg == std::string::npos ? 0 : beg + 1, end - (beg == std::string::npos ? 0 : beg + 1));
}

bool parse_fields(const std::string& line, std::vector<double>& out)
{
    out.clear();
    const char* p = line.c_str();
    while (*p) {
        char* e = nullptr;
        errno = 0;
        const double v = std::strtod(p, &e);
        if (e == p || errno == ERANGE) return false;
        out.push_back(v);
        p = e;
        while (*p == ' ' || *p == '\r') ++p;
        if (*p == ',') ++p;
        else if (*p) return false;
    }
    return true;
}

struct CkptHeader {
    char magic[8];
    int32_t version;
    int32_t n;
    double dt, kin, kout, sim_time;
    int64_t step;
};
constexpr char kMagic[8] = {'S', 'L', 'C', 'K', 'P', 'T', '0', '1'};

}  // namespace

extern "C" {

int slh_write_simdata_header(const char* path, int n)
{
    if (!path || n < 1) return 1;
    std::string s = "x0,y0,z0,wx0,wy0,wz0,wmag0,vx0,vy0,vz0,bound0";
    static const char* cols[kProperties] = {"x", "y", "z", "wx", "wy", "wz", "wmag", "vx", "vy", "vz", "bound"};
    for (int b = 1; b < n; ++b)
        for (const char* c : cols) {
            s += ',';
            s += c;
            s += std::to_string(b);
        }
    return append_text(path, s, "wb");
}

int slh_append_simdata_row(const char* path, int n, const double* pos, const double* w, const double* vel,
                           int precision)
{
    if (!path || n < 1 || !pos || !w || !vel || precision < 1 || precision > 17) return 1;
    std::string s = "\n";
    s.reserve((size_t)n * kProperties * (precision + 8));
    for (int b = 0; b < n; ++b) {
        if (b) s += ',';
        const double* p = pos + 3 * (size_t)b;
        const double* o = w + 3 * (size_t)b;
        const double* v = vel + 3 * (size_t)b;
        const double wmag = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);  // vec3::norm
        const double vals[10] = {p[0], p[1], p[2], o[0], o[1], o[2], wmag, v[0], v[1], v[2]};
        for (int k = 0; k < 10; ++k) {
            put_num(s, vals[k], precision);
            s += ',';
        }
        s += '0';  // bound (always written as 0, ball_group.hpp:496,502)
    }
    return append_text(path, s, "ab");
}

int slh_write_energy_header(const char* path)
{
    if (!path) return 1;
    return append_text(path, "Time,PE,KE,E,p,L", "wb");
}

int slh_append_energy_row(const char* path, double time, double PE, double KE, double p, double L, int precision)
{
    if (!path || precision < 1 || precision > 17) return 1;
    std::string s = "\n";
    const double vals[6] = {time, PE, KE, PE + KE, p, L};
    for (int k = 0; k < 6; ++k) {
        if (k) s += ',';
        put_num(s, vals[k], precision);
    }
    return append_text(path, s, "ab");
}

int slh_write_constants(const char* path, int n, const double* R, const double* m, const double* moi, int precision)
{
    if (!path || n < 1 || !R || !m || !moi || precision < 1 || precision > 17) return 1;
    std::string s;
    for (int b = 0; b < n; ++b) {
        put_num(s, R[b], precision);
        s += ',';
        put_num(s, m[b], precision);
        s += ',';
        put_num(s, moi[b], precision);
        s += '\n';
    }
    return append_text(path, s, "wb");
}

int slh_count_last_state(const char* simdata_path, int* n)
{
    if (!simdata_path || !n) return 1;
    std::string text;
    if (read_file(simdata_path, text)) return 3;
    const std::string line = last_line(text);
    if (line.empty()) return 4;
    long commas = 0;
    for (char c : line) commas += (c == ',');
    *n = (int)(commas / kProperties + 1);  // parseSimData, ball_group.hpp:984
    return 0;
}

int slh_read_last_state(const char* simdata_path, int n, double* pos, double* vel, double* w)
{
    if (!simdata_path || n < 1 || !pos || !vel || !w) return 1;
    std::string text;
    if (read_file(simdata_path, text)) return 3;
    std::vector<double> f;
    if (!parse_fields(last_line(text), f)) return 4;
    if ((long)f.size() != (long)n * kProperties) return 4;
    for (int b = 0; b < n; ++b) {
        const double* r = f.data() + (size_t)b * kProperties;
        for (int c = 0; c < 3; ++c) {
            pos[3 * (size_t)b + c] = r[c];
            w[3 * (size_t)b + c] = r[3 + c];
            vel[3 * (size_t)b + c] = r[7 + c];  // r[6] is |w|, r[10] is bound
        }
    }
    return 0;
}

int slh_read_constants(const char* constants_path, int n, double* R, double* m, double* moi)
{
    if (!constants_path || n < 1 || !R || !m || !moi) return 1;
    std::string text;
    if (read_file(constants_path, text)) return 3;
    size_t pos = 0;
    std::vector<double> f;
    for (int b = 0; b < n; ++b) {
        const size_t nl = text.find('\n', pos);
        if (pos >= text.size()) return 4;
        const std::string line = text.substr(pos, (nl == std::string::npos ? text.size() : nl) - pos);
        if (!parse_fields(line, f) || f.size() != 3) return 4;
        R[b] = f[0]; m[b] = f[1]; moi[b] = f[2];
        pos = (nl == std::string::npos) ? text.size() : nl + 1;
    }
    return 0;
}

int slh_write_checkpoint(const char* path, int n, const double* pos, const double* vel, const double* w,
                         const double* acc, const double* aacc, const double* pos_prev, const double* R,
                         const double* m, const double* moi, double dt, double kin, double kout, double sim_time,
                         long long step)
{
    if (!path || n < 1 || !pos || !vel || !w || !acc || !aacc || !pos_prev || !R || !m || !moi) return 1;
    CkptHeader h{};
    std::memcpy(h.magic, kMagic, 8);
    h.version = 1; h.n = n; h.dt = dt; h.kin = kin; h.kout = kout; h.sim_time = sim_time; h.step = step;
    FILE* f = std::fopen(path, "wb");
    if (!f) return 3;
    bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
    const double* v3[6] = {pos, vel, w, acc, aacc, pos_prev};
    for (const double* a : v3) ok = ok && std::fwrite(a, sizeof(double), 3 * (size_t)n, f) == 3 * (size_t)n;
    const double* s1[3] = {R, m, moi};
    for (const double* a : s1) ok = ok && std::fwrite(a, sizeof(double), (size_t)n, f) == (size_t)n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? 0 : 3;
}

int slh_read_checkpoint_header(const char* path, int* n, double* dt, double* kin, double* kout, double* sim_time,
                               long long* step)
{
    if (!path || !n) return 1;
    FILE* f = std::fopen(path, "rb");
    if (!f) return 3;
    CkptHeader h{};
    const bool ok = std::fread(&h, sizeof h, 1, f) == 1;
    std::fclose(f);
    if (!ok || std::memcmp(h.magic, kMagic, 8) != 0 || h.version != 1 || h.n < 1) return 4;
    *n = h.n;
    if (dt) *dt = h.dt;
    if (kin) *kin = h.kin;
    if (kout) *kout = h.kout;
    if (sim_time) *sim_time = h.sim_time;
    if (step) *step = h.step;
    return 0;
}

int slh_read_checkpoint(const char* path, int n, double* pos, double* vel, double* w, double* acc, double* aacc,
                        double* pos_prev, double* R, double* m, double* moi)
{
    if (!path || n < 1 || !pos || !vel || !w || !acc || !aacc || !pos_prev || !R || !m || !moi) return 1;
    FILE* f = std::fopen(path, "rb");
    if (!f) return 3;
    CkptHeader h{};
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 && std::memcmp(h.magic, kMagic, 8) == 0 && h.version == 1 &&
              h.n == n;
    double* v3[6] = {pos, vel, w, acc, aacc, pos_prev};
    for (double* a : v3) ok = ok && std::fread(a, sizeof(double), 3 * (size_t)n, f) == 3 * (size_t)n;
    double* s1[3] = {R, m, moi};
    for (double* a : s1) ok = ok && std::fread(a, sizeof(double), (size_t)n, f) == (size_t)n;
    std::fclose(f);
    return ok ? 0 : 4;
}

}  // extern "C"

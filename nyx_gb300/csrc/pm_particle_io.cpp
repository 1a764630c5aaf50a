// The particle directories of Nyx's checkpoints and plotfiles ("DM" inside
// chkNNNNN/ and pltNNNNN/): the AMReX particle container layout of
// Version_Two_Dot_Zero, which Nyx writes through NyxCheckpoint / WriteNyxPlotFile
// (Source/Particle/NyxParticleContainer.H:499-517, called from
// Source/IO/Nyx_output.cpp:646-680, 726-750) and reads back through Restart
// (Source/Particle/NyxParticles.cpp:584-586, 928-934).  The layout, as the
// reference's own reader Util/Converters/plotfile2HDF5_particles_amr.py:24-111
// parses it:
//
//   <dir>/Header (text, one item per line)
//     Version_Two_Dot_Zero_double | Version_Two_Dot_Zero_single  (real precision)
//     3                                   space dimension
//     NR, then NR names                   real components after the position
//                                         (Nyx DM: mass xvel yvel zvel,
//                                         Source/Particle/DarkMatterParticleContainer.H:14-18)
//     NI, then NI names                   int components after id and cpu
//     1 | 0                               checkpoint (ids stored) or plotfile
//     number of particles
//     the next particle id to hand out
//     finest level
//     one grid count per level
//     one "file count offset" line per grid, level by level
//   <dir>/Level_<l>/DATA_<file, 5 digits> (binary, native byte order), per grid at
//     its offset: a checkpoint's count x (2 + NI) int32 (id, cpu, ...), then
//     count x (3 + NR) reals (x y z and the NR components), particle by particle
//   <dir>/Level_<l>/Particle_H          the level's particle BoxArray (text)
//
// The writer produces one level with one grid covering the periodic domain:
// ids 1..np, cpu 0, the Nyx DM components.  The reader takes every grid of every
// level in header order, finds mass and the three velocities by name (by
// position when the names are not Nyx's), and skips other components.
#include "../../include/nyxpm.h"

#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace {

nyxpm_status pio_fail(char* errbuf, size_t errlen, const std::string& msg)
{
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", msg.c_str());
    return NYXPM_INVALID_ARG;
}

const char* kVersionDouble = "Version_Two_Dot_Zero_double";
const char* kVersionSingle = "Version_Two_Dot_Zero_single";
const char* kDmNames[4] = {"mass", "xvel", "yvel", "zvel"};

struct Grid {
    int level;
    long long which, count, where;
};

struct Header {
    bool single = false;
    int dim = 0;
    std::vector<std::string> real_names, int_names;
    int is_checkpoint = 0;
    long long num_particles = 0, max_next_id = 0;
    int finest_level = 0;
    std::vector<Grid> grids;
};

bool next_line(std::istream& in, std::string* s)
{
    if (!std::getline(in, *s)) return false;
    while (!s->empty() && (s->back() == '\r' || s->back() == ' ' || s->back() == '\t')) s->pop_back();
    size_t b = 0;
    while (b < s->size() && ((*s)[b] == ' ' || (*s)[b] == '\t')) ++b;
    s->erase(0, b);
    return true;
}

bool parse_ll(const std::string& s, long long* v)
{
    if (s.empty()) return false;
    char* end = nullptr;
    errno = 0;
    const long long x = std::strtoll(s.c_str(), &end, 10);
    if (errno != 0 || end == s.c_str() || *end != '\0') return false;
    *v = x;
    return true;
}

nyxpm_status read_header(const std::string& dir, Header* h, char* errbuf, size_t errlen)
{
    const std::string path = dir + "/Header";
    std::ifstream in(path);
    if (!in) return pio_fail(errbuf, errlen, "cannot open " + path);
    const std::string bad = path + ": ";
    std::string s;
    long long v = 0;
    if (!next_line(in, &s)) return pio_fail(errbuf, errlen, bad + "empty");
    if (s == kVersionDouble) {
        h->single = false;
    } else if (s == kVersionSingle) {
        h->single = true;
    } else {
        return pio_fail(errbuf, errlen, bad + "version '" + s + "' (Version_Two_Dot_Zero_double or _single expected)");
    }
    if (!next_line(in, &s) || !parse_ll(s, &v) || v != 3) return pio_fail(errbuf, errlen, bad + "dimension must be 3");
    h->dim = 3;
    if (!next_line(in, &s) || !parse_ll(s, &v) || v < 0 || v > 1024)
        return pio_fail(errbuf, errlen, bad + "number of real components");
    h->real_names.resize((size_t)v);
    for (auto& nm : h->real_names)
        if (!next_line(in, &nm)) return pio_fail(errbuf, errlen, bad + "real component names");
    if (!next_line(in, &s) || !parse_ll(s, &v) || v < 0 || v > 1024)
        return pio_fail(errbuf, errlen, bad + "number of int components");
    h->int_names.resize((size_t)v);
    for (auto& nm : h->int_names)
        if (!next_line(in, &nm)) return pio_fail(errbuf, errlen, bad + "int component names");
    if (!next_line(in, &s) || !parse_ll(s, &v) || (v != 0 && v != 1))
        return pio_fail(errbuf, errlen, bad + "checkpoint flag");
    h->is_checkpoint = (int)v;
    if (!next_line(in, &s) || !parse_ll(s, &h->num_particles) || h->num_particles < 0)
        return pio_fail(errbuf, errlen, bad + "particle count");
    if (!next_line(in, &s) || !parse_ll(s, &h->max_next_id)) return pio_fail(errbuf, errlen, bad + "next id");
    if (!next_line(in, &s) || !parse_ll(s, &v) || v < 0 || v > 64) return pio_fail(errbuf, errlen, bad + "finest level");
    h->finest_level = (int)v;
    std::vector<long long> ngrids(h->finest_level + 1);
    for (auto& g : ngrids)
        if (!next_line(in, &s) || !parse_ll(s, &g) || g < 0) return pio_fail(errbuf, errlen, bad + "grid counts");
    long long total = 0;
    for (int lev = 0; lev <= h->finest_level; ++lev) {
        for (long long gi = 0; gi < ngrids[lev]; ++gi) {
            if (!next_line(in, &s)) return pio_fail(errbuf, errlen, bad + "grid table");
            std::istringstream ls(s);
            Grid g{lev, 0, 0, 0};
            std::string extra;
            if (!(ls >> g.which >> g.count >> g.where) || (ls >> extra) || g.which < 0 || g.count < 0 ||
                g.where < 0)
                return pio_fail(errbuf, errlen, bad + "grid line '" + s + "'");
            total += g.count;
            h->grids.push_back(g);
        }
    }
    if (total != h->num_particles)
        return pio_fail(errbuf, errlen, bad + "the grids hold " + std::to_string(total) +
                                            " particles, the header says " + std::to_string(h->num_particles));
    return NYXPM_OK;
}

std::string data_file(const std::string& dir, int level, long long which)
{
    char name[64];
    std::snprintf(name, sizeof(name), "/Level_%d/DATA_%05lld", level, which);
    return dir + name;
}

bool make_dir(const std::string& d)
{
    if (::mkdir(d.c_str(), 0755) == 0) return true;
    struct stat st;
    return errno == EEXIST && ::stat(d.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

}  // namespace

extern "C" {

nyxpm_status nyxpm_particles_info(const char* dir, nyxpm_particle_header* out, char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!dir || !out) return pio_fail(errbuf, errlen, "null argument");
    Header h;
    const nyxpm_status st = read_header(dir, &h, errbuf, errlen);
    if (st != NYXPM_OK) return st;
    out->single_precision = h.single ? 1 : 0;
    out->dim = h.dim;
    out->n_real_extra = (int)h.real_names.size();
    out->n_int_extra = (int)h.int_names.size();
    out->is_checkpoint = h.is_checkpoint;
    out->num_particles = h.num_particles;
    out->max_next_id = h.max_next_id;
    out->finest_level = h.finest_level;
    out->ngrids = (int)h.grids.size();
    return NYXPM_OK;
}

nyxpm_status nyxpm_particles_read(const char* dir, int64_t capacity, double* pos, double* vel, double* mass,
                                  int64_t* ids, int64_t* np_read, char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!dir || !pos || !vel || !mass) return pio_fail(errbuf, errlen, "null argument");
    Header h;
    nyxpm_status st = read_header(dir, &h, errbuf, errlen);
    if (st != NYXPM_OK) return st;
    if (h.num_particles > capacity)
        return pio_fail(errbuf, errlen, std::string(dir) + " holds " + std::to_string(h.num_particles) +
                                            " particles, more than the arrays' " + std::to_string(capacity));
    if (ids && !h.is_checkpoint)
        return pio_fail(errbuf, errlen, std::string(dir) + " is a plotfile's: no particle ids stored");
    // the Nyx DM components by name, else the first four in Nyx's order
    const int nr = (int)h.real_names.size();
    int col[4];
    bool by_name = true;
    for (int c = 0; c < 4; ++c) {
        col[c] = -1;
        for (int r = 0; r < nr; ++r)
            if (h.real_names[r] == kDmNames[c]) col[c] = r;
        by_name = by_name && col[c] >= 0;
    }
    if (!by_name) {
        if (nr < 4)
            return pio_fail(errbuf, errlen, std::string(dir) + ": fewer than 4 real components (mass, xvel, yvel, zvel)");
        for (int c = 0; c < 4; ++c) col[c] = c;
    }
    const int nints = h.is_checkpoint ? 2 + (int)h.int_names.size() : 0;
    const int nreals = 3 + nr;
    const size_t rsize = h.single ? 4 : 8;
    std::vector<unsigned char> rbuf;
    std::vector<int32_t> ibuf;
    long long got = 0;
    for (const Grid& g : h.grids) {
        if (g.count == 0) continue;
        const std::string path = data_file(dir, g.level, g.which);
        FILE* f = std::fopen(path.c_str(), "rb");
        if (!f) return pio_fail(errbuf, errlen, "cannot open " + path);
        bool ok = std::fseek(f, (long)g.where, SEEK_SET) == 0;
        ibuf.resize((size_t)g.count * nints);
        rbuf.resize((size_t)g.count * nreals * rsize);
        if (ok && nints) ok = std::fread(ibuf.data(), sizeof(int32_t), ibuf.size(), f) == ibuf.size();
        if (ok) ok = std::fread(rbuf.data(), 1, rbuf.size(), f) == rbuf.size();
        std::fclose(f);
        if (!ok) return pio_fail(errbuf, errlen, path + ": short read at offset " + std::to_string(g.where));
        for (long long q = 0; q < g.count; ++q) {
            double r[3 + 1024];
            for (int c = 0; c < nreals; ++c) {
                const unsigned char* src = rbuf.data() + ((size_t)q * nreals + c) * rsize;
                if (h.single) {
                    float x;
                    std::memcpy(&x, src, 4);
                    r[c] = x;
                } else {
                    std::memcpy(&r[c], src, 8);
                }
            }
            const long long p = got + q;
            for (int d = 0; d < 3; ++d) {
                pos[3 * p + d] = r[d];
                vel[3 * p + d] = r[3 + col[1 + d]];
            }
            mass[p] = r[3 + col[0]];
            if (ids) ids[p] = ibuf[(size_t)q * nints];
        }
        got += g.count;
    }
    if (np_read) *np_read = got;
    return NYXPM_OK;
}

nyxpm_status nyxpm_particles_write(const char* dir, int n, int64_t np, const double* pos, const double* vel,
                                   const double* mass, double mass_scalar, int is_checkpoint,
                                   int single_precision, char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!dir || !pos || !vel || np < 0 || n < 1) return pio_fail(errbuf, errlen, "bad argument");
    if (is_checkpoint && np > 2147483646LL)
        return pio_fail(errbuf, errlen, "a checkpoint's particle ids are int32: too many particles");
    const std::string d(dir), lev = d + "/Level_0";
    if (!make_dir(d) || !make_dir(lev)) return pio_fail(errbuf, errlen, "cannot create " + lev);
    // the data: one grid, ids and cpus first (checkpoint), then the reals
    const std::string data = data_file(d, 0, 0);
    FILE* f = std::fopen(data.c_str(), "wb");
    if (!f) return pio_fail(errbuf, errlen, "cannot write " + data);
    bool ok = true;
    const int64_t block = 1 << 16;
    if (is_checkpoint) {
        std::vector<int32_t> ib;
        for (int64_t q0 = 0; q0 < np && ok; q0 += block) {
            const int64_t q1 = std::min<int64_t>(np, q0 + block);
            ib.resize(2 * (size_t)(q1 - q0));
            for (int64_t q = q0; q < q1; ++q) {
                ib[2 * (q - q0)] = (int32_t)(q + 1);
                ib[2 * (q - q0) + 1] = 0;
            }
            ok = std::fwrite(ib.data(), sizeof(int32_t), ib.size(), f) == ib.size();
        }
    }
    std::vector<double> rd;
    std::vector<float> rf;
    for (int64_t q0 = 0; q0 < np && ok; q0 += block) {
        const int64_t q1 = std::min<int64_t>(np, q0 + block);
        rd.resize(7 * (size_t)(q1 - q0));
        for (int64_t q = q0; q < q1; ++q) {
            double* r = rd.data() + 7 * (q - q0);
            r[0] = pos[3 * q];
            r[1] = pos[3 * q + 1];
            r[2] = pos[3 * q + 2];
            r[3] = mass ? mass[q] : mass_scalar;
            r[4] = vel[3 * q];
            r[5] = vel[3 * q + 1];
            r[6] = vel[3 * q + 2];
        }
        if (single_precision) {
            rf.assign(rd.begin(), rd.end());
            ok = std::fwrite(rf.data(), sizeof(float), rf.size(), f) == rf.size();
        } else {
            ok = std::fwrite(rd.data(), sizeof(double), rd.size(), f) == rd.size();
        }
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) return pio_fail(errbuf, errlen, "write failed: " + data);
    std::ofstream hdr(d + "/Header");
    hdr << (single_precision ? kVersionSingle : kVersionDouble) << '\n' << 3 << '\n' << 4 << '\n';
    for (const char* nm : kDmNames) hdr << nm << '\n';
    hdr << 0 << '\n' << (is_checkpoint ? 1 : 0) << '\n' << np << '\n' << np + 1 << '\n' << 0 << '\n'
        << 1 << '\n' << 0 << ' ' << np << ' ' << 0 << '\n';
    hdr.close();
    std::ofstream ph(lev + "/Particle_H");
    ph << "(1 0\n((0,0,0) (" << n - 1 << ',' << n - 1 << ',' << n - 1 << ") (0,0,0))\n)\n";
    ph.close();
    if (!hdr || !ph) return pio_fail(errbuf, errlen, "write failed: " + d + "/Header");
    return NYXPM_OK;
}

}  // extern "C"

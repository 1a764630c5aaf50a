// Host-side file formats of the path: Nyx's particle initial-condition files
// and the comoving_a file of a checkpoint or plotfile.
//
// Particle files (formats of Docs/sphinx_documentation/source/ICs.rst:13-78,
// read by Nyx::init_particles, Source/Particle/NyxParticles.cpp:506-560):
//   AsciiFile       first line: the particle count; then one line per particle
//                   "x y z mass vx vy vz".
//   BinaryFile      header: int64 NP, int32 DM (= 3), int32 NX (extra fields,
//                   at least 4); then NP records of DM + NX values
//                   "x y z mass vx vy vz [more extras, skipped]", float32 or
//                   float64 (told apart by the file size); native byte order.
//   BinaryMetaFile  a text file listing binary particle files, one path per
//                   line, read in the order listed.
// comoving_a: one number written with 15 significant digits
// (Source/IO/Nyx_output.cpp:994-1010) and read back at restart
// (Source/Driver/comoving.cpp:690-705).
//
// Readers fill the AoS host arrays nyxpm_box_upload takes: pos[3 np],
// vel[3 np], mass[np].
#include "../../include/nyxpm.h"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

nyxpm_status io_fail(char* errbuf, size_t errlen, const std::string& msg)
{
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", msg.c_str());
    return NYXPM_INVALID_ARG;
}

bool read_all(const char* path, std::string& out)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    out.clear();
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, got);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

// the next number of a text buffer, skipping white space; false at the end or
// on text that is not a number
bool next_number(const char*& p, const char* end, double* v)
{
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    if (p >= end) return false;
    char* stop = nullptr;
    errno = 0;
    *v = std::strtod(p, &stop);
    if (stop == p || errno == ERANGE) return false;
    p = stop;
    return true;
}

struct BinHeader {
    int64_t np = 0;
    int32_t dm = 0, nx = 0;
};

bool read_bin_header(FILE* f, BinHeader* h)
{
    return std::fread(&h->np, sizeof(h->np), 1, f) == 1 && std::fread(&h->dm, sizeof(h->dm), 1, f) == 1 &&
           std::fread(&h->nx, sizeof(h->nx), 1, f) == 1;
}

nyxpm_status bin_header(const char* path, BinHeader* h, char* errbuf, size_t errlen)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return io_fail(errbuf, errlen, std::string("cannot open ") + path);
    const bool ok = read_bin_header(f, h);
    std::fclose(f);
    if (!ok) return io_fail(errbuf, errlen, std::string("short header in ") + path);
    if (h->np < 0 || h->dm != 3 || h->nx < 4)
        return io_fail(errbuf, errlen, std::string("unsupported header in ") + path +
                                           " (want NP >= 0, DM = 3, NX >= 4)");
    return NYXPM_OK;
}

// the binary files a BinaryMetaFile lists
nyxpm_status meta_list(const char* path, std::vector<std::string>* files, char* errbuf, size_t errlen)
{
    std::string txt;
    if (!read_all(path, txt)) return io_fail(errbuf, errlen, std::string("cannot read ") + path);
    files->clear();
    size_t i = 0;
    while (i < txt.size()) {
        size_t e = txt.find('\n', i);
        if (e == std::string::npos) e = txt.size();
        std::string line = txt.substr(i, e - i);
        while (!line.empty() && (line.back() == '\r' || line.back() == ' ' || line.back() == '\t'))
            line.pop_back();
        size_t s = 0;
        while (s < line.size() && (line[s] == ' ' || line[s] == '\t')) ++s;
        if (s < line.size()) files->push_back(line.substr(s));
        i = e + 1;
    }
    return NYXPM_OK;
}

}  // namespace

extern "C" {

nyxpm_status nyxpm_particle_file_count(const char* path, nyxpm_file_format fmt, int64_t* np,
                                       char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!path || !np) return io_fail(errbuf, errlen, "null argument");
    *np = 0;
    if (fmt == NYXPM_FILE_ASCII) {
        FILE* f = std::fopen(path, "rb");
        if (!f) return io_fail(errbuf, errlen, std::string("cannot open ") + path);
        char line[256] = {0};
        const bool ok = std::fgets(line, sizeof(line), f) != nullptr;
        std::fclose(f);
        char* stop = nullptr;
        const long long v = ok ? std::strtoll(line, &stop, 10) : -1;
        if (!ok || stop == line || v < 0) return io_fail(errbuf, errlen, std::string("no particle count in ") + path);
        *np = v;
        return NYXPM_OK;
    }
    if (fmt == NYXPM_FILE_BINARY || fmt == NYXPM_FILE_BINARY_F64) {
        BinHeader h;
        const nyxpm_status st = bin_header(path, &h, errbuf, errlen);
        if (st == NYXPM_OK) *np = h.np;
        return st;
    }
    if (fmt == NYXPM_FILE_BINARY_META) {
        std::vector<std::string> files;
        nyxpm_status st = meta_list(path, &files, errbuf, errlen);
        if (st != NYXPM_OK) return st;
        int64_t total = 0;
        for (const auto& fn : files) {
            BinHeader h;
            if ((st = bin_header(fn.c_str(), &h, errbuf, errlen)) != NYXPM_OK) return st;
            total += h.np;
        }
        *np = total;
        return NYXPM_OK;
    }
    return io_fail(errbuf, errlen, "unknown particle file format");
}

nyxpm_status nyxpm_particle_file_read(const char* path, nyxpm_file_format fmt, int64_t capacity,
                                      double* pos, double* vel, double* mass, int64_t* np_read,
                                      char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!path || !pos || !vel || !mass || !np_read) return io_fail(errbuf, errlen, "null argument");
    *np_read = 0;
    int64_t np = 0;
    nyxpm_status st = nyxpm_particle_file_count(path, fmt, &np, errbuf, errlen);
    if (st != NYXPM_OK) return st;
    if (np > capacity)
        return io_fail(errbuf, errlen, "the file holds " + std::to_string(np) +
                                           " particles, more than the arrays' capacity " +
                                           std::to_string(capacity));
    if (fmt == NYXPM_FILE_ASCII) {
        std::string txt;
        if (!read_all(path, txt)) return io_fail(errbuf, errlen, std::string("cannot read ") + path);
        const char* p = txt.data();
        const char* end = p + txt.size();
        while (p < end && *p != '\n') ++p;   // the count line
        for (int64_t q = 0; q < np; ++q) {
            double v[7];
            for (int c = 0; c < 7; ++c)
                if (!next_number(p, end, &v[c]))
                    return io_fail(errbuf, errlen, "particle " + std::to_string(q) + " of " + path +
                                                       " is incomplete or not numeric");
            pos[3 * q] = v[0];
            pos[3 * q + 1] = v[1];
            pos[3 * q + 2] = v[2];
            mass[q] = v[3];
            vel[3 * q] = v[4];
            vel[3 * q + 1] = v[5];
            vel[3 * q + 2] = v[6];
        }
        *np_read = np;
        return NYXPM_OK;
    }
    std::vector<std::string> files;
    if (fmt == NYXPM_FILE_BINARY || fmt == NYXPM_FILE_BINARY_F64) {
        files.push_back(path);
    } else if ((st = meta_list(path, &files, errbuf, errlen)) != NYXPM_OK) {
        return st;
    }
    int64_t q = 0;
    for (const auto& fn : files) {
        FILE* f = std::fopen(fn.c_str(), "rb");
        if (!f) return io_fail(errbuf, errlen, "cannot open " + fn);
        BinHeader h;
        if (!read_bin_header(f, &h) || h.np < 0 || h.dm != 3 || h.nx < 4 || q + h.np > capacity) {
            std::fclose(f);
            return io_fail(errbuf, errlen, "bad header in " + fn);
        }
        const int rec = h.dm + h.nx;
        // the record precision follows from the file size: DM + NX float32 or float64
        // values per particle (the ICs doc writes floats; Exec/LyA/32.nyx holds doubles)
        long long data_bytes = -1;
        if (std::fseek(f, 0, SEEK_END) == 0) data_bytes = (long long)std::ftell(f) - 16;
        std::fseek(f, 16, SEEK_SET);
        int width = 0;
        if (data_bytes == h.np * rec * 4LL) width = 4;
        else if (data_bytes == h.np * rec * 8LL) width = 8;
        if (width == 0 && h.np > 0) {
            std::fclose(f);
            return io_fail(errbuf, errlen, "size of " + fn + " fits neither float32 nor float64 records");
        }
        std::vector<unsigned char> buf((size_t)rec * width * 65536);
        for (int64_t done = 0; done < h.np;) {
            const int64_t chunk = std::min<int64_t>(65536, h.np - done);
            if (std::fread(buf.data(), (size_t)width * rec, (size_t)chunk, f) != (size_t)chunk) {
                std::fclose(f);
                return io_fail(errbuf, errlen, "short record data in " + fn);
            }
            for (int64_t r = 0; r < chunk; ++r, ++q) {
                double v[7];
                const unsigned char* src = buf.data() + (size_t)width * rec * r;
                for (int c = 0; c < 7; ++c) {
                    if (width == 4) {
                        float x;
                        std::memcpy(&x, src + 4 * c, 4);
                        v[c] = x;
                    } else {
                        std::memcpy(&v[c], src + 8 * c, 8);
                    }
                }
                pos[3 * q] = v[0];
                pos[3 * q + 1] = v[1];
                pos[3 * q + 2] = v[2];
                mass[q] = v[3];
                vel[3 * q] = v[4];
                vel[3 * q + 1] = v[5];
                vel[3 * q + 2] = v[6];
            }
            done += chunk;
        }
        std::fclose(f);
    }
    *np_read = q;
    return NYXPM_OK;
}

nyxpm_status nyxpm_particle_file_write(const char* path, nyxpm_file_format fmt, int64_t np,
                                       const double* pos, const double* vel, const double* mass,
                                       double mass_scalar, char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!path || np < 0 || (np > 0 && (!pos || !vel))) return io_fail(errbuf, errlen, "null argument");
    if (fmt != NYXPM_FILE_ASCII && fmt != NYXPM_FILE_BINARY && fmt != NYXPM_FILE_BINARY_F64)
        return io_fail(errbuf, errlen, "writes AsciiFile or BinaryFile only");
    FILE* f = std::fopen(path, fmt == NYXPM_FILE_ASCII ? "w" : "wb");
    if (!f) return io_fail(errbuf, errlen, std::string("cannot create ") + path);
    bool ok = true;
    if (fmt == NYXPM_FILE_ASCII) {
        ok = std::fprintf(f, "%lld\n", (long long)np) > 0;
        for (int64_t q = 0; ok && q < np; ++q)
            ok = std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", pos[3 * q], pos[3 * q + 1],
                              pos[3 * q + 2], mass ? mass[q] : mass_scalar, vel[3 * q], vel[3 * q + 1],
                              vel[3 * q + 2]) > 0;
    } else {
        const int64_t n64 = np;
        const int32_t dm = 3, nx = 4;
        ok = std::fwrite(&n64, sizeof(n64), 1, f) == 1 && std::fwrite(&dm, sizeof(dm), 1, f) == 1 &&
             std::fwrite(&nx, sizeof(nx), 1, f) == 1;
        for (int64_t q = 0; ok && q < np; ++q) {
            const double d[7] = {pos[3 * q], pos[3 * q + 1], pos[3 * q + 2], mass ? mass[q] : mass_scalar,
                                 vel[3 * q], vel[3 * q + 1], vel[3 * q + 2]};
            if (fmt == NYXPM_FILE_BINARY_F64) {
                ok = std::fwrite(d, sizeof(double), 7, f) == 7;
            } else {
                float v[7];
                for (int c = 0; c < 7; ++c) v[c] = (float)d[c];
                ok = std::fwrite(v, sizeof(float), 7, f) == 7;
            }
        }
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? NYXPM_OK : io_fail(errbuf, errlen, std::string("write failed: ") + path);
}

// ---------------------------------------------------------------------------
// one-particle-per-cell cosmological ICs
// ---------------------------------------------------------------------------
nyxpm_status nyxpm_cosmo_1ppc_particles(int n, double L, const double* disp, const double* vel,
                                        const double* disp_fac, const double* vel_fac, double* pos_out,
                                        double* vel_out)
{
    if (n < 1 || !(L > 0) || !disp || !vel || !disp_fac || !vel_fac || !pos_out || !vel_out)
        return NYXPM_INVALID_ARG;
    const int64_t nc = (int64_t)n * n * n;
    const double dx = L / n;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                const int64_t c = i + (int64_t)n * (j + (int64_t)n * k);
                const int idx[3] = {i, j, k};
                for (int d = 0; d < 3; ++d) {
                    // cell centre, then the displacement (DarkMatterParticleContainer.cpp:376-386)
                    double x = (idx[d] + 0.5) * dx;
                    x = x + disp[d * nc + c] * disp_fac[d];
                    // periodic shift into [0, L)
                    if (x >= L) x = x - L;
                    else if (x < 0.0) x = x + L;
                    if (x >= L || x < 0.0) x = x - L * std::floor(x / L);
                    if (x >= L) x = 0.0;
                    pos_out[3 * c + d] = x;
                    vel_out[3 * c + d] = vel[d * nc + c] * vel_fac[d];
                }
            }
    return NYXPM_OK;
}

nyxpm_status nyxpm_cosmo_ic_factors(const nyxpm_params* p, int source, int n, double L,
                                    double redshift, double* disp_fac, double* vel_fac,
                                    double* particle_mass)
{
    if (!p || n < 1 || !(L > 0) || !disp_fac || !vel_fac || !particle_mass) return NYXPM_INVALID_ARG;
    const double h = p->comoving_h, OmM = p->comoving_OmM;
    // dark matter carries all the matter when there is no hydro (Nyx_initcosmo.cpp:185-208)
    const double rho_m = 3.0 * h * 100.0 * h * 100.0 * OmM / (8.0 * M_PI * p->gconst);
    const double dx = L / n;
    if (source == 0) {              // MUSIC (Nyx_initcosmo.cpp:259-266)
        for (int d = 0; d < 3; ++d) {
            vel_fac[d] = L * h;
            disp_fac[d] = L;
        }
        *particle_mass = rho_m * dx * dx * dx;
    } else if (source == 1) {       // nyx (Nyx_initcosmo.cpp:281-294)
        if (!(redshift > -1.0)) return NYXPM_INVALID_ARG;
        const double a = 1.0 / (1.0 + redshift);
        const double OmL = 1.0 - OmM;
        for (int d = 0; d < 3; ++d) {
            vel_fac[d] = L * a * std::sqrt(OmM / std::pow(a, 3) + OmL) * h * 100.0;
            disp_fac[d] = L;
        }
        *particle_mass = rho_m * (L * L * L) / ((double)n * n * n);
    } else {
        return NYXPM_INVALID_ARG;
    }
    return NYXPM_OK;
}

nyxpm_status nyxpm_write_comoving_a(const char* dir, double a, char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!dir) return io_fail(errbuf, errlen, "null directory");
    const std::string fn = std::string(dir) + "/comoving_a";
    FILE* f = std::fopen(fn.c_str(), "w");
    if (!f) return io_fail(errbuf, errlen, "cannot create " + fn);
    const bool ok = std::fprintf(f, "%.15g\n", a) > 0;
    return (std::fclose(f) == 0 && ok) ? NYXPM_OK : io_fail(errbuf, errlen, "write failed: " + fn);
}

nyxpm_status nyxpm_read_comoving_a(const char* dir, double* a, char* errbuf, size_t errlen)
{
    if (errbuf && errlen) errbuf[0] = '\0';
    if (!dir || !a) return io_fail(errbuf, errlen, "null argument");
    const std::string fn = std::string(dir) + "/comoving_a";
    std::string txt;
    if (!read_all(fn.c_str(), txt)) return io_fail(errbuf, errlen, "cannot read " + fn);
    const char* p = txt.data();
    if (!next_number(p, p + txt.size(), a)) return io_fail(errbuf, errlen, "no number in " + fn);
    return NYXPM_OK;
}

}  // extern "C"

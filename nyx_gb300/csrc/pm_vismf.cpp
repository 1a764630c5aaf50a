// AMReX MultiFab files as VisMF writes them (header version 1), host side.
//
// Nyx reads its cosmological initial conditions as one such MultiFab,
// <initDirName>/Level_0/Cell (Nyx::icReadAndPrepareFab,
// Source/Initialization/Nyx_initcosmo.cpp:15-96, by VisMF::Read); the slices
// of Util/SliceUtils are stored the same way.  A MultiFab <name> is
//   <name>_H   text: the header version (1), the write mode (1), ncomp, ngrow
//              (an int, or an IntVect "(g,g,g)" in later writers), the
//              BoxArray "(N 0" with one "((lx,ly,lz) (hx,hy,hz) (0,0,0))" per
//              line and ")", the count N and one "FabOnDisk: <file> <offset>"
//              per box, then two tables "N,ncomp" of per-box, per-component
//              minima and maxima, 17 significant digits, each value followed
//              by a comma, one box per line;
//   data files each FAB at its offset: a text line
//              "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))"
//              "<box> <ncomp>\n" -- the real descriptor (bytes and IEEE layout;
//              byte order, here little-endian) and the FAB's box, ghost cells
//              included -- then the values, component after component, x
//              fastest.
// The reader takes IEEE float64 or float32 in either byte order; the writer
// writes float64 in the host's byte order into one data file.
#include "../../include/nyxpm.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace {

nyxpm_status mf_fail(char* errbuf, size_t errlen, const std::string& msg)
{
    if (errbuf && errlen) std::snprintf(errbuf, errlen, "%s", msg.c_str());
    return NYXPM_INVALID_ARG;
}

struct IBox {
    int lo[3], hi[3];
    long long cells() const
    {
        return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
    }
};

struct Header {
    int version = 0, how = 0, ncomp = 0, ngrow = 0;
    std::vector<IBox> boxes;
    std::vector<std::string> files;
    std::vector<long long> offsets;
    std::vector<double> mins, maxs;  // nboxes x ncomp, empty when absent
};

// a small cursor over text
struct Text {
    const char* p;
    const char* end;
    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool lit(char c)
    {
        ws();
        if (p < end && *p == c) {
            ++p;
            return true;
        }
        return false;
    }
    bool integer(long long* v)
    {
        ws();
        if (p >= end) return false;
        char buf[32];
        size_t k = 0;
        while (p + k < end && k + 1 < sizeof(buf) && (p[k] == '-' || p[k] == '+' || (p[k] >= '0' && p[k] <= '9')))
            buf[k] = p[k], ++k;
        if (k == 0) return false;
        buf[k] = 0;
        char* stop = nullptr;
        *v = std::strtoll(buf, &stop, 10);
        if (stop != buf + k) return false;
        p += k;
        return true;
    }
    bool integer(int* v)
    {
        long long t;
        if (!integer(&t) || t < INT32_MIN || t > INT32_MAX) return false;
        *v = (int)t;
        return true;
    }
    bool real(double* v)
    {
        ws();
        if (p >= end) return false;
        char buf[64];
        size_t k = 0;
        while (p + k < end && k + 1 < sizeof(buf) && p[k] != ',' && p[k] != ' ' && p[k] != '\n' &&
               p[k] != '\r' && p[k] != '\t')
            buf[k] = p[k], ++k;
        if (k == 0) return false;
        buf[k] = 0;
        char* stop = nullptr;
        *v = std::strtod(buf, &stop);
        if (stop != buf + k) return false;
        p += k;
        return true;
    }
    bool word(std::string* w)
    {
        ws();
        const char* s = p;
        while (p < end && *p != ' ' && *p != '\t' && *p != '\n' && *p != '\r') ++p;
        w->assign(s, p);
        return !w->empty();
    }
    // "(a,b,c)"
    bool ivect(int v[3])
    {
        return lit('(') && integer(&v[0]) && lit(',') && integer(&v[1]) && lit(',') && integer(&v[2]) &&
               lit(')');
    }
    // "((lo) (hi) (type))"; cell-centred boxes only
    bool box(IBox* b)
    {
        int t[3];
        if (!(lit('(') && ivect(b->lo) && ivect(b->hi) && ivect(t) && lit(')'))) return false;
        if (t[0] || t[1] || t[2]) return false;
        for (int d = 0; d < 3; ++d)
            if (b->hi[d] < b->lo[d]) return false;
        return true;
    }
};

bool slurp(const std::string& path, std::string& out)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    out.clear();
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, got);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

std::string dir_of(const std::string& name)
{
    const size_t s = name.find_last_of('/');
    return s == std::string::npos ? std::string() : name.substr(0, s + 1);
}

std::string base_of(const std::string& name)
{
    const size_t s = name.find_last_of('/');
    return s == std::string::npos ? name : name.substr(s + 1);
}

nyxpm_status read_header(const char* name, Header* h, char* errbuf, size_t errlen)
{
    if (!name || !*name) return mf_fail(errbuf, errlen, "multifab: empty name");
    const std::string path = std::string(name) + "_H";
    std::string s;
    if (!slurp(path, s)) return mf_fail(errbuf, errlen, "multifab: cannot read " + path);
    Text t{s.data(), s.data() + s.size()};
    const std::string bad = "multifab: malformed header " + path + ": ";
    if (!t.integer(&h->version)) return mf_fail(errbuf, errlen, bad + "version");
    if (h->version != 1)
        return mf_fail(errbuf, errlen,
                       "multifab: header version " + std::to_string(h->version) + " of " + path +
                           " is not supported (version 1, FABs with their own headers, is)");
    if (!t.integer(&h->how)) return mf_fail(errbuf, errlen, bad + "write mode");
    if (!t.integer(&h->ncomp) || h->ncomp < 1) return mf_fail(errbuf, errlen, bad + "ncomp");
    t.ws();
    if (t.p < t.end && *t.p == '(') {
        int g[3];
        if (!t.ivect(g) || g[0] != g[1] || g[1] != g[2]) return mf_fail(errbuf, errlen, bad + "ngrow");
        h->ngrow = g[0];
    } else if (!t.integer(&h->ngrow)) {
        return mf_fail(errbuf, errlen, bad + "ngrow");
    }
    if (h->ngrow < 0) return mf_fail(errbuf, errlen, bad + "ngrow");
    int nb = 0, hash = 0;
    if (!(t.lit('(') && t.integer(&nb) && t.integer(&hash)) || nb < 0)
        return mf_fail(errbuf, errlen, bad + "BoxArray");
    h->boxes.resize(nb);
    for (int i = 0; i < nb; ++i)
        if (!t.box(&h->boxes[i])) return mf_fail(errbuf, errlen, bad + "box " + std::to_string(i));
    if (!t.lit(')')) return mf_fail(errbuf, errlen, bad + "BoxArray end");
    int nf = 0;
    if (!t.integer(&nf) || nf != nb) return mf_fail(errbuf, errlen, bad + "FabOnDisk count");
    h->files.resize(nb);
    h->offsets.resize(nb);
    for (int i = 0; i < nb; ++i) {
        std::string tag;
        if (!t.word(&tag) || tag != "FabOnDisk:" || !t.word(&h->files[i]) || !t.integer(&h->offsets[i]) ||
            h->offsets[i] < 0)
            return mf_fail(errbuf, errlen, bad + "FabOnDisk " + std::to_string(i));
    }
    // min / max tables (optional in the sense that a truncated header still reads)
    for (int tab = 0; tab < 2; ++tab) {
        int rows = 0, cols = 0;
        const char* save = t.p;
        if (!(t.integer(&rows) && t.lit(',') && t.integer(&cols))) {
            t.p = save;
            break;
        }
        if (rows != nb || cols != h->ncomp) return mf_fail(errbuf, errlen, bad + "min/max table shape");
        std::vector<double>& v = tab ? h->maxs : h->mins;
        v.resize((size_t)nb * cols);
        for (size_t k = 0; k < v.size(); ++k)
            if (!t.real(&v[k]) || !t.lit(',')) return mf_fail(errbuf, errlen, bad + "min/max value");
    }
    return NYXPM_OK;
}

// the FAB text header at the current position of f
struct FabHead {
    int nbytes = 0;
    bool little = true;
    IBox box;
    int ncomp = 0;
    long data_off = 0;
};

bool read_fab_head(FILE* f, FabHead* fh, std::string* why)
{
    std::string line;
    int c;
    while ((c = std::fgetc(f)) != EOF && c != '\n') {
        line.push_back((char)c);
        if (line.size() > 4096) break;
    }
    if (c != '\n') {
        *why = "no FAB header line";
        return false;
    }
    fh->data_off = std::ftell(f);
    Text t{line.data(), line.data() + line.size()};
    std::string tag;
    if (!t.word(&tag) || tag != "FAB") {
        *why = "FAB header does not start with FAB";
        return false;
    }
    // ((nbytes, (nbits ebits fbits ...)),(nbytes, (order...)))
    int nb1 = 0, fmt[8], nb2 = 0, ord[16];
    if (!(t.lit('(') && t.lit('(') && t.integer(&nb1) && t.lit(',') && t.lit('('))) {
        *why = "real descriptor";
        return false;
    }
    for (int i = 0; i < 8; ++i)
        if (!t.integer(&fmt[i])) {
            *why = "real descriptor format";
            return false;
        }
    if (!(t.lit(')') && t.lit(')') && t.lit(',') && t.lit('(') && t.integer(&nb2) && t.lit(',') && t.lit('(')) ||
        nb2 != nb1 || (nb1 != 8 && nb1 != 4)) {
        *why = "real descriptor byte order";
        return false;
    }
    for (int i = 0; i < nb2; ++i)
        if (!t.integer(&ord[i])) {
            *why = "real descriptor byte order";
            return false;
        }
    if (!(t.lit(')') && t.lit(')') && t.lit(')'))) {
        *why = "real descriptor end";
        return false;
    }
    static const int f64[8] = {64, 11, 52, 0, 1, 12, 0, 1023};
    static const int f32[8] = {32, 8, 23, 0, 1, 9, 0, 127};
    if (std::memcmp(fmt, nb1 == 8 ? f64 : f32, sizeof(fmt)) != 0) {
        *why = "the FAB's reals are not IEEE float64 / float32";
        return false;
    }
    bool asc = true, desc = true;
    for (int i = 0; i < nb2; ++i) {
        asc = asc && ord[i] == i + 1;
        desc = desc && ord[i] == nb2 - i;
    }
    if (!asc && !desc) {
        *why = "byte order neither ascending nor descending";
        return false;
    }
    fh->nbytes = nb1;
    fh->little = desc;
    if (!t.box(&fh->box) || !t.integer(&fh->ncomp) || fh->ncomp < 1) {
        *why = "FAB box or ncomp";
        return false;
    }
    return true;
}

bool host_little()
{
    const uint16_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

double decode(const unsigned char* p, int nbytes, bool swap)
{
    unsigned char b[8];
    for (int i = 0; i < nbytes; ++i) b[i] = swap ? p[nbytes - 1 - i] : p[i];
    if (nbytes == 8) {
        double v;
        std::memcpy(&v, b, 8);
        return v;
    }
    float v;
    std::memcpy(&v, b, 4);
    return (double)v;
}

// boxes of at most mgs cells per edge tiling [lo, hi], x fastest; each edge is
// cut into ceil(len / mgs) nearly equal pieces
std::vector<IBox> chop(const int lo[3], const int hi[3], int mgs)
{
    std::vector<int> cuts[3];
    for (int d = 0; d < 3; ++d) {
        const int len = hi[d] - lo[d] + 1;
        const int nblk = (len + mgs - 1) / mgs;
        const int size = len / nblk, extra = len % nblk;
        int at = lo[d];
        cuts[d].push_back(at);
        for (int k = 0; k < nblk; ++k) {
            at += size + (k < extra ? 1 : 0);
            cuts[d].push_back(at);
        }
    }
    std::vector<IBox> out;
    for (size_t kz = 0; kz + 1 < cuts[2].size(); ++kz)
        for (size_t ky = 0; ky + 1 < cuts[1].size(); ++ky)
            for (size_t kx = 0; kx + 1 < cuts[0].size(); ++kx) {
                IBox b;
                b.lo[0] = cuts[0][kx], b.hi[0] = cuts[0][kx + 1] - 1;
                b.lo[1] = cuts[1][ky], b.hi[1] = cuts[1][ky + 1] - 1;
                b.lo[2] = cuts[2][kz], b.hi[2] = cuts[2][kz + 1] - 1;
                out.push_back(b);
            }
    return out;
}

std::string fmt_box(const IBox& b)
{
    char buf[160];
    std::snprintf(buf, sizeof(buf), "((%d,%d,%d) (%d,%d,%d) (0,0,0))", b.lo[0], b.lo[1], b.lo[2], b.hi[0],
                  b.hi[1], b.hi[2]);
    return buf;
}

struct FileCloser {
    void operator()(FILE* f) const
    {
        if (f) std::fclose(f);
    }
};

}  // namespace

extern "C" {

nyxpm_status nyxpm_multifab_info_read(const char* name, nyxpm_multifab_info* info, char* errbuf, size_t errlen)
{
    if (!info) return mf_fail(errbuf, errlen, "multifab: info is NULL");
    Header h;
    nyxpm_status st = read_header(name, &h, errbuf, errlen);
    if (st != NYXPM_OK) return st;
    info->ncomp = h.ncomp;
    info->ngrow = h.ngrow;
    info->nboxes = (int)h.boxes.size();
    for (int d = 0; d < 3; ++d) {
        info->lo[d] = h.boxes.empty() ? 0 : h.boxes[0].lo[d];
        info->hi[d] = h.boxes.empty() ? -1 : h.boxes[0].hi[d];
        for (const IBox& b : h.boxes) {
            info->lo[d] = b.lo[d] < info->lo[d] ? b.lo[d] : info->lo[d];
            info->hi[d] = b.hi[d] > info->hi[d] ? b.hi[d] : info->hi[d];
        }
    }
    info->has_minmax = !h.mins.empty() && !h.maxs.empty();
    return NYXPM_OK;
}

nyxpm_status nyxpm_multifab_boxes(const char* name, int* boxes_out, double* minmax_out, char* errbuf,
                                  size_t errlen)
{
    Header h;
    nyxpm_status st = read_header(name, &h, errbuf, errlen);
    if (st != NYXPM_OK) return st;
    if (minmax_out && (h.mins.empty() || h.maxs.empty()))
        return mf_fail(errbuf, errlen, "multifab: the header has no min/max tables");
    for (size_t i = 0; i < h.boxes.size(); ++i) {
        if (boxes_out)
            for (int d = 0; d < 3; ++d) {
                boxes_out[6 * i + d] = h.boxes[i].lo[d];
                boxes_out[6 * i + 3 + d] = h.boxes[i].hi[d];
            }
        if (minmax_out)
            for (int c = 0; c < h.ncomp; ++c) {
                minmax_out[(i * h.ncomp + c) * 2] = h.mins[i * h.ncomp + c];
                minmax_out[(i * h.ncomp + c) * 2 + 1] = h.maxs[i * h.ncomp + c];
            }
    }
    return NYXPM_OK;
}

nyxpm_status nyxpm_multifab_read(const char* name, int comp0, int ncomp, const int* lo, const int* hi,
                                 unsigned flags, double* out, char* errbuf, size_t errlen)
{
    if (!lo || !hi || !out || ncomp < 1 || comp0 < 0) return mf_fail(errbuf, errlen, "multifab_read: bad arguments");
    IBox dom;
    for (int d = 0; d < 3; ++d) {
        dom.lo[d] = lo[d];
        dom.hi[d] = hi[d];
        if (hi[d] < lo[d]) return mf_fail(errbuf, errlen, "multifab_read: empty region");
    }
    Header h;
    nyxpm_status st = read_header(name, &h, errbuf, errlen);
    if (st != NYXPM_OK) return st;
    if (comp0 + ncomp > h.ncomp)
        return mf_fail(errbuf, errlen, "multifab_read: components " + std::to_string(comp0) + ".." +
                                           std::to_string(comp0 + ncomp - 1) + " of a MultiFab with " +
                                           std::to_string(h.ncomp));
    const long long nx = dom.hi[0] - dom.lo[0] + 1, ny = dom.hi[1] - dom.lo[1] + 1;
    const long long ncell = dom.cells();
    std::vector<unsigned char> seen((size_t)ncell, 0);
    const std::string dir = dir_of(name);
    std::map<std::string, std::unique_ptr<FILE, FileCloser>> files;
    const bool hl = host_little();
    std::vector<unsigned char> buf;
    for (size_t ib = 0; ib < h.boxes.size(); ++ib) {
        const IBox& vb = h.boxes[ib];
        IBox cut;
        bool any = true;
        for (int d = 0; d < 3; ++d) {
            cut.lo[d] = vb.lo[d] > dom.lo[d] ? vb.lo[d] : dom.lo[d];
            cut.hi[d] = vb.hi[d] < dom.hi[d] ? vb.hi[d] : dom.hi[d];
            any = any && cut.lo[d] <= cut.hi[d];
        }
        if (!any) continue;
        auto it = files.find(h.files[ib]);
        if (it == files.end()) {
            FILE* f = std::fopen((dir + h.files[ib]).c_str(), "rb");
            if (!f) return mf_fail(errbuf, errlen, "multifab_read: cannot open " + dir + h.files[ib]);
            it = files.emplace(h.files[ib], std::unique_ptr<FILE, FileCloser>(f)).first;
        }
        FILE* f = it->second.get();
        const std::string where = dir + h.files[ib] + " at " + std::to_string(h.offsets[ib]);
        if (std::fseek(f, (long)h.offsets[ib], SEEK_SET) != 0)
            return mf_fail(errbuf, errlen, "multifab_read: cannot seek " + where);
        FabHead fh;
        std::string why;
        if (!read_fab_head(f, &fh, &why)) return mf_fail(errbuf, errlen, "multifab_read: " + why + " in " + where);
        for (int d = 0; d < 3; ++d)
            if (fh.box.lo[d] > vb.lo[d] || fh.box.hi[d] < vb.hi[d])
                return mf_fail(errbuf, errlen, "multifab_read: the FAB box does not hold its valid box in " + where);
        if (fh.ncomp < h.ncomp) return mf_fail(errbuf, errlen, "multifab_read: FAB with too few components in " + where);
        const long long fx = fh.box.hi[0] - fh.box.lo[0] + 1, fy = fh.box.hi[1] - fh.box.lo[1] + 1;
        const long long fcells = fh.box.cells();
        const bool swap = fh.little != hl;
        buf.resize((size_t)(fcells * fh.nbytes));
        for (int c = 0; c < ncomp; ++c) {
            const long pos = fh.data_off + (long)((comp0 + c) * fcells * fh.nbytes);
            if (std::fseek(f, pos, SEEK_SET) != 0 || std::fread(buf.data(), 1, buf.size(), f) != buf.size())
                return mf_fail(errbuf, errlen, "multifab_read: short FAB data in " + where);
            double* oc = out + (size_t)c * ncell;
            for (int k = cut.lo[2]; k <= cut.hi[2]; ++k)
                for (int j = cut.lo[1]; j <= cut.hi[1]; ++j)
                    for (int i = cut.lo[0]; i <= cut.hi[0]; ++i) {
                        const long long src =
                            (i - fh.box.lo[0]) + fx * ((j - fh.box.lo[1]) + fy * (long long)(k - fh.box.lo[2]));
                        const long long dst = (i - dom.lo[0]) + nx * ((j - dom.lo[1]) + ny * (long long)(k - dom.lo[2]));
                        const double v = decode(buf.data() + src * fh.nbytes, fh.nbytes, swap);
                        if ((flags & NYXPM_MF_REJECT_NAN) && std::isnan(v))
                            return mf_fail(errbuf, errlen, "multifab_read: NaN in component " +
                                                               std::to_string(comp0 + c) + " of " + where);
                        oc[dst] = v;
                        if (c == 0) {
                            if (seen[dst]) return mf_fail(errbuf, errlen, "multifab_read: boxes overlap");
                            seen[dst] = 1;
                        }
                    }
        }
    }
    for (long long q = 0; q < ncell; ++q)
        if (!seen[q]) return mf_fail(errbuf, errlen, "multifab_read: the boxes do not cover the region");
    return NYXPM_OK;
}

nyxpm_status nyxpm_multifab_write(const char* name, int ncomp, const int* lo, const int* hi, int max_grid_size,
                                  int nboxes, const int* boxes, const double* data, char* errbuf, size_t errlen)
{
    if (!name || !*name || !lo || !hi || !data || ncomp < 1)
        return mf_fail(errbuf, errlen, "multifab_write: bad arguments");
    IBox dom;
    for (int d = 0; d < 3; ++d) {
        dom.lo[d] = lo[d];
        dom.hi[d] = hi[d];
        if (hi[d] < lo[d]) return mf_fail(errbuf, errlen, "multifab_write: empty region");
    }
    std::vector<IBox> bl;
    if (boxes && nboxes > 0) {
        for (int i = 0; i < nboxes; ++i) {
            IBox b;
            for (int d = 0; d < 3; ++d) {
                b.lo[d] = boxes[6 * i + d];
                b.hi[d] = boxes[6 * i + 3 + d];
                if (b.lo[d] < dom.lo[d] || b.hi[d] > dom.hi[d] || b.hi[d] < b.lo[d])
                    return mf_fail(errbuf, errlen, "multifab_write: box " + std::to_string(i) + " outside the region");
            }
            bl.push_back(b);
        }
        long long tot = 0;
        for (const IBox& b : bl) tot += b.cells();
        std::vector<unsigned char> seen((size_t)dom.cells(), 0);
        const long long nx = dom.hi[0] - dom.lo[0] + 1, ny = dom.hi[1] - dom.lo[1] + 1;
        for (const IBox& b : bl)
            for (int k = b.lo[2]; k <= b.hi[2]; ++k)
                for (int j = b.lo[1]; j <= b.hi[1]; ++j)
                    for (int i = b.lo[0]; i <= b.hi[0]; ++i) {
                        const long long q = (i - dom.lo[0]) + nx * ((j - dom.lo[1]) + ny * (long long)(k - dom.lo[2]));
                        if (seen[q]) return mf_fail(errbuf, errlen, "multifab_write: boxes overlap");
                        seen[q] = 1;
                    }
        if (tot != dom.cells()) return mf_fail(errbuf, errlen, "multifab_write: the boxes do not tile the region");
    } else {
        if (max_grid_size < 1) return mf_fail(errbuf, errlen, "multifab_write: max_grid_size < 1");
        bl = chop(dom.lo, dom.hi, max_grid_size);
    }
    const std::string dname = std::string(name) + "_D_00000";
    const std::string fname = base_of(name) + "_D_00000";
    std::unique_ptr<FILE, FileCloser> df(std::fopen(dname.c_str(), "wb"));
    if (!df) return mf_fail(errbuf, errlen, "multifab_write: cannot create " + dname);
    const char* order = host_little() ? "(8 7 6 5 4 3 2 1)" : "(1 2 3 4 5 6 7 8)";
    const long long nx = dom.hi[0] - dom.lo[0] + 1, ny = dom.hi[1] - dom.lo[1] + 1, ncell = dom.cells();
    std::vector<long long> offs;
    std::vector<double> mins, maxs, vals;
    long long at = 0;
    for (const IBox& b : bl) {
        offs.push_back(at);
        std::string fh = "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, ";
        fh += order;
        fh += "))" + fmt_box(b) + " " + std::to_string(ncomp) + "\n";
        if (std::fwrite(fh.data(), 1, fh.size(), df.get()) != fh.size())
            return mf_fail(errbuf, errlen, "multifab_write: write failed for " + dname);
        at += (long long)fh.size();
        vals.resize((size_t)b.cells());
        for (int c = 0; c < ncomp; ++c) {
            const double* dc = data + (size_t)c * ncell;
            size_t q = 0;
            double mn = 0, mx = 0;
            for (int k = b.lo[2]; k <= b.hi[2]; ++k)
                for (int j = b.lo[1]; j <= b.hi[1]; ++j)
                    for (int i = b.lo[0]; i <= b.hi[0]; ++i, ++q) {
                        const double v = dc[(i - dom.lo[0]) + nx * ((j - dom.lo[1]) + ny * (long long)(k - dom.lo[2]))];
                        vals[q] = v;
                        if (q == 0 || v < mn) mn = v;
                        if (q == 0 || v > mx) mx = v;
                    }
            mins.push_back(mn);
            maxs.push_back(mx);
            if (std::fwrite(vals.data(), 8, vals.size(), df.get()) != vals.size())
                return mf_fail(errbuf, errlen, "multifab_write: write failed for " + dname);
            at += (long long)vals.size() * 8;
        }
    }
    if (std::fflush(df.get()) != 0) return mf_fail(errbuf, errlen, "multifab_write: write failed for " + dname);
    df.reset();
    std::string hs = "1\n1\n" + std::to_string(ncomp) + "\n0\n(" + std::to_string(bl.size()) + " 0\n";
    for (const IBox& b : bl) hs += fmt_box(b) + "\n";
    hs += ")\n" + std::to_string(bl.size()) + "\n";
    for (size_t i = 0; i < bl.size(); ++i) hs += "FabOnDisk: " + fname + " " + std::to_string(offs[i]) + "\n";
    char num[64];
    for (int tab = 0; tab < 2; ++tab) {
        hs += "\n" + std::to_string(bl.size()) + "," + std::to_string(ncomp) + "\n";
        const std::vector<double>& v = tab ? maxs : mins;
        for (size_t i = 0; i < bl.size(); ++i) {
            for (int c = 0; c < ncomp; ++c) {
                std::snprintf(num, sizeof(num), "%.16e,", v[i * ncomp + c]);
                hs += num;
            }
            hs += "\n";
        }
    }
    hs += "\n";
    const std::string hname = std::string(name) + "_H";
    std::unique_ptr<FILE, FileCloser> hf(std::fopen(hname.c_str(), "wb"));
    if (!hf || std::fwrite(hs.data(), 1, hs.size(), hf.get()) != hs.size() || std::fflush(hf.get()) != 0)
        return mf_fail(errbuf, errlen, "multifab_write: cannot write " + hname);
    return NYXPM_OK;
}

}  // extern "C"

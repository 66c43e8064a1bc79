// Input formats on either side of the expectation path: MRC image stacks
// (src/Image/ImageFile.cpp, include/Image/MRCHeader.h) and the .thu particle
// database (src/Database.cpp, include/Database.h; written by
// Optimiser::saveDatabase, src/Optimiser.cpp:8167-8262).  Host code only.
//
// MRC: the 1024-byte header (nx, ny, nz, mode, ..., nsymbt at byte 92,
// 'MAP ' at byte 208), then nsymbt bytes of extended header, then the data,
// x fastest.  Data are returned in file order; the reference's Image keeps
// them with the centre pixel at index 0 (MESH_IMAGE_INDEX), a reindexing the
// device preprocessing does.  Modes read: 0 (int8), 1 (int16), 2 (float32),
// 6 (uint16), as ImageFile plus the unsigned mode of the MRC-2014 standard;
// writing is float32 (mode 2), as ImageFile::writeImageMRC.
//
// .thu: one particle per line, whitespace-separated columns THU_VOLTAGE (0)
// ... THU_SCORE (26): seven CTF attributes, the particle path, the
// micrograph path, coordinates, group and class ids, quaternion, k1..k3,
// translation, its standard deviations, defocus factor, its standard
// deviation, score.  Numeric columns are returned as a [n][27] double table
// (columns 7 and 8 hold NaN); the two paths as fixed-stride strings.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "thunder_gb300.h"

namespace tg3 {
// the library's error record (tg3_last_error)
int fail(int status, const std::string& msg);
}  // namespace tg3

namespace {

constexpr int kThuColumns = 27;
constexpr int kThuPath = 7, kThuMicrograph = 8, kThuGroup = 11, kThuClass = 12;

int io_fail(int code, const std::string& msg) { return tg3::fail(code, msg); }

struct File {
    FILE* f = nullptr;
    explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
};

struct MrcHead {
    int32_t nx, ny, nz, mode, nsymbt;
};

int read_head(FILE* f, MrcHead* h)
{
    unsigned char b[1024];
    if (std::fread(b, 1, 1024, f) != 1024) return io_fail(TG3_ERR_ARG, "short MRC header");
    std::memcpy(&h->nx, b + 0, 4);
    std::memcpy(&h->ny, b + 4, 4);
    std::memcpy(&h->nz, b + 8, 4);
    std::memcpy(&h->mode, b + 12, 4);
    std::memcpy(&h->nsymbt, b + 92, 4);
    if (h->nx <= 0 || h->ny <= 0 || h->nz <= 0 || h->nsymbt < 0)
        return io_fail(TG3_ERR_ARG, "bad MRC dimensions");
    return TG3_OK;
}

int mode_bytes(int mode)
{
    switch (mode) {
    case 0: return 1;
    case 1: return 2;
    case 2: return 4;
    case 6: return 2;
    default: return -1;
    }
}

}  // namespace

extern "C" int tg3_mrc_info(const char* path, int* nx, int* ny, int* nz, int* mode,
                            float* pixelSize)
{
    if (!path || !nx || !ny || !nz || !mode) return io_fail(TG3_ERR_ARG, "null pointer");
    File F(path, "rb");
    if (!F.f) return io_fail(TG3_ERR_ARG, std::string("cannot open ") + path);
    MrcHead h;
    int st = read_head(F.f, &h);
    if (st) return st;
    *nx = h.nx;
    *ny = h.ny;
    *nz = h.nz;
    *mode = h.mode;
    if (pixelSize) {
        // cella[0] / mx: the header's cell over its sampling (ImageFile writes
        // cella = n pixelSize and mx = n)
        float cella0 = 0.f;
        int32_t mx = 0;
        std::fseek(F.f, 28, SEEK_SET);
        if (std::fread(&mx, 4, 1, F.f) != 1) return io_fail(TG3_ERR_ARG, "short MRC header");
        std::fseek(F.f, 40, SEEK_SET);
        if (std::fread(&cella0, 4, 1, F.f) != 1) return io_fail(TG3_ERR_ARG, "short MRC header");
        *pixelSize = mx > 0 ? cella0 / (float)mx : 0.f;
    }
    return TG3_OK;
}

// Sections [first, first + count) as float32, file order ([count][ny][nx]).
extern "C" int tg3_mrc_read(const char* path, int first, int count, float* out)
{
    if (!path || !out || first < 0 || count <= 0) return io_fail(TG3_ERR_ARG, "bad arguments");
    File F(path, "rb");
    if (!F.f) return io_fail(TG3_ERR_ARG, std::string("cannot open ") + path);
    MrcHead h;
    int st = read_head(F.f, &h);
    if (st) return st;
    const int mb = mode_bytes(h.mode);
    if (mb < 0) return io_fail(TG3_ERR_UNSUPPORTED, "MRC mode not supported (0, 1, 2, 6 are)");
    if ((long long)first + count > h.nz) return io_fail(TG3_ERR_ARG, "sections out of range");
    const size_t sec = (size_t)h.nx * h.ny;
    const long long off = 1024LL + h.nsymbt + (long long)first * (long long)sec * mb;
    if (std::fseek(F.f, (long)off, SEEK_SET) != 0) return io_fail(TG3_ERR_ARG, "seek failed");
    const size_t n = sec * (size_t)count;
    if (h.mode == 2) {
        if (std::fread(out, 4, n, F.f) != n) return io_fail(TG3_ERR_ARG, "short MRC data");
        return TG3_OK;
    }
    std::vector<unsigned char> raw(n * (size_t)mb);
    if (std::fread(raw.data(), 1, raw.size(), F.f) != raw.size())
        return io_fail(TG3_ERR_ARG, "short MRC data");
    for (size_t i = 0; i < n; i++) {
        switch (h.mode) {
        case 0: out[i] = (float)(int8_t)raw[i]; break;
        case 1: {
            int16_t v;
            std::memcpy(&v, &raw[2 * i], 2);
            out[i] = (float)v;
            break;
        }
        default: {
            uint16_t v;
            std::memcpy(&v, &raw[2 * i], 2);
            out[i] = (float)v;
        }
        }
    }
    return TG3_OK;
}

// float32 stack or volume [nz][ny][nx] in file order; the header as
// ImageFile::fillMRCHeader fills it, with the cell in Angstrom (x and y
// scaled by the pixel size; z too for a volume).
extern "C" int tg3_mrc_write(const char* path, const float* data, int nx, int ny, int nz,
                             float pixelSize, int volume)
{
    if (!path || !data || nx <= 0 || ny <= 0 || nz <= 0) return io_fail(TG3_ERR_ARG, "bad arguments");
    unsigned char b[1024];
    std::memset(b, 0, sizeof(b));
    const int32_t ints[10] = {nx, ny, nz, 2, 0, 0, 0, nx, ny, nz};
    std::memcpy(b, ints, sizeof(ints));
    const float cella[3] = {nx * pixelSize, ny * pixelSize, volume ? nz * pixelSize : (float)nz};
    const float cellb[3] = {90.f, 90.f, 90.f};
    const int32_t map3[3] = {1, 2, 3};
    std::memcpy(b + 40, cella, 12);
    std::memcpy(b + 52, cellb, 12);
    std::memcpy(b + 64, map3, 12);
    // density statistics of the data (dmin, dmax, dmean at bytes 76-87, rms at 216)
    const size_t n = (size_t)nx * ny * nz;
    double mn = data[0], mx = data[0], s = 0.0, s2 = 0.0;
    for (size_t i = 0; i < n; i++) {
        mn = std::fmin(mn, data[i]);
        mx = std::fmax(mx, data[i]);
        s += data[i];
        s2 += (double)data[i] * data[i];
    }
    const float stats[3] = {(float)mn, (float)mx, (float)(s / n)};
    std::memcpy(b + 76, stats, 12);
    const int32_t ispg = 1;
    std::memcpy(b + 88, &ispg, 4);
    std::memcpy(b + 208, "MAP ", 4);
    const uint32_t stamp = 0x00004144u;          // little-endian machine stamp
    std::memcpy(b + 212, &stamp, 4);
    const float rms = (float)std::sqrt(std::fmax(0.0, s2 / n - (s / n) * (s / n)));
    std::memcpy(b + 216, &rms, 4);
    File F(path, "wb");
    if (!F.f) return io_fail(TG3_ERR_ARG, std::string("cannot create ") + path);
    if (std::fwrite(b, 1, 1024, F.f) != 1024 || std::fwrite(data, 4, n, F.f) != n)
        return io_fail(TG3_ERR_ARG, "write failed");
    return TG3_OK;
}

namespace {

// whitespace-separated tokens of one line (the reference splits on spaces)
void split_ws(const char* line, std::vector<std::string>& tok)
{
    tok.clear();
    const char* p = line;
    while (*p) {
        while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n') p++;
        if (!*p) break;
        const char* q = p;
        while (*q && *q != ' ' && *q != '\t' && *q != '\r' && *q != '\n') q++;
        tok.emplace_back(p, q - p);
        p = q;
    }
}

int read_lines(const char* path, std::vector<std::string>& lines)
{
    File F(path, "r");
    if (!F.f) return io_fail(TG3_ERR_ARG, std::string("cannot open ") + path);
    std::string cur;
    char buf[4096];
    lines.clear();
    while (std::fgets(buf, sizeof(buf), F.f)) {
        cur += buf;
        if (!cur.empty() && cur.back() == '\n') {
            lines.push_back(cur);
            cur.clear();
        }
    }
    if (!cur.empty()) lines.push_back(cur);
    // blank lines carry no particle
    std::vector<std::string> keep;
    std::vector<std::string> tok;
    for (auto& l : lines) {
        split_ws(l.c_str(), tok);
        if (!tok.empty()) keep.push_back(l);
    }
    lines.swap(keep);
    return TG3_OK;
}

}  // namespace

extern "C" int tg3_thu_count(const char* path, int* n)
{
    if (!path || !n) return io_fail(TG3_ERR_ARG, "null pointer");
    std::vector<std::string> lines;
    int st = read_lines(path, lines);
    if (st) return st;
    *n = (int)lines.size();
    return TG3_OK;
}

// cols [n][27] (double; 7 and 8 NaN); paths / micrographs: n strings of
// `stride` bytes each, NUL-terminated (either may be NULL).
extern "C" int tg3_thu_read(const char* path, int n, double* cols, char* paths,
                            char* micrographs, int stride)
{
    if (!path || !cols || n < 0 || ((paths || micrographs) && stride <= 1))
        return io_fail(TG3_ERR_ARG, "bad arguments");
    std::vector<std::string> lines;
    int st = read_lines(path, lines);
    if (st) return st;
    if ((int)lines.size() != n) return io_fail(TG3_ERR_ARG, "particle count differs from the file's");
    std::vector<std::string> tok;
    for (int i = 0; i < n; i++) {
        split_ws(lines[i].c_str(), tok);
        if ((int)tok.size() < kThuColumns)
            return io_fail(TG3_ERR_ARG, "line " + std::to_string(i + 1) + " has fewer than 27 columns");
        for (int c = 0; c < kThuColumns; c++) {
            double v = NAN;
            if (c != kThuPath && c != kThuMicrograph) {
                char* end = nullptr;
                errno = 0;
                v = std::strtod(tok[c].c_str(), &end);
                if (end == tok[c].c_str() || *end)
                    return io_fail(TG3_ERR_ARG, "line " + std::to_string(i + 1) + ", column " +
                                                    std::to_string(c) + ": not a number");
            }
            cols[(size_t)i * kThuColumns + c] = v;
        }
        auto put = [&](char* dst, const std::string& s) -> int {
            if (!dst) return TG3_OK;
            if ((int)s.size() >= stride) return io_fail(TG3_ERR_ARG, "path longer than the stride");
            std::memcpy(dst + (size_t)i * stride, s.c_str(), s.size() + 1);
            return TG3_OK;
        };
        if ((st = put(paths, tok[kThuPath]))) return st;
        if ((st = put(micrographs, tok[kThuMicrograph]))) return st;
    }
    return TG3_OK;
}

// The writer of Optimiser::saveDatabase: %18.9f for reals, %6d for the group
// and class ids, the two paths as strings, single spaces between columns.
extern "C" int tg3_thu_write(const char* path, int n, const double* cols, const char* paths,
                             const char* micrographs, int stride)
{
    if (!path || !cols || !paths || !micrographs || n < 0 || stride <= 1)
        return io_fail(TG3_ERR_ARG, "bad arguments");
    File F(path, "w");
    if (!F.f) return io_fail(TG3_ERR_ARG, std::string("cannot create ") + path);
    for (int i = 0; i < n; i++) {
        const double* r = cols + (size_t)i * kThuColumns;
        for (int c = 0; c < kThuColumns; c++) {
            if (c) std::fputc(' ', F.f);
            if (c == kThuPath || c == kThuMicrograph) {
                const char* s = (c == kThuPath ? paths : micrographs) + (size_t)i * stride;
                if (!*s || std::strpbrk(s, " \t\r\n"))
                    return io_fail(TG3_ERR_ARG, "path empty or with whitespace");
                std::fputs(s, F.f);
            } else if (c == kThuGroup || c == kThuClass) {
                std::fprintf(F.f, "%6d", (int)std::lround(r[c]));
            } else {
                std::fprintf(F.f, "%18.9f", r[c]);
            }
        }
        std::fputc('\n', F.f);
    }
    if (std::ferror(F.f)) return io_fail(TG3_ERR_ARG, "write failed");
    return TG3_OK;
}

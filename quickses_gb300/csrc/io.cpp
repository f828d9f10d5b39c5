// File front-end of the QuickSES command line: PDB ATOM records in, OBJ mesh out.
//
// PDB reading follows the parser QuickSES links (cpdb/cpdb.cpp:35-158, 211-265) as the
// QuickSES executable calls it (CudaSurf.cu:931-968):
//   * lines are read with fgets into one persistent 128-byte buffer (a line longer than
//     127 bytes continues as the next "line", and bytes past a short line's terminator are
//     whatever an earlier, longer line left there);
//   * only records starting with "ATOM  " are atoms (HETATM is not); reading stops at the
//     first line starting with "END" (which covers END and ENDMDL);
//   * alternate locations other than 'A' and ' ' (column 17) are skipped; hydrogens are kept;
//   * x, y, z are atof of columns 31-38, 39-46, 47-54 (8 bytes each, stopping at a NUL);
//   * the radius comes from the first non-blank byte of columns 77-79 (the element field):
//     O 1.52, C 1.70, N 1.55, H 1.20, S 1.80, P 1.80, anything else 1.40
//     (CudaSurf.h:64-73, CudaSurf.cu:961-964);
//   * atoms come out in file order (the reference walks chains in creation order and each
//     chain's atom list, which is the order the records were appended).
// One deliberate difference: when columns 77-79 are all blank the reference's field
// extraction underflows its length and overruns the element buffer; here the atom gets the
// default radius 1.40.
//
// OBJ writing follows writeToObj (CudaSurf.cu:329-371): "v %.3f %.3f %.3f" per vertex, one
// blank line, then "f %d %d %d" per triangle with the corners in (second, first, third)
// order, 1-based.  Formatting is done here (in parallel chunks) instead of by fprintf; the
// decimal rounding is exact with ties to even, which is what glibc's printf produces.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "qses_internal.h"
#include "quickses.h"

namespace {

float radius_of(char e) {
    switch (e) {
        case 'O': return 1.52f;
        case 'C': return 1.70f;
        case 'N': return 1.55f;
        case 'H': return 1.20f;
        case 'S': return 1.80f;
        case 'P': return 1.80f;
        default: return 1.40f;
    }
}

// atof of up to 8 bytes starting at `from` (stops at a NUL, like strncpy into a 9-byte,
// zero-initialised buffer).
float coord(const char *line, int from) {
    char tmp[9] = {0};
    for (int k = 0; k < 8 && line[from + k]; k++) tmp[k] = line[from + k];
    return (float)atof(tmp);
}

// ---- exact "%.3f" of a float: round(|v| * 1000) with ties to even, in integers.
// v = M * 2^E with a 24-bit M, so M * 1000 < 2^34 and the quotient/remainder are exact.
char *put_fixed3(char *o, float v) {
    uint32_t bits;
    memcpy(&bits, &v, 4);
    const bool neg = bits >> 31;
    const int ebits = (int)((bits >> 23) & 0xff);
    uint64_t mant = bits & 0x7fffff;
    int e;
    if (ebits == 0) {
        e = -149;  // subnormal (or zero)
    } else {
        mant |= 0x800000;
        e = ebits - 150;
    }
    uint64_t q;  // round(|v| * 1000)
    if (ebits == 0xff) {  // inf / nan: not produced by the mesher; print as printf would
        const char *s = mant ? (neg ? "-nan" : "nan") : (neg ? "-inf" : "inf");
        while (*s) *o++ = *s++;
        return o;
    }
    const uint64_t n = mant * 1000ull;
    if (e >= 0) {  // |v| >= 2^23: an integer, nothing to round
        return o + snprintf(o, 64, "%.3f", (double)v);
    } else if (-e >= 64) {
        q = 0;  // |v| * 1000 < 2^35 * 2^-64 < 0.5
    } else {
        const int sh = -e;
        q = n >> sh;
        const uint64_t r = n - (q << sh), half = 1ull << (sh - 1);
        if (r > half || (r == half && (q & 1))) q++;
    }
    if (neg) *o++ = '-';
    const uint64_t ip = q / 1000;
    const unsigned fp = (unsigned)(q % 1000);
    char tmp[24];
    int k = 0;
    uint64_t t = ip;
    do {
        tmp[k++] = (char)('0' + t % 10);
        t /= 10;
    } while (t);
    while (k) *o++ = tmp[--k];
    *o++ = '.';
    *o++ = (char)('0' + fp / 100);
    *o++ = (char)('0' + (fp / 10) % 10);
    *o++ = (char)('0' + fp % 10);
    return o;
}

char *put_int(char *o, long long v) {
    if (v < 0) {
        *o++ = '-';
        v = -v;
    }
    char tmp[24];
    int k = 0;
    do {
        tmp[k++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    while (k) *o++ = tmp[--k];
    return o;
}

// Formats items [lo, hi) of one section into `out`.
void format_vertices(const qses_float3 *v, size_t lo, size_t hi, std::string &out) {
    out.resize((hi - lo) * 200 + 64);  // a float wider than 2^23 may print up to ~50 digits
    char *o = &out[0];
    for (size_t i = lo; i < hi; i++) {
        *o++ = 'v';
        *o++ = ' ';
        o = put_fixed3(o, v[i].x);
        *o++ = ' ';
        o = put_fixed3(o, v[i].y);
        *o++ = ' ';
        o = put_fixed3(o, v[i].z);
        *o++ = '\n';
    }
    out.resize((size_t)(o - &out[0]));
}

void format_faces(const int *t, size_t lo, size_t hi, std::string &out) {
    out.resize((hi - lo) * 40);
    char *o = &out[0];
    for (size_t i = lo; i < hi; i++) {
        *o++ = 'f';
        *o++ = ' ';
        o = put_int(o, (long long)t[3 * i + 1] + 1);
        *o++ = ' ';
        o = put_int(o, (long long)t[3 * i] + 1);
        *o++ = ' ';
        o = put_int(o, (long long)t[3 * i + 2] + 1);
        *o++ = '\n';
    }
    out.resize((size_t)(o - &out[0]));
}

// Formats a section in parallel chunks and writes them in order.
template <typename F>
bool write_section(FILE *f, size_t n, int threads, F fmt) {
    const size_t chunk = 1u << 16;
    size_t at = 0;
    std::vector<std::string> bufs((size_t)threads);
    while (at < n) {
        std::vector<std::thread> pool;
        size_t used = 0;
        for (int k = 0; k < threads && at + (size_t)k * chunk < n; k++) {
            const size_t lo = at + (size_t)k * chunk, hi = std::min(n, lo + chunk);
            pool.emplace_back([&, k, lo, hi] { fmt(lo, hi, bufs[(size_t)k]); });
            used++;
        }
        for (auto &th : pool) th.join();
        for (size_t k = 0; k < used; k++)
            if (fwrite(bufs[k].data(), 1, bufs[k].size(), f) != bufs[k].size()) return false;
        at += used * chunk;
    }
    return true;
}

}  // namespace

extern "C" {

QSES_API int qses_read_pdb(const char *path, float **xyz, float **radii, unsigned *n) {
    if (!path || !xyz || !radii || !n) return QSES_ERR_INVALID_ARG;
    *xyz = nullptr;
    *radii = nullptr;
    *n = 0;
    FILE *f = fopen(path, "r");
    if (!f) return QSES_ERR_INVALID_ARG;
    std::vector<float> p, r;
    char line[128];
    memset(line, 0, sizeof(line));
    while (fgets(line, sizeof(line), f)) {
        if (!strncmp(line, "ATOM  ", 6)) {
            const char alt = line[16];
            if (!(alt == 'A' || alt == ' ')) continue;
            p.push_back(coord(line, 30));
            p.push_back(coord(line, 38));
            p.push_back(coord(line, 46));
            char e = 0;
            for (int k = 76; k <= 78; k++)
                if (line[k] != ' ') {
                    e = line[k];
                    break;
                }
            r.push_back(radius_of(e));
        } else if (!strncmp(line, "END", 3)) {
            break;
        }
    }
    fclose(f);
    const unsigned cnt = (unsigned)r.size();
    if (cnt) {
        *xyz = (float *)malloc(p.size() * sizeof(float));
        *radii = (float *)malloc(r.size() * sizeof(float));
        if (!*xyz || !*radii) {
            free(*xyz);
            free(*radii);
            *xyz = nullptr;
            *radii = nullptr;
            return QSES_ERR_OUT_OF_MEMORY;
        }
        memcpy(*xyz, p.data(), p.size() * sizeof(float));
        memcpy(*radii, r.data(), r.size() * sizeof(float));
    }
    *n = cnt;
    return QSES_OK;
}

QSES_API void qses_free(void *p) { free(p); }

QSES_API int qses_write_obj(const char *path, const qses_float3 *vertices, unsigned nv, const int *triangles,
                            unsigned nt, int threads) {
    if (!path || (nv && !vertices) || (nt && !triangles)) return QSES_ERR_INVALID_ARG;
    if (threads <= 0) {
        const unsigned hc = std::thread::hardware_concurrency();
        threads = hc ? (int)std::min(hc, 16u) : 4;
    }
    FILE *f = fopen(path, "w");
    if (!f) return QSES_ERR_INVALID_ARG;
    bool ok = write_section(f, nv, threads,
                            [&](size_t lo, size_t hi, std::string &o) { format_vertices(vertices, lo, hi, o); });
    ok = ok && fputc('\n', f) != EOF;
    ok = ok && write_section(f, nt, threads,
                             [&](size_t lo, size_t hi, std::string &o) { format_faces(triangles, lo, hi, o); });
    ok = (fclose(f) == 0) && ok;
    return ok ? QSES_OK : QSES_ERR_INVALID_ARG;
}

// Formats one float as "%.3f" would (test hook for the exact rounding).
QSES_API int qses_format_fixed3(float v, char *out, int cap) {
    char tmp[64];
    char *e = put_fixed3(tmp, v);
    const int len = (int)(e - tmp);
    if (!out || cap <= len) return -1;
    memcpy(out, tmp, (size_t)len);
    out[len] = 0;
    return len;
}

}  // extern "C"

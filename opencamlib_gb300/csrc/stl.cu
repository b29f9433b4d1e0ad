// stl.cu -- STL file reading (host code): the triangles an STLReader would
// add to an STLSurf (src/geo/stlreader.cpp:57-150), as a flat array.
//
// Format choice and parsing follow the reference:
//   * a file whose first five bytes are not "solid" is binary: an 80-byte
//     header, a little-endian uint32 facet count, then per facet a normal and
//     three vertices as 12 little-endian float32 and a 2-byte attribute;
//   * otherwise it is ASCII, read line by line: a line's first five
//     non-blank characters (blanks between them are skipped too) select
//     "verte" (sscanf " vertex %f %f %f" into the current vertex, which then
//     advances, at most to the third), "facet" (back to the first vertex) or
//     "endfa" (a triangle when the vertex index is 2, i.e. after two or more
//     vertex lines).  Coordinates are parsed as float and widened to double;
//     a vertex line that does not parse keeps the previous values.
// Where the reference does not terminate or reads memory it never wrote,
// this reader does something defined instead:
//   * a binary file whose header starts with "solid" (the reference parses it
//     as ASCII and, on a line longer than its 1,024-byte buffer, loops
//     forever) is read as binary when the file size is exactly
//     84 + 50 x (facet count) with a non-zero count;
//   * ASCII lines longer than 1,023 characters are cut there;
//   * vertex values before any vertex line are 0 (the reference's are
//     uninitialised);
//   * a binary file shorter than its facet count says yields the complete
//     facets and the status OCL_GB300_BAD_ARG (the reference adds the
//     missing facets with stale coordinates).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "util.cuh"

namespace oclg {

namespace {

struct TriSink {
    double* out;
    uint64_t cap;
    uint64_t n = 0;
    void add(const float x[3][3]) {
        if (out && n < cap)
            for (int k = 0; k < 9; ++k) out[9 * n + k] = (double)x[k / 3][k % 3];
        ++n;
    }
};

float le_f32(const unsigned char* p) {
    uint32_t u = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

uint32_t le_u32(const unsigned char* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// sscanf(s, " <word> %f %f %f", ...) on a NUL-terminated line: the number of
// values converted; v[] keeps its old values beyond that.
int scan_word_floats(const char* s, const char* word, float* v) {
    while (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\v' || *s == '\f' || *s == '\r') ++s;
    const size_t wl = std::strlen(word);
    if (std::strncmp(s, word, wl) != 0) return 0;
    s += wl;
    int got = 0;
    for (int k = 0; k < 3; ++k) {
        char* end = nullptr;
        const float f = std::strtof(s, &end);
        if (end == s) break;
        v[k] = f;
        ++got;
        s = end;
    }
    return got;
}

int read_binary(const std::vector<unsigned char>& b, TriSink& sink) {
    if (b.size() < 84) return OCL_GB300_OK;  // the reference reads a zero count
    const uint32_t nf = le_u32(&b[80]);
    float x[3][3];
    for (uint32_t i = 0; i < nf; ++i) {
        const size_t off = 84 + (size_t)i * 50;
        if (off + 50 > b.size()) {
            set_error("STL: binary file shorter than its facet count");
            return OCL_GB300_BAD_ARG;
        }
        for (int k = 0; k < 9; ++k) x[k / 3][k % 3] = le_f32(&b[off + 12 + 4 * k]);
        sink.add(x);
    }
    return OCL_GB300_OK;
}

void read_ascii(const std::vector<unsigned char>& b, TriSink& sink) {
    float x[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    int vertex = 0;
    size_t pos = 5;  // "solid"
    // the rest of the first line is the title
    while (pos < b.size() && b[pos] != '\n') ++pos;
    if (pos < b.size()) ++pos;
    char line[1024];
    while (pos < b.size()) {
        size_t len = 0;
        while (pos < b.size() && b[pos] != '\n') {
            if (len < sizeof(line) - 1) line[len++] = (char)b[pos];
            ++pos;
        }
        if (pos < b.size()) ++pos;  // the newline
        line[len] = 0;
        // first five non-blank characters, blanks between them skipped
        char five[6] = {0, 0, 0, 0, 0, 0};
        int i = 0;
        size_t j = 0;
        for (; i < 5; ++i, ++j) {
            if (j >= len) break;
            while (j < len && (line[j] == ' ' || line[j] == '\t')) ++j;
            if (j >= len) break;
            five[i] = line[j];
        }
        if (i != 5) continue;
        if (!std::strcmp(five, "verte")) {
            scan_word_floats(line, "vertex", x[vertex]);
            if (++vertex > 2) vertex = 2;
        } else if (!std::strcmp(five, "facet")) {
            vertex = 0;  // the facet normal is read there but never used
        } else if (!std::strcmp(five, "endfa")) {
            if (vertex == 2) sink.add(x);
        }
    }
}

}  // namespace

}  // namespace oclg

using namespace oclg;

extern "C" int ocl_gb300_stl_read(const char* path, double* tris, uint64_t cap, uint64_t* count) {
    if (!path || !count || (cap && !tris)) {
        set_error("stl_read: null argument");
        return OCL_GB300_BAD_ARG;
    }
    *count = 0;
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("stl_read: cannot open ") + path);
        return OCL_GB300_BAD_ARG;
    }
    std::vector<unsigned char> b;
    unsigned char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) b.insert(b.end(), buf, buf + got);
    std::fclose(f);
    TriSink sink{tris, cap};
    int st = OCL_GB300_OK;
    if (b.size() < 5) {
        // the reference stops at end of file before the format check
    } else if (std::memcmp(b.data(), "solid", 5) != 0) {
        st = read_binary(b, sink);
    } else if (b.size() >= 84 && le_u32(&b[80]) > 0 && b.size() == 84 + 50 * (uint64_t)le_u32(&b[80])) {
        st = read_binary(b, sink);  // binary with a "solid" header
    } else {
        read_ascii(b, sink);
    }
    *count = sink.n;
    if (st == OCL_GB300_OK && sink.n > cap && tris) {
        set_error("stl_read: more triangles than the output holds");
        return OCL_GB300_BAD_ARG;
    }
    return st;
}

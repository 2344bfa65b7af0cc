// binio.cpp -- binary cache of an edge list and of a shortest-path tree.
//
// The text formats (all_structure_undir.cuh:133-198 read them with fgets/sscanf) cost seconds
// per 10^8 lines even with the parallel parser; a binary image of the same arrays loads at
// file-system speed.  A file is a 32-byte header -- 8-byte magic, two int64 sizes, a 64-bit
// checksum of the payload -- followed by the arrays, little-endian:
//   graph  "DSSPG001", n, m, checksum, u[m] int32, v[m] int32, w[m] int32
//   tree   "DSSPT001", n, 0, checksum, parent[n] int32, dist[n] int64
// The checksum is position-dependent and computed in parallel: the sum over the payload's
// 8-byte words x_i of mix64(x_i ^ (i * golden)), the trailing bytes zero-padded.  A reader
// rejects a file with another magic, other sizes than the caller expects, a short payload or
// a checksum mismatch (DSSSP_E_IO), so a stale or truncated cache is never used.
#include <omp.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/dsssp.h"
#include "host_common.h"

using namespace dsssp;

namespace {

constexpr char kGraphMagic[8] = {'D', 'S', 'S', 'P', 'G', '0', '0', '1'};
constexpr char kTreeMagic[8] = {'D', 'S', 'S', 'P', 'T', '0', '0', '1'};

struct Header {
    char magic[8];
    int64_t a, b;
    uint64_t sum;
};
static_assert(sizeof(Header) == 32, "binary header is 32 bytes");

struct Part {
    const void* p;
    size_t bytes;
};

// Checksum of the concatenation of the parts (word index runs across parts).
uint64_t checksum(const std::vector<Part>& parts) {
    std::vector<uint8_t> tail;
    uint64_t total = 0, word_base = 0;
    for (const Part& pt : parts) {
        const size_t words = pt.bytes / 8;
        const uint8_t* base = static_cast<const uint8_t*>(pt.p);
        uint64_t s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (int64_t i = 0; i < (int64_t)words; i++) {
            uint64_t x;
            memcpy(&x, base + 8 * (size_t)i, 8);
            s += mix64(x ^ ((word_base + (uint64_t)i) * kGolden));
        }
        total += s;
        word_base += words;
        const size_t rest = pt.bytes - 8 * words;
        if (rest) {  // every array here is a multiple of 4 bytes: pad the tail word
            uint64_t x = 0;
            memcpy(&x, base + 8 * words, rest);
            total += mix64(x ^ (word_base * kGolden) ^ 0xA5A5A5A5ull);
            word_base++;
        }
    }
    return total;
}

int write_file(const char* path, const char (&magic)[8], int64_t a, int64_t b, const std::vector<Part>& parts) {
    Header h;
    memcpy(h.magic, magic, 8);
    h.a = a;
    h.b = b;
    h.sum = checksum(parts);
    FILE* f = fopen(path, "wb");
    if (!f) return fail(DSSSP_E_IO, "cannot create %s: %s", path, strerror(errno));
    bool ok = fwrite(&h, sizeof h, 1, f) == 1;
    for (const Part& pt : parts)
        if (ok && pt.bytes) ok = fwrite(pt.p, 1, pt.bytes, f) == pt.bytes;
    if (fclose(f) != 0) ok = false;
    if (!ok) {
        remove(path);
        return fail(DSSSP_E_IO, "write to %s failed", path);
    }
    return DSSSP_OK;
}

int read_header(FILE* f, const char* path, const char (&magic)[8], Header& h) {
    if (fread(&h, sizeof h, 1, f) != 1) return fail(DSSSP_E_IO, "%s: no binary header", path);
    if (memcmp(h.magic, magic, 8) != 0) return fail(DSSSP_E_IO, "%s: not a binary %s file", path,
                                                   magic[4] == 'G' ? "graph" : "tree");
    return DSSSP_OK;
}

// Bytes from the current position to the end of f (the position is kept); -1 if unknown.
long long bytes_left(FILE* f) {
    const long here = ftell(f);
    if (here < 0 || fseek(f, 0, SEEK_END) != 0) return -1;
    const long end = ftell(f);
    if (fseek(f, here, SEEK_SET) != 0 || end < here) return -1;
    return (long long)(end - here);
}

int read_parts(FILE* f, const char* path, const std::vector<Part>& parts, uint64_t want) {
    for (const Part& pt : parts)
        if (pt.bytes && fread(const_cast<void*>(pt.p), 1, pt.bytes, f) != pt.bytes)
            return fail(DSSSP_E_IO, "%s: file is shorter than its header says", path);
    if (checksum(parts) != want) return fail(DSSSP_E_IO, "%s: checksum mismatch", path);
    return DSSSP_OK;
}

}  // namespace

extern "C" {

int dsssp_write_graph_binary(const char* path, int32_t n, int64_t m, const int32_t* u, const int32_t* v,
                             const int32_t* w) {
    if (!path || n <= 0 || m < 0 || (m > 0 && (!u || !v || !w)))
        return fail(DSSSP_E_INVAL, "write_graph_binary: bad arguments");
    const size_t b = sizeof(int32_t) * (size_t)m;
    return write_file(path, kGraphMagic, n, m, {{u, b}, {v, b}, {w, b}});
}

int dsssp_read_graph_binary(const char* path, int32_t n, int32_t** u, int32_t** v, int32_t** w, int64_t* m) {
    if (!path || n <= 0 || !u || !v || !w || !m) return fail(DSSSP_E_INVAL, "read_graph_binary: bad arguments");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(DSSSP_E_IO, "cannot open %s: %s", path, strerror(errno));
    Header h;
    int rc = read_header(f, path, kGraphMagic, h);
    if (!rc && h.a != n) rc = fail(DSSSP_E_IO, "%s: cached graph has %lld vertices, not %d", path, (long long)h.a, n);
    // the header's edge count must match the file's size before anything is allocated for it
    if (!rc) {
        const long long left = bytes_left(f), per_edge = 3 * (long long)sizeof(int32_t);
        if (h.b < 0 || left < 0 || h.b > left / per_edge || h.b * per_edge != left)
            rc = fail(DSSSP_E_IO, "%s: the edge count in the header does not match the file size", path);
    }
    int32_t *a = nullptr, *bb = nullptr, *c = nullptr;
    if (!rc) {
        const size_t bytes = sizeof(int32_t) * (size_t)(h.b ? h.b : 1);
        a = (int32_t*)malloc(bytes);
        bb = (int32_t*)malloc(bytes);
        c = (int32_t*)malloc(bytes);
        if (!a || !bb || !c) rc = fail(DSSSP_E_OOM, "read_graph_binary: host allocation failed");
    }
    if (!rc) {
        const size_t b = sizeof(int32_t) * (size_t)h.b;
        rc = read_parts(f, path, {{a, b}, {bb, b}, {c, b}}, h.sum);
    }
    fclose(f);
    if (!rc) {  // the same range check as the text reader
        int64_t bad = -1;
#pragma omp parallel for reduction(max : bad)
        for (int64_t i = 0; i < h.b; i++)
            if (a[i] < 0 || a[i] >= n || bb[i] < 0 || bb[i] >= n) bad = i > bad ? i : bad;
        if (bad >= 0) rc = fail(DSSSP_E_BAD_VERTEX, "%s: edge %lld names a vertex outside 0..%d", path, (long long)bad, n - 1);
    }
    if (rc) {
        free(a);
        free(bb);
        free(c);
        return rc;
    }
    *u = a;
    *v = bb;
    *w = c;
    *m = h.b;
    return DSSSP_OK;
}

int dsssp_write_sssp_binary(const char* path, int32_t n, const int32_t* parent, const int64_t* dist) {
    if (!path || n <= 0 || !parent || !dist) return fail(DSSSP_E_INVAL, "write_sssp_binary: bad arguments");
    return write_file(path, kTreeMagic, n, 0,
                      {{parent, sizeof(int32_t) * (size_t)n}, {dist, sizeof(int64_t) * (size_t)n}});
}

int dsssp_read_sssp_binary(const char* path, int32_t n, int32_t* parent, int64_t* dist) {
    if (!path || n <= 0 || !parent || !dist) return fail(DSSSP_E_INVAL, "read_sssp_binary: bad arguments");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(DSSSP_E_IO, "cannot open %s: %s", path, strerror(errno));
    Header h;
    int rc = read_header(f, path, kTreeMagic, h);
    if (!rc && h.a != n) rc = fail(DSSSP_E_IO, "%s: cached tree has %lld vertices, not %d", path, (long long)h.a, n);
    if (!rc && bytes_left(f) != (long long)(sizeof(int32_t) + sizeof(int64_t)) * n)
        rc = fail(DSSSP_E_IO, "%s: the file size does not match a tree of %d vertices", path, n);
    if (!rc)
        rc = read_parts(f, path, {{parent, sizeof(int32_t) * (size_t)n}, {dist, sizeof(int64_t) * (size_t)n}}, h.sum);
    fclose(f);
    return rc;
}

}  // extern "C"

// MatrixMarket edge-list loader (host, multi-threaded).
//
// Two semantics, chosen by `mode`:
//   KC_LOAD_COO  -- Graph::ReadGraph (index2core/shared/graph.cpp:17-95) and
//                   the id shift of VirtualGraph::VirtualGraph
//                   (virtual_graph.cpp:16-23): skip two lines, read `u v` per
//                   line, drop self-loops, keep duplicate lines; n = max id,
//                   plus one if id 0 occurs; without id 0 all ids shift down.
//   KC_LOAD_CSR_DEDUP -- Graph::readFile (peel/src/graph.cpp:58-102): skip
//                   two lines, ids are 1-based, self-loops dropped, V = largest
//                   id (1 when no edge survives, as the reference's V++ gives).
//                   De-duplication happens in the device CSR build.
// Lines that start with '%' and blank lines are skipped.  In the reference a
// comment line after the second line re-parses into a self-loop and is
// dropped, so the results agree for files with long comment headers.  A line
// without two integer ids is rejected (KC_ERR_INVALID, with its line number)
// instead of silently repeating the previous edge as the reference does.
//
// The file is read in one piece and split into per-thread chunks at line
// boundaries; each thread parses its chunk and the chunks are concatenated in
// file order, so the edge order (and with it the row order of the COO build)
// equals the reference's.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "kc_internal.h"

namespace kc {

namespace {

struct Chunk {
    std::vector<uint32_t> src, dst;
    uint64_t max_id = 0;
    bool has_zero = false;
    bool bad = false;
    uint64_t bad_offset = 0;
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\f' || c == '\v'; }

// Parses an unsigned decimal at p (after skipping blanks); returns false if
// none is there or it overflows 32 bits.
inline bool parse_u32(const char *&p, const char *end, uint64_t &out) {
    while (p < end && is_space(*p)) p++;
    if (p >= end || *p < '0' || *p > '9') return false;
    uint64_t v = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        v = v * 10 + (uint64_t)(*p - '0');
        if (v > 0xffffffffull) return false;
        p++;
    }
    out = v;
    return true;
}

void parse_range(const char *begin, const char *end, Chunk &c) {
    const char *p = begin;
    c.src.reserve((size_t)(end - begin) / 12 + 16);
    c.dst.reserve((size_t)(end - begin) / 12 + 16);
    while (p < end) {
        const char *eol = static_cast<const char *>(memchr(p, '\n', (size_t)(end - p)));
        if (!eol) eol = end;
        const char *q = p;
        while (q < eol && is_space(*q)) q++;
        if (q < eol && *q != '%') {
            uint64_t a, b;
            const char *r = q;
            if (!parse_u32(r, eol, a) || !parse_u32(r, eol, b) || (r < eol && !is_space(*r))) {
                c.bad = true;
                c.bad_offset = (uint64_t)(p - begin);
                return;
            }
            if (a != b) {
                c.src.push_back((uint32_t)a);
                c.dst.push_back((uint32_t)b);
                if (a == 0 || b == 0) c.has_zero = true;
                c.max_id = std::max(c.max_id, std::max(a, b));
            }
        }
        p = eol + 1;
    }
}

}  // namespace

int parse_mtx(const char *path, int mode, uint32_t *n_out, uint64_t *m_out, uint32_t **src_out,
              uint32_t **dst_out) {
    if (!path || !n_out || !m_out || !src_out || !dst_out) return fail(KC_ERR_INVALID, "parse_mtx: null argument");
    if (mode != KC_LOAD_COO && mode != KC_LOAD_CSR_DEDUP) return fail(KC_ERR_INVALID, "unknown load mode %d", mode);
    FILE *f = fopen(path, "rb");
    if (!f) return fail(KC_ERR_IO, "cannot open %s", path);
    std::vector<char> buf;
    if (fseek(f, 0, SEEK_END) == 0) {
        long sz = ftell(f);
        if (sz > 0) {
            buf.resize((size_t)sz);
            fseek(f, 0, SEEK_SET);
            if (fread(buf.data(), 1, (size_t)sz, f) != (size_t)sz) {
                fclose(f);
                return fail(KC_ERR_IO, "short read on %s", path);
            }
        }
    }
    fclose(f);
    const char *b = buf.data(), *e = b + buf.size();
    // skip exactly two lines: the %%MatrixMarket banner and the size line
    const char *body = b;
    for (int skip = 0; skip < 2 && body < e; skip++) {
        const char *nl = static_cast<const char *>(memchr(body, '\n', (size_t)(e - body)));
        body = nl ? nl + 1 : e;
    }
    size_t bytes = (size_t)(e - body);
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    unsigned T = (unsigned)std::min<size_t>(std::min<unsigned>(hw, 64), bytes / (1u << 20) + 1);
    std::vector<const char *> cut(T + 1);
    cut[0] = body;
    cut[T] = e;
    for (unsigned t = 1; t < T; t++) {
        const char *p = body + bytes * t / T;
        if (p < cut[t - 1]) p = cut[t - 1];
        const char *nl = static_cast<const char *>(memchr(p, '\n', (size_t)(e - p)));
        cut[t] = nl ? nl + 1 : e;
    }
    std::vector<Chunk> chunks(T);
    if (T == 1) {
        parse_range(cut[0], cut[1], chunks[0]);
    } else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < T; t++) th.emplace_back(parse_range, cut[t], cut[t + 1], std::ref(chunks[t]));
        for (auto &x : th) x.join();
    }
    uint64_t m = 0, max_id = 0;
    bool has_zero = false;
    for (unsigned t = 0; t < T; t++) {
        if (chunks[t].bad) {
            const char *at = cut[t] + chunks[t].bad_offset;
            uint64_t line = 1 + (uint64_t)std::count(b, at, '\n');
            return fail(KC_ERR_INVALID, "%s:%llu: expected two integer vertex ids", path, (unsigned long long)line);
        }
        m += chunks[t].src.size();
        max_id = std::max(max_id, chunks[t].max_id);
        has_zero |= chunks[t].has_zero;
    }
    uint32_t n;
    int shift;
    if (mode == KC_LOAD_COO) {
        n = (uint32_t)(has_zero ? max_id + 1 : max_id);
        if (has_zero && max_id == 0xffffffffull) return fail(KC_ERR_INVALID, "vertex id range exceeds uint32");
        shift = has_zero ? 0 : 1;
    } else {
        if (has_zero) return fail(KC_ERR_INVALID, "%s: id 0 in a 1-based file (KC_LOAD_CSR_DEDUP)", path);
        n = m ? (uint32_t)max_id : 1u;
        shift = 1;
    }
    uint32_t *src = static_cast<uint32_t *>(malloc(std::max<uint64_t>(m, 1) * 4));
    uint32_t *dst = static_cast<uint32_t *>(malloc(std::max<uint64_t>(m, 1) * 4));
    if (!src || !dst) {
        free(src);
        free(dst);
        return fail(KC_ERR_NOMEM, "host allocation of %llu edges", (unsigned long long)m);
    }
    uint64_t off = 0;
    for (unsigned t = 0; t < T; t++) {
        const Chunk &c = chunks[t];
        for (size_t i = 0; i < c.src.size(); i++) {
            src[off + i] = c.src[i] - (uint32_t)shift;
            dst[off + i] = c.dst[i] - (uint32_t)shift;
        }
        off += c.src.size();
    }
    *n_out = n;
    *m_out = m;
    *src_out = src;
    *dst_out = dst;
    return KC_OK;
}

}  // namespace kc

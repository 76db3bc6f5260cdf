// Event-file ingestion on the host (no GPU work): the "ts x y polarity" text format of
// utils/event_camera/event.py:11-39, parsed by several threads into structure-of-arrays
// buffers that the event-frame kernels take directly.
//
// The reference reads the file line by line in Python (an Event object per line), which
// takes minutes for the 10^8-event sequences of the VECTOR datasets; here the buffer is
// cut at line boundaries into one chunk per thread, each thread counts its lines, parses
// its chunk into the output at its first line's index, and the chunks are then moved
// together (blank lines are skipped, so a chunk can hold fewer events than lines).
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "gsevt.h"

namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// One signed decimal integer at *p (after spaces and tabs); false if none or on overflow.
inline bool parse_int(const char *&p, const char *end, int64_t &v)
{
    while (p < end && is_space(*p)) ++p;
    bool neg = false;
    if (p < end && (*p == '-' || *p == '+')) {
        neg = *p == '-';
        ++p;
    }
    if (p >= end || *p < '0' || *p > '9') return false;
    uint64_t acc = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        const uint64_t d = (uint64_t)(*p - '0');
        if (acc > (UINT64_C(9223372036854775807) - d) / 10) return false;
        acc = acc * 10 + d;
        ++p;
    }
    v = neg ? -(int64_t)acc : (int64_t)acc;
    return true;
}

struct Chunk {
    const char *begin, *end;
    size_t first_line;  // index of the chunk's first line in the buffer
    size_t events;      // events parsed
    int status;         // GSEVT_OK or GSEVT_ERR_ARG
    size_t bad_line;    // line index of the first malformed line
};

// Parses the lines of one chunk into the outputs at index c.first_line onwards: each line
// holds exactly four integers (ts, x, y, polarity) or only white space.
void parse_chunk(Chunk &c, int64_t *ts, uint16_t *x, uint16_t *y, uint8_t *pol)
{
    const char *p = c.begin;
    size_t line = c.first_line, out = c.first_line;
    c.status = GSEVT_OK;
    while (p < c.end) {
        const char *q = p;
        while (q < c.end && is_space(*q)) ++q;
        if (q >= c.end || *q == '\n') {  // blank line
            p = q < c.end ? q + 1 : q;
            ++line;
            continue;
        }
        int64_t v[4];
        bool ok = true;
        for (int k = 0; k < 4 && ok; ++k) ok = parse_int(q, c.end, v[k]);
        while (ok && q < c.end && is_space(*q)) ++q;
        ok = ok && (q >= c.end || *q == '\n') && v[1] >= 0 && v[1] <= 65535 && v[2] >= 0 && v[2] <= 65535;
        if (!ok) {
            c.status = GSEVT_ERR_ARG;
            c.bad_line = line;
            break;
        }
        ts[out] = v[0];
        x[out] = (uint16_t)v[1];
        y[out] = (uint16_t)v[2];
        pol[out] = v[3] != 0 ? 1 : 0;
        ++out;
        ++line;
        p = q < c.end ? q + 1 : q;
    }
    c.events = out - c.first_line;
}

}  // namespace

extern "C" int gsevt_parse_events_txt(const char *text, size_t len, int64_t *ts, uint16_t *x, uint16_t *y,
                                      uint8_t *polarity, size_t capacity, size_t *count, int32_t threads)
{
    if (count) *count = 0;
    if (!count || (len > 0 && !text)) return GSEVT_ERR_ARG;
    if (len == 0) return GSEVT_OK;
    // lines in the buffer (a last line without a newline counts too): the output capacity
    // that every chunk's placement at its first line's index needs
    size_t lines = 0;
    for (const char *p = text, *e = text + len; (p = (const char *)std::memchr(p, '\n', (size_t)(e - p))) != nullptr;
         ++p)
        ++lines;
    if (text[len - 1] != '\n') ++lines;
    if (capacity < lines || !ts || !x || !y || !polarity) return GSEVT_ERR_TOO_LARGE;
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    nt = nt < 1 ? 1 : (nt > 64 ? 64 : nt);
    if (len < ((size_t)1 << 20)) nt = 1;  // not worth the threads below 1 MB
    // chunk boundaries just after a newline
    std::vector<Chunk> ch((size_t)nt);
    const char *start = text, *const end = text + len;
    for (int i = 0; i < nt; ++i) {
        const char *e = (i == nt - 1) ? end : text + (len / (size_t)nt) * (size_t)(i + 1);
        if (e < start) e = start;
        if (e < end) {
            const char *nl = (const char *)std::memchr(e, '\n', (size_t)(end - e));
            e = nl ? nl + 1 : end;
        }
        ch[(size_t)i].begin = start;
        ch[(size_t)i].end = e;
        start = e;
    }
    // first line index of each chunk
    std::vector<size_t> nlines((size_t)nt, 0);
    auto count_lines = [&](int i) {
        size_t n = 0;
        for (const char *p = ch[(size_t)i].begin, *e = ch[(size_t)i].end;
             p < e && (p = (const char *)std::memchr(p, '\n', (size_t)(e - p))) != nullptr; ++p)
            ++n;
        nlines[(size_t)i] = n;
    };
    auto run = [&](auto fn) {
        std::vector<std::thread> th;
        for (int i = 1; i < nt; ++i) th.emplace_back(fn, i);
        fn(0);
        for (auto &t : th) t.join();
    };
    run(count_lines);
    size_t acc = 0;
    for (int i = 0; i < nt; ++i) {
        ch[(size_t)i].first_line = acc;
        acc += nlines[(size_t)i];
    }
    run([&](int i) { parse_chunk(ch[(size_t)i], ts, x, y, polarity); });
    // move the chunks together, in order; stop at the first malformed line
    size_t out = 0;
    for (int i = 0; i < nt; ++i) {
        const Chunk &c = ch[(size_t)i];
        if (c.events && out != c.first_line) {
            std::memmove(ts + out, ts + c.first_line, c.events * sizeof(int64_t));
            std::memmove(x + out, x + c.first_line, c.events * sizeof(uint16_t));
            std::memmove(y + out, y + c.first_line, c.events * sizeof(uint16_t));
            std::memmove(polarity + out, polarity + c.first_line, c.events);
        }
        out += c.events;
        if (c.status != GSEVT_OK) {
            *count = out;
            return c.status;
        }
    }
    *count = out;
    return GSEVT_OK;
}

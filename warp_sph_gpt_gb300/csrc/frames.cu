// frames.cu -- host-side text formatting of particle frames (VTK XML
// PolyData, ASCII), the hot part of the reference's frame output
// (output/output.py:16-25 _fmt_float / _fmt_int): values printed "%.6g"
// (floats, as doubles) or "%d", separated by one space, per_line values per
// line, lines joined by '\n' (no trailing newline).  The work is split over
// host threads by whole lines, each formatting into its own buffer; the pieces
// are then concatenated in order, so the text equals the single-threaded one.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace {

template <class T>
void format_lines(const T* v, int64_t begin, int64_t end, int per_line, bool is_float, std::string& out) {
    char buf[64];
    out.clear();
    out.reserve((size_t)(end - begin) * (is_float ? 13 : 8));
    for (int64_t i = begin; i < end; ++i) {
        int len = is_float ? snprintf(buf, sizeof(buf), "%.6g", (double)v[i])
                           : snprintf(buf, sizeof(buf), "%d", (int)v[i]);
        out.append(buf, (size_t)len);
        if (i + 1 < end || end < 0) out.push_back(((i + 1) % per_line) ? ' ' : '\n');
    }
}

template <class T>
int64_t format_all(const T* v, int64_t n, int per_line, bool is_float, char* out, int64_t cap, int threads) {
    if (n <= 0) return 0;
    const int64_t lines = (n + per_line - 1) / per_line;
    int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
    if (nt < 1) nt = 1;
    if (nt > 64) nt = 64;
    if ((int64_t)nt > lines) nt = (int)lines;
    if (n < 4096) nt = 1;
    std::vector<std::string> parts((size_t)nt);
    std::vector<std::thread> pool;
    const int64_t per = (lines + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        const int64_t b = std::min(n, (int64_t)t * per * per_line), e = std::min(n, (int64_t)(t + 1) * per * per_line);
        pool.emplace_back([&, b, e, t]() {
            format_lines(v, b, e, per_line, is_float, parts[(size_t)t]);
            if (e < n && e > b) parts[(size_t)t].push_back('\n');  // chunk ends on a line boundary
        });
    }
    for (auto& th : pool) th.join();
    int64_t total = 0;
    for (auto& p : parts) total += (int64_t)p.size();
    if (!out) return total;  // size query
    if (total > cap) return -1;
    int64_t off = 0;
    for (auto& p : parts) {
        memcpy(out + off, p.data(), p.size());
        off += (int64_t)p.size();
    }
    return total;
}

}  // namespace

extern "C" int64_t sphdem_format_f32(const float* v, int64_t n, int32_t per_line, char* out, int64_t cap,
                                     int32_t threads) {
    if ((!v && n > 0) || per_line <= 0 || n < 0) return -2;
    return format_all(v, n, per_line, true, out, cap, threads);
}

extern "C" int64_t sphdem_format_i32(const int32_t* v, int64_t n, int32_t per_line, char* out, int64_t cap,
                                     int32_t threads) {
    if ((!v && n > 0) || per_line <= 0 || n < 0) return -2;
    return format_all(v, n, per_line, false, out, cap, threads);
}

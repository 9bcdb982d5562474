// snapio.cpp — text encodings of the reference's particle files (host code).
//
// The reference writes its checkpoints as one text line per particle with
// every FP64 value printed as the hexadecimal image of its bits ("%llx",
// HelmholtzGas::writeHexa, hdr_hgas.hpp:286-316), so that a restart is
// bit-exact, and its snapshots as fixed-format decimal text
// (HelmholtzGas::writeAscii, hdr_hgas.hpp:136-180).  These functions produce
// and parse such lines for n particles at once; the column order and units
// are the caller's (research_codes_gb300/snapshot.py).
#include <cinttypes>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../include/sph_gb300.h"

namespace {

uint64_t bits(double x) {
    uint64_t u;
    std::memcpy(&u, &x, sizeof(u));
    return u;
}

double from_bits(uint64_t u) {
    double x;
    std::memcpy(&x, &u, sizeof(x));
    return x;
}

// Appends printf output to out[pos..cap) (counting only when out is null or
// full) and returns the new position.
template <class... A>
int64_t put(char *out, int64_t cap, int64_t pos, const char *fmt, A... a) {
    char buf[64];
    const int k = std::snprintf(buf, sizeof(buf), fmt, a...);
    if (out && pos + k <= cap) std::memcpy(out + pos, buf, (size_t)k);
    return pos + k;
}

}  // namespace

extern "C" int64_t sph_format_hexa_rows(int64_t n, const int64_t *id, const int64_t *istar, int32_t ncol,
                                        const double *cols, char *out, int64_t cap) {
    if (n < 0 || ncol < 1 || (n > 0 && (!id || !istar || !cols))) return -SPH_ERR_INVALID_ARGUMENT;
    int64_t pos = 0;
    for (int64_t i = 0; i < n; ++i) {
        const double *c = cols + i * ncol;
        pos = put(out, cap, pos, "%6" PRId64 " %2" PRId64 " %" PRIx64, id[i], istar[i], bits(c[0]));
        for (int32_t k = 1; k < ncol; ++k) pos = put(out, cap, pos, " %" PRIx64, bits(c[k]));
        pos = put(out, cap, pos, "\n");
    }
    return pos;
}

extern "C" int64_t sph_parse_hexa_rows(const char *text, int64_t len, int64_t n, int32_t ncol, int64_t *id,
                                       int64_t *istar, double *cols) {
    if (!text || len < 0 || n < 0 || ncol < 1 || (n > 0 && (!id || !istar || !cols)))
        return -SPH_ERR_INVALID_ARGUMENT;
    const char *p = text, *end = text + len;
    auto skip = [&]() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r')) ++p;
    };
    auto token = [&](int base, bool sign, uint64_t *u, int64_t *s) -> bool {
        skip();
        if (p >= end) return false;
        char buf[40];
        int k = 0;
        while (p < end && k < 39 && *p != ' ' && *p != '\n' && *p != '\t' && *p != '\r') buf[k++] = *p++;
        buf[k] = 0;
        char *e = nullptr;
        if (sign) *s = std::strtoll(buf, &e, base);
        else *u = std::strtoull(buf, &e, base);
        return e && *e == 0 && k > 0;
    };
    for (int64_t i = 0; i < n; ++i) {
        uint64_t u = 0;
        int64_t s = 0;
        if (!token(10, true, &u, &s)) return i;
        id[i] = s;
        if (!token(10, true, &u, &s)) return i;
        istar[i] = s;
        for (int32_t k = 0; k < ncol; ++k) {
            if (!token(16, false, &u, &s)) return i;
            cols[i * ncol + k] = from_bits(u);
        }
    }
    return n;
}

// kinds[k]: 'e' -> " %+e", 'c' -> " %+.3e", 'd' -> " %6lld" (value truncated
// to an integer).
extern "C" int64_t sph_format_ascii_rows(int64_t n, const int64_t *id, const int64_t *istar, int32_t ncol,
                                         const double *cols, const char *kinds, char *out, int64_t cap) {
    if (n < 0 || ncol < 0 || !kinds || (int32_t)std::strlen(kinds) != ncol || (n > 0 && (!id || !istar)) ||
        (n > 0 && ncol > 0 && !cols))
        return -SPH_ERR_INVALID_ARGUMENT;
    int64_t pos = 0;
    for (int64_t i = 0; i < n; ++i) {
        const double *c = cols + i * ncol;
        pos = put(out, cap, pos, "%6" PRId64 " %2" PRId64, id[i], istar[i]);
        for (int32_t k = 0; k < ncol; ++k) {
            switch (kinds[k]) {
                case 'c': pos = put(out, cap, pos, " %+.3e", c[k]); break;
                case 'd': pos = put(out, cap, pos, " %6" PRId64, (int64_t)c[k]); break;
                default: pos = put(out, cap, pos, " %+e", c[k]); break;
            }
        }
        pos = put(out, cap, pos, "\n");
    }
    return pos;
}

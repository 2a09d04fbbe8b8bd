// gpumpi_libc.h.cuh — C library string and number functions for ranks' device code.
//
// A converted C program calls atoi, strlen, strcmp, ... from device code, where the host C library is not
// available.  The reference ships a device libc for this (gpu_libs/gpu_libc/stdlib.cu, string.cu, with
// headers that map the standard names); here they are small inline device functions with a gpumpi_
// prefix.  A program that defines GPUMPI_LIBC_NAMES before including this header gets the standard
// names mapped onto them (the source converter does this).  malloc, free, memcpy, memset and the math
// functions are CUDA's own device functions and need no mapping; calloc is malloc zeroed; realloc has no
// device counterpart (CUDA's heap does not tell a block's size).
//
// gpumpi_strtod / gpumpi_atof read decimal and hexadecimal digits, exponents, "inf" and "nan"; the value is
// the decimal significand (up to 19 digits) scaled by powers of ten, which can differ from the correctly
// rounded value in the last bit.
#pragma once
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

__device__ inline size_t gpumpi_strlen(const char* s) {
    size_t n = 0;
    while (s[n]) n++;
    return n;
}
__device__ inline size_t gpumpi_strnlen(const char* s, size_t max) {
    size_t n = 0;
    while (n < max && s[n]) n++;
    return n;
}
__device__ inline int gpumpi_strcmp(const char* a, const char* b) {
    while (*a && *a == *b) a++, b++;
    return (int)(unsigned char)*a - (int)(unsigned char)*b;
}
__device__ inline int gpumpi_strncmp(const char* a, const char* b, size_t n) {
    for (; n; n--, a++, b++) {
        if (*a != *b || !*a) return (int)(unsigned char)*a - (int)(unsigned char)*b;
    }
    return 0;
}
__device__ inline char* gpumpi_strcpy(char* d, const char* s) {
    char* r = d;
    while ((*d++ = *s++)) {}
    return r;
}
__device__ inline char* gpumpi_strncpy(char* d, const char* s, size_t n) {
    size_t i = 0;
    for (; i < n && s[i]; i++) d[i] = s[i];
    for (; i < n; i++) d[i] = 0;
    return d;
}
__device__ inline char* gpumpi_strcat(char* d, const char* s) {
    gpumpi_strcpy(d + gpumpi_strlen(d), s);
    return d;
}
__device__ inline char* gpumpi_strncat(char* d, const char* s, size_t n) {
    char* e = d + gpumpi_strlen(d);
    size_t i = 0;
    for (; i < n && s[i]; i++) e[i] = s[i];
    e[i] = 0;
    return d;
}
__device__ inline char* gpumpi_strchr(const char* s, int c) {
    for (;; s++) {
        if (*s == (char)c) return (char*)s;
        if (!*s) return nullptr;
    }
}
__device__ inline char* gpumpi_strrchr(const char* s, int c) {
    const char* r = nullptr;
    for (;; s++) {
        if (*s == (char)c) r = s;
        if (!*s) return (char*)r;
    }
}
__device__ inline char* gpumpi_strstr(const char* h, const char* n) {
    if (!*n) return (char*)h;
    for (; *h; h++) {
        size_t i = 0;
        while (n[i] && h[i] == n[i]) i++;
        if (!n[i]) return (char*)h;
    }
    return nullptr;
}
__device__ inline int gpumpi_memcmp(const void* a, const void* b, size_t n) {
    const unsigned char *x = (const unsigned char*)a, *y = (const unsigned char*)b;
    for (size_t i = 0; i < n; i++)
        if (x[i] != y[i]) return (int)x[i] - (int)y[i];
    return 0;
}
__device__ inline void* gpumpi_memchr(const void* s, int c, size_t n) {
    const unsigned char* p = (const unsigned char*)s;
    for (size_t i = 0; i < n; i++)
        if (p[i] == (unsigned char)c) return (void*)(p + i);
    return nullptr;
}

// strdup / strndup: copies on CUDA's device heap (released with free)
__device__ inline char* gpumpi_strndup(const char* s, size_t n) {
    const size_t len = gpumpi_strnlen(s, n);
    char* d = (char*)malloc(len + 1);
    if (d) {
        for (size_t i = 0; i < len; i++) d[i] = s[i];
        d[len] = 0;
    }
    return d;
}
__device__ inline char* gpumpi_strdup(const char* s) { return gpumpi_strndup(s, (size_t)-1); }

// calloc: CUDA's device malloc, zeroed (the block can be released with free)
__device__ inline void* gpumpi_calloc(size_t n, size_t size) {
    if (size && n > ((size_t)-1) / size) return nullptr;
    void* p = malloc(n * size);
    if (p) memset(p, 0, n * size);
    return p;
}

// getenv: the host process's environment, asked over the world's host channel (nullptr without one); the
// value (at most 255 bytes) stays valid until the rank's next call.  Defined by the runtime library.
__device__ char* gpumpi_getenv(const char* name);
// exit: the calling rank ends with `status` as if its program had returned it (from the rank's program
// thread; ranks still waiting on it get bounded-wait errors).  Defined by the runtime library.
__device__ void gpumpi_exit(int status);

__device__ inline int gpumpi_isspace_(int c) { return c == ' ' || (c >= '\t' && c <= '\r'); }
__device__ inline int gpumpi_digit_(int c, int base) {
    int v = c >= '0' && c <= '9' ? c - '0' : c >= 'a' && c <= 'z' ? c - 'a' + 10 : c >= 'A' && c <= 'Z' ? c - 'A' + 10 : 99;
    return v < base ? v : -1;
}

// strtoull's digit loop; *neg tells whether a '-' preceded the digits, *any whether digits were read
__device__ inline unsigned long long gpumpi_strtou_(const char* s, char** end, int base, int* neg, int* any,
                                                    int* overflow) {
    const char* p = s;
    while (gpumpi_isspace_(*p)) p++;
    *neg = 0;
    if (*p == '+' || *p == '-') *neg = *p++ == '-';
    if ((base == 0 || base == 16) && p[0] == '0' && (p[1] == 'x' || p[1] == 'X') && gpumpi_digit_(p[2], 16) >= 0) {
        p += 2;
        base = 16;
    } else if (base == 0) {
        base = p[0] == '0' ? 8 : 10;
    }
    unsigned long long v = 0;
    *any = 0;
    *overflow = 0;
    for (int d; (d = gpumpi_digit_(*p, base)) >= 0; p++) {
        if (v > (~0ull - (unsigned)d) / (unsigned)base) *overflow = 1;
        v = v * (unsigned)base + (unsigned)d;
        *any = 1;
    }
    if (end) *end = (char*)(*any ? p : s);
    return v;
}
__device__ inline unsigned long long gpumpi_strtoull(const char* s, char** end, int base) {
    int neg, any, of;
    unsigned long long v = gpumpi_strtou_(s, end, base, &neg, &any, &of);
    if (of) return ~0ull;
    return neg ? (unsigned long long)(-(long long)v) : v;
}
__device__ inline long long gpumpi_strtoll(const char* s, char** end, int base) {
    int neg, any, of;
    unsigned long long v = gpumpi_strtou_(s, end, base, &neg, &any, &of);
    const unsigned long long lim = neg ? 0x8000000000000000ull : 0x7fffffffffffffffull;
    if (of || v > lim) return neg ? (long long)0x8000000000000000ull : 0x7fffffffffffffffll;
    return neg ? (long long)(0 - v) : (long long)v;
}
__device__ inline long gpumpi_strtol(const char* s, char** end, int base) { return (long)gpumpi_strtoll(s, end, base); }
__device__ inline unsigned long gpumpi_strtoul(const char* s, char** end, int base) {
    return (unsigned long)gpumpi_strtoull(s, end, base);
}
__device__ inline int gpumpi_atoi(const char* s) { return (int)gpumpi_strtol(s, nullptr, 10); }
__device__ inline long gpumpi_atol(const char* s) { return gpumpi_strtol(s, nullptr, 10); }
__device__ inline long long gpumpi_atoll(const char* s) { return gpumpi_strtoll(s, nullptr, 10); }

__device__ inline double gpumpi_pow10_(int e) {
    // powers of ten up to 1e22 are exact doubles; larger ones multiply exact factors
    const double exact[] = {1e0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10, 1e11,
                            1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    double r = 1.0;
    while (e > 22) {
        r *= 1e22;
        e -= 22;
    }
    return r * exact[e];
}
__device__ inline double gpumpi_strtod(const char* s, char** end) {
    const char* p = s;
    while (gpumpi_isspace_(*p)) p++;
    bool neg = false;
    if (*p == '+' || *p == '-') neg = *p++ == '-';
    auto lower = [](char c) { return (char)(c >= 'A' && c <= 'Z' ? c + 32 : c); };
    if (lower(p[0]) == 'i' && lower(p[1]) == 'n' && lower(p[2]) == 'f') {
        p += 3;
        if (lower(p[0]) == 'i' && lower(p[1]) == 'n' && lower(p[2]) == 'i' && lower(p[3]) == 't' &&
            lower(p[4]) == 'y')
            p += 5;
        if (end) *end = (char*)p;
        return neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll);
    }
    if (lower(p[0]) == 'n' && lower(p[1]) == 'a' && lower(p[2]) == 'n') {
        if (end) *end = (char*)(p + 3);
        return __longlong_as_double(0x7ff8000000000000ll);
    }
    if (p[0] == '0' && (p[1] == 'x' || p[1] == 'X')) {
        const char* q = p + 2;
        double v = 0;
        int any = 0, exp2 = 0;
        for (int d; (d = gpumpi_digit_(*q, 16)) >= 0; q++, any = 1) v = v * 16 + d;
        if (*q == '.')
            for (q++; gpumpi_digit_(*q, 16) >= 0; q++, any = 1) {
                v = v * 16 + gpumpi_digit_(*q, 16);
                exp2 -= 4;
            }
        if (any && (*q == 'p' || *q == 'P')) {
            char* e2;
            long x = gpumpi_strtol(q + 1, &e2, 10);
            if (e2 != q + 1) {
                exp2 += (int)x;
                q = e2;
            }
        }
        if (!any) {
            if (end) *end = (char*)s;
            return 0.0;
        }
        if (end) *end = (char*)q;
        v = ldexp(v, exp2);
        return neg ? -v : v;
    }
    unsigned long long m = 0;
    int digits = 0, dexp = 0, any = 0;
    for (; *p >= '0' && *p <= '9'; p++, any = 1) {
        if (digits < 19) {
            m = m * 10 + (unsigned)(*p - '0');
            if (m) digits++;
        } else {
            dexp++;
        }
    }
    if (*p == '.') {
        for (p++; *p >= '0' && *p <= '9'; p++, any = 1) {
            if (digits < 19) {
                m = m * 10 + (unsigned)(*p - '0');
                if (m) digits++;
                dexp--;
            }
        }
    }
    if (!any) {
        if (end) *end = (char*)s;
        return 0.0;
    }
    if (*p == 'e' || *p == 'E') {
        char* e2;
        long x = gpumpi_strtol(p + 1, &e2, 10);
        if (e2 != p + 1) {
            dexp += (int)(x > 100000 ? 100000 : x < -100000 ? -100000 : x);
            p = e2;
        }
    }
    if (end) *end = (char*)p;
    double v = (double)m;
    if (m == 0) return neg ? -0.0 : 0.0;
    if (dexp > 0) v = dexp > 308 ? v * gpumpi_pow10_(308) * gpumpi_pow10_(dexp - 308 > 308 ? 308 : dexp - 308)
                                 : v * gpumpi_pow10_(dexp);
    else if (dexp < 0) v = -dexp > 308 ? v / gpumpi_pow10_(308) / gpumpi_pow10_(-dexp - 308 > 308 ? 308 : -dexp - 308)
                                       : v / gpumpi_pow10_(-dexp);
    return neg ? -v : v;
}
__device__ inline double gpumpi_atof(const char* s) { return gpumpi_strtod(s, nullptr); }

#ifdef GPUMPI_LIBC_NAMES
#define strlen gpumpi_strlen
#define strnlen gpumpi_strnlen
#define strcmp gpumpi_strcmp
#define strncmp gpumpi_strncmp
#define strcpy gpumpi_strcpy
#define strncpy gpumpi_strncpy
#define strcat gpumpi_strcat
#define strncat gpumpi_strncat
#define strchr gpumpi_strchr
#define strrchr gpumpi_strrchr
#define strstr gpumpi_strstr
#define memcmp gpumpi_memcmp
#define memchr gpumpi_memchr
#define strtol gpumpi_strtol
#define strtoll gpumpi_strtoll
#define strtoul gpumpi_strtoul
#define strtoull gpumpi_strtoull
#define strtod gpumpi_strtod
#define atoi gpumpi_atoi
#define atol gpumpi_atol
#define atoll gpumpi_atoll
#define atof gpumpi_atof
#define calloc gpumpi_calloc
#define strdup gpumpi_strdup
#define strndup gpumpi_strndup
#define getenv gpumpi_getenv
#define exit gpumpi_exit
#endif

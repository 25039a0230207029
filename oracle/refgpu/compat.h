// compat.h -- the MSVC library functions the reference's host code calls
// (fopen_s, strncpy_s, errno_t), forced into each translation unit of the
// reference's build on Linux.  TEST INFRASTRUCTURE.
#pragma once
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <sys/stat.h>
#include <sys/types.h>

typedef int errno_t;
static inline errno_t fopen_s(FILE** f, const char* name, const char* mode) {
    *f = std::fopen(name, mode);
    return *f ? 0 : errno;
}
static inline errno_t strncpy_s(char* dst, size_t size, const char* src, size_t count) {
    if (!dst || size == 0) return EINVAL;
    size_t n = std::strlen(src);
    if (n > count) n = count;
    if (n >= size) n = size - 1;
    std::memcpy(dst, src, n);
    dst[n] = 0;
    return 0;
}

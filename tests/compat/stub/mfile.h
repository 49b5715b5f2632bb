// Stand-in for BOINC's MFILE (buffered output file) with the calls the
// CUDA port's host code makes.
#pragma once
#include <cstdarg>
#include <cstdio>

class MFILE {
public:
    int open(const char *path, const char *mode)
    {
        f_ = std::fopen(path, mode);
        return f_ ? 0 : -1;
    }
    int printf(const char *fmt, ...)
    {
        va_list ap;
        va_start(ap, fmt);
        const int n = std::vfprintf(f_, fmt, ap);
        va_end(ap);
        return n;
    }
    int flush() { return std::fflush(f_); }
    int close()
    {
        const int r = f_ ? std::fclose(f_) : 0;
        f_ = nullptr;
        return r;
    }

private:
    std::FILE *f_ = nullptr;
};

/* Stand-in for BOINC's MFILE used by the reference period_search app.
 * Besides the formatted text it writes a sidecar "<name>.full" with the six
 * row values at %.17g, so that tests can compare binary doubles. */
#ifndef PS_REF_STUB_MFILE_H
#define PS_REF_STUB_MFILE_H
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

class MFILE {
    FILE *f_ = nullptr, *full_ = nullptr;

public:
    int open(const char *path, const char *mode)
    {
        f_ = std::fopen(path, mode);
        std::string side = std::string(path) + ".full";
        full_ = std::fopen(side.c_str(), mode);
        return (f_ && full_) ? 0 : 1;
    }
    int printf(const char *fmt, ...)
    {
        va_list ap, ap2;
        va_start(ap, fmt);
        va_copy(ap2, ap);
        int n = std::vfprintf(f_, fmt, ap);
        if (std::strncmp(fmt, "%.8f", 4) == 0) {
            for (int i = 0; i < 6; i++) std::fprintf(full_, i ? " %.17g" : "%.17g", va_arg(ap2, double));
            std::fprintf(full_, "\n");
        }
        va_end(ap2);
        va_end(ap);
        return n;
    }
    int flush()
    {
        std::fflush(full_);
        return std::fflush(f_);
    }
    int close()
    {
        if (full_) std::fclose(full_);
        int r = f_ ? std::fclose(f_) : 0;
        f_ = full_ = nullptr;
        return r;
    }
};
#endif

/* Minimal stand-in for the BOINC client API, enough to build the reference
 * period_search CPU app standalone.  Written for this project; it only
 * resolves logical file names to the same names in the working directory. */
#ifndef PS_REF_STUB_BOINC_API_H
#define PS_REF_STUB_BOINC_API_H
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

inline int boinc_init() { return 0; }
inline int boinc_resolve_filename(const char *name, char *out, int len)
{
    std::snprintf(out, (size_t)len, "%s", name);
    return 0;
}
inline int boinc_resolve_filename_s(const char *name, std::string &out)
{
    out = name;
    return 0;
}
inline FILE *boinc_fopen(const char *path, const char *mode) { return std::fopen(path, mode); }
inline char *boinc_msg_prefix(char *buf, int len)
{
    std::snprintf(buf, (size_t)len, "ps_ref");
    return buf;
}
inline int boinc_is_standalone() { return 1; }
inline int boinc_fraction_done(double) { return 0; }
inline int boinc_time_to_checkpoint() { return 0; }
inline int boinc_checkpoint_completed() { return 0; }
inline int boinc_rename(const char *a, const char *b) { return std::rename(a, b); }
inline void boinc_finish(int status) { std::exit(status); }
// used by the AVX/FMA variant of the reference app
struct APP_INIT_DATA {
    int major_version = 0, minor_version = 0, release = 0;
};
inline int boinc_get_init_data(APP_INIT_DATA &) { return 0; }
#endif

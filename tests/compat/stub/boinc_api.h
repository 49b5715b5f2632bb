// Stand-ins for the BOINC API calls that the CUDA port's host code makes,
// for building the drop-in adaptor into a test program: standalone mode,
// no checkpoint requests.
#pragma once
#include <cstdio>

inline int boinc_time_to_checkpoint() { return 0; }
inline int boinc_is_standalone() { return 1; }
inline void boinc_checkpoint_completed() {}
inline int boinc_fraction_done(double) { return 0; }
inline char *boinc_msg_prefix(char *buf, int len)
{
    if (len > 0) buf[0] = 0;
    return buf;
}

// Replica validator: the agreement rule by which two period_search_out files
// of one work unit are accepted as the same result
// (validator/period_search_validator4.cpp:23-109), as a library for
// cross-build agreement reports (CPU oracle, FP64 form, mixed form).
//
// Reader (init_result, :23-69): entries of six numbers are read with
// fscanf until end of file; a read that yields neither 6 numbers nor end of
// file, or a NaN period, rms or chi^2, rejects the file.  The end-of-file
// read still stores an entry holding the previous values, so a file ending
// in a newline yields one entry more than it has rows; both replicas get
// the same extra entry.  An empty file is rejected here (the reference reads
// uninitialised values there).
//
// Rule (compare_results, :71-109): the replicas match when both hold
// entries, the same number of them, and on every entry
// |(a - b) / (a + b)| / 2 stays within 0.1 for the period, 0.1 for the rms
// and 0.5 for chi^2.

#include <cmath>
#include <cstdio>
#include <vector>

#include "ps_gb300.h"

namespace {

const double kTol[3] = {0.1, 0.1, 0.5};

struct Entry {
    double v[3];
};

double half_rel(double a, double b) { return std::fabs((a - b) / (a + b)) / 2; }

// Returns PS_OK, PS_ERR_IO (unreadable) or PS_ERR_ARG (rejected by the
// reader: *parse_error set).
ps_status read_entries(const char *path, std::vector<Entry> &out, int32_t *parse_error)
{
    out.clear();
    std::FILE *f = std::fopen(path, "r");
    if (!f) return PS_ERR_IO;
    double per = NAN, rms = NAN, chisq = NAN, dark = 0, lam = 0, bet = 0;
    while (!std::feof(f)) {
        const int n = std::fscanf(f, "%lf %lf %lf %lf %lf %lf", &per, &rms, &chisq, &dark, &lam, &bet);
        if ((n != 6 && n != EOF) || std::isnan(per) || std::isnan(rms) || std::isnan(chisq)) {
            std::fclose(f);
            *parse_error = 1;
            return PS_ERR_ARG;
        }
        out.push_back(Entry{{per, rms, chisq}});
    }
    std::fclose(f);
    return PS_OK;
}

void compare(const std::vector<Entry> &a, const std::vector<Entry> &b, const double *tol, ps_validate_report *r)
{
    const double *t = tol ? tol : kTol;
    r->entries_a = static_cast<int64_t>(a.size());
    r->entries_b = static_cast<int64_t>(b.size());
    r->first_mismatch = -1;
    r->mismatch_column = -1;
    for (int k = 0; k < 3; k++) {
        r->max_dev[k] = 0;
        r->argmax_dev[k] = -1;
    }
    r->match = !a.empty() && a.size() == b.size();
    const size_t n = a.size() < b.size() ? a.size() : b.size();
    for (size_t i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) {
            const double d = half_rel(a[i].v[k], b[i].v[k]);
            if (!(d <= r->max_dev[k])) {        // NaN counts as the largest deviation
                r->max_dev[k] = d;
                r->argmax_dev[k] = static_cast<int64_t>(i);
            }
            if (r->first_mismatch < 0 && !(d <= t[k])) {
                r->first_mismatch = static_cast<int64_t>(i);
                r->mismatch_column = k;
            }
        }
    }
    if (r->first_mismatch >= 0) r->match = 0;
}

std::vector<Entry> entries_of(const ps_row *rows, int64_t n)
{
    std::vector<Entry> e(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; i++) e[static_cast<size_t>(i)] = Entry{{rows[i].period_h, rows[i].rms, rows[i].chi2}};
    return e;
}

}  // namespace

extern "C" {

ps_status ps_validate_rows(const ps_row *a, int64_t na, const ps_row *b, int64_t nb, const double *tol,
                           ps_validate_report *report)
{
    if (!report || na < 0 || nb < 0 || (na && !a) || (nb && !b)) return PS_ERR_ARG;
    *report = ps_validate_report{};
    compare(entries_of(a, na), entries_of(b, nb), tol, report);
    return PS_OK;
}

ps_status ps_validate_files(const char *path_a, const char *path_b, const double *tol, ps_validate_report *report)
{
    if (!path_a || !path_b || !report) return PS_ERR_ARG;
    *report = ps_validate_report{};
    std::vector<Entry> a, b;
    ps_status st = read_entries(path_a, a, &report->parse_error_a);
    if (st == PS_ERR_IO) return st;
    ps_status st2 = read_entries(path_b, b, &report->parse_error_b);
    if (st2 == PS_ERR_IO) return st2;
    if (st != PS_OK || st2 != PS_OK) {
        report->entries_a = static_cast<int64_t>(a.size());
        report->entries_b = static_cast<int64_t>(b.size());
        report->first_mismatch = -1;
        report->mismatch_column = -1;
        report->match = 0;          // a rejected replica never matches
        return PS_OK;
    }
    compare(a, b, tol, report);
    return PS_OK;
}

}  // extern "C"

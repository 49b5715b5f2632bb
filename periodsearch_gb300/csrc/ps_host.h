// ps_host.h -- internal host-side structures of the GB300 period-search engine.
//
// HostObject holds one object after the reference's input preparation
// (period_search/period_search_BOINC.cpp:322-485) and L0 set-up (trifac.c,
// areanorm.c, sphfunc.c, ellfit.c).  All arrays are 0-based.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "ps_gb300.h"

namespace psg {

constexpr int kNPhPar = 3;  // phase-function parameters (period_search_BOINC.cpp:563)

// Shape tables of the trifac grid for one (nrows, lmax, mmax).
struct ShapeTables {
    int nrows = 0, lmax = 0, mmax = 0;
    int nfac = 0, ndir = 0, ncoef = 0, npairs = 0;
    std::vector<int> ifp;          // [nfac*3] vertex numbers (1-based values)
    std::vector<double> at, af;    // [nfac] normal direction angles
    std::vector<double> nor;       // [nfac*3]
    std::vector<double> darea;     // [nfac]
    std::vector<double> fc, fs;    // [nfac*(mmax+1)]
    std::vector<double> pleg;      // [nfac*npairs] P_l^m per (m, l) pair in basis order
    std::vector<int> pair_m, pair_n;  // [npairs] order m and first coefficient index
    std::vector<double> dsph;      // [nfac*ncoef] basis functions
};

void build_shape(ShapeTables &s, int nrows, int lmax, int mmax);
// Initial ellipsoid coefficients; returns false when the normal matrix is
// singular (the reference exits with code 4).
bool ellipsoid_coefficients(const ShapeTables &s, double a, double b, double c,
                            std::vector<double> &cg);

struct HostObject {
    ps_header hdr{};
    int n_lc = 0;                      // real lightcurves
    std::vector<int> lc_points;        // [n_lc + 1], the last entry = 3 convexity rows
    std::vector<int> lc_rel;           // [n_lc + 1], 1 = relative lightcurve
    std::vector<int> lc_start;         // [n_lc + 1]
    int ndata = 0;                     // real points
    std::vector<double> tim, bright, sig, weight;  // [ndata + 3]
    std::vector<double> ee, ee0;       // [(ndata) * 3] unit vectors to Earth / Sun
    bool onlyrel = true;
    double jd_min = 0, jd_max = 0, jd0 = 0, phi0 = 0;
    double escl = 0, a = 0, b = 0, c = 0;
    double conw_r0 = 0;
    double freq_start = 0, freq_end = 0, freq_step = 0;
    int64_t n_max = 0;
    int ncoef = 0, ma = 0, mfit = 0;
    std::vector<int> ia;               // [ma]
    std::vector<int> free_list;        // [mfit]
    std::vector<double> cg_first;      // [ncoef]
    ShapeTables shape;
    int max_rel_points = 0;            // longest relative lightcurve
};

// Input preparation of one problem; returns PS_OK or the reference's error.
ps_status prepare_object(const ps_problem &p, HostObject &o, std::string &err);
// The same from the reference's prepared state (no input preparation).
ps_status prepare_object_state(const ps_state &st, HostObject &o, std::string &err);
// Sets the convexity rows for a given conw_r (brightness 0, sigma 1/conw_r).
void set_convexity_rows(HostObject &o, double conw_r);

// Parsed period_search_in text, owning its arrays.
struct ParsedInput {
    ps_header hdr{};
    std::vector<int32_t> lc_points, lc_calibrated;
    std::vector<double> lc_weight;
    std::vector<double> jd, brightness, sun, earth;
};
ps_status parse_input_file(const std::string &path, ParsedInput &in, std::string &err);

// Reduction of the 10 pole fits of one period into one output row
// (period_search_BOINC.cpp:913-925).
ps_row best_of_poles(const ps_fit *fits, int ndata);

}  // namespace psg

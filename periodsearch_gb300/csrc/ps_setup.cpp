// ps_setup.cpp -- host-side preparation of one object.
//
// Restates, in 0-based C++, the parts of the reference that run once per
// object: reading period_search_in, normalising the geometry vectors, the
// per-lightcurve sigma, weights, epoch, size guess (period_search_BOINC.cpp
// :277-485), the facet grid (:509-540, trifac.c), normals and areas
// (areanorm.c), the Laplace-series basis (sphfunc.c) and the initial
// ellipsoid (ellfit.c with ludcmp.c/lubksb.c).  The arithmetic keeps the
// reference's operation order so that the tables, and hence the starting
// point of every fit, are bit-identical to the reference's on the same libm.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "ps_host.h"

namespace psg {

namespace {

constexpr double kPi = M_PI;
constexpr double kDeg2Rad = kPi / 180;

// Vertex (theta, phi) of the Gaussian-image grid: north pole, nrows rings of
// 4i vertices, the mirrored rings, south pole.
int vertex_directions(int nrows, std::vector<double> &t, std::vector<double> &f)
{
    int ndir = 4 * nrows * nrows + 2;
    t.assign(ndir, 0.0);
    f.assign(ndir, 0.0);
    double dth = kPi / (2 * nrows);
    int k = 0;
    for (int ring = 1; ring <= nrows; ring++) {
        double dph = kPi / (2 * ring);
        for (int j = 0; j < 4 * ring; j++) {
            ++k;
            t[k] = ring * dth;
            f[k] = j * dph;
        }
    }
    for (int ring = nrows - 1; ring >= 1; ring--) {
        double dph = kPi / (2 * ring);
        for (int j = 0; j < 4 * ring; j++) {
            ++k;
            t[k] = kPi - ring * dth;
            f[k] = j * dph;
        }
    }
    t[k + 1] = kPi;
    f[k + 1] = 0;
    return k + 2;
}

// Facet vertex triplets; vertex numbers are 1-based as in the reference's
// output (trifac.c:10-82).  node(r, j) is the j-th vertex of latitude row r,
// with the first vertex of a row repeated at j = 4*row.
void facet_triplets(int nrows, std::vector<int> &ifp)
{
    int rows = 2 * nrows + 1, cols = 4 * nrows + 1;
    std::vector<int> node(static_cast<size_t>(rows) * cols, 0);
    auto at = [&](int r, int j) -> int & { return node[static_cast<size_t>(r) * cols + j]; };
    int v = 1;
    at(0, 0) = v;
    for (int r = 1; r <= nrows; r++)
        for (int j = 0; j < 4 * r; j++) {
            at(r, j) = ++v;
            if (j == 0) at(r, 4 * r) = v;
        }
    for (int r = nrows - 1; r >= 1; r--)
        for (int j = 0; j < 4 * r; j++) {
            at(2 * nrows - r, j) = ++v;
            if (j == 0) at(2 * nrows - r, 4 * r) = v;
        }
    at(2 * nrows, 0) = v + 1;

    ifp.clear();
    auto emit = [&](int p1, int p2, int p3) {
        ifp.push_back(p1);
        ifp.push_back(p2);
        ifp.push_back(p3);
    };
    for (int r = 1; r <= nrows; r++)
        for (int oct = 0; oct < 4; oct++) {
            int j0 = oct * r;
            emit(at(r - 1, j0 - oct), at(r, j0), at(r, j0 + 1));
            for (int j = j0 + 1; j <= j0 + r - 1; j++) {
                emit(at(r, j), at(r - 1, j - oct), at(r - 1, j - 1 - oct));
                emit(at(r - 1, j - oct), at(r, j), at(r, j + 1));
            }
        }
    for (int r = nrows + 1; r <= 2 * nrows; r++)
        for (int oct = 0; oct < 4; oct++) {
            int width = 2 * nrows - r;
            int j0 = oct * width;
            emit(at(r, j0), at(r - 1, j0 + 1 + oct), at(r - 1, j0 + oct));
            for (int j = j0 + 1; j <= j0 + width; j++) {
                emit(at(r, j), at(r - 1, j + oct), at(r, j - 1));
                emit(at(r, j), at(r - 1, j + 1 + oct), at(r - 1, j + oct));
            }
        }
}

// Solves the normal equations of the ellipsoid fit by Crout LU with implicit
// partial pivoting and back substitution (ludcmp.c / lubksb.c).  m is n*n
// row-major; returns false for a singular matrix.
bool lu_solve(std::vector<double> &m, int n, std::vector<double> &rhs)
{
    auto A = [&](int i, int j) -> double & { return m[static_cast<size_t>(i) * n + j]; };
    std::vector<double> rowscale(n);
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) {
        double big = 0.0;
        for (int j = 0; j < n; j++) big = std::max(big, std::fabs(A(i, j)));
        if (big == 0.0) return false;
        rowscale[i] = 1.0 / big;
    }
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < j; i++) {
            double sum = A(i, j);
            for (int k = 0; k < i; k++) sum -= A(i, k) * A(k, j);
            A(i, j) = sum;
        }
        double big = 0.0;
        int imax = -1;
        for (int i = j; i < n; i++) {
            double sum = A(i, j);
            for (int k = 0; k < j; k++) sum -= A(i, k) * A(k, j);
            A(i, j) = sum;
            double d = rowscale[i] * std::fabs(sum);
            if (d >= big) {
                big = d;
                imax = i;
            }
        }
        if (imax < 0) return false;
        if (j != imax) {
            for (int k = 0; k < n; k++) std::swap(A(imax, k), A(j, k));
            rowscale[imax] = rowscale[j];
        }
        perm[j] = imax;
        if (A(j, j) == 0.0) A(j, j) = 1.0e-20;
        if (j != n - 1) {
            double inv = 1.0 / A(j, j);
            for (int i = j + 1; i < n; i++) A(i, j) *= inv;
        }
    }
    int first = -1;
    for (int i = 0; i < n; i++) {
        int ip = perm[i];
        double sum = rhs[ip];
        rhs[ip] = rhs[i];
        if (first >= 0)
            for (int j = first; j <= i - 1; j++) sum -= A(i, j) * rhs[j];
        else if (sum)
            first = i;
        rhs[i] = sum;
    }
    for (int i = n - 1; i >= 0; i--) {
        double sum = rhs[i];
        for (int j = i + 1; j < n; j++) sum -= A(i, j) * rhs[j];
        rhs[i] = sum / A(i, i);
    }
    return true;
}

}  // namespace

void build_shape(ShapeTables &s, int nrows, int lmax, int mmax)
{
    s.nrows = nrows;
    s.lmax = lmax;
    s.mmax = mmax;
    s.nfac = 8 * nrows * nrows;
    s.ncoef = 0;
    s.npairs = 0;
    s.pair_m.clear();
    s.pair_n.clear();
    for (int m = 0; m <= mmax; m++)
        for (int l = m; l <= lmax; l++) {
            s.pair_m.push_back(m);
            s.pair_n.push_back(s.ncoef);
            s.ncoef += (m != 0) ? 2 : 1;
            s.npairs++;
        }

    std::vector<double> t, f;
    s.ndir = vertex_directions(nrows, t, f);
    facet_triplets(nrows, s.ifp);

    // Unit vectors of the vertices, then per facet the cross product of the
    // two edges from its first vertex: normal, direction angles, half area.
    // Vertex v (1-based, as stored in ifp) lives at index v-1.
    std::vector<double> x(s.ndir), y(s.ndir), z(s.ndir);
    for (int i = 0; i < s.ndir; i++) {
        double st = std::sin(t[i]);
        x[i] = st * std::cos(f[i]);
        y[i] = st * std::sin(f[i]);
        z[i] = std::cos(t[i]);
    }
    s.nor.assign(3 * s.nfac, 0.0);
    s.darea.assign(s.nfac, 0.0);
    s.at.assign(s.nfac, 0.0);
    s.af.assign(s.nfac, 0.0);
    for (int i = 0; i < s.nfac; i++) {
        int v1 = s.ifp[3 * i] - 1, v2 = s.ifp[3 * i + 1] - 1, v3 = s.ifp[3 * i + 2] - 1;
        double ax = x[v2] - x[v1], ay = y[v2] - y[v1], az = z[v2] - z[v1];
        double bx = x[v3] - x[v1], by = y[v3] - y[v1], bz = z[v3] - z[v1];
        double cx = ay * bz - by * az;
        double cy = az * bx - bz * ax;
        double cz = ax * by - bx * ay;
        double len = std::sqrt(cx * cx + cy * cy + cz * cz);
        s.nor[3 * i] = cx / len;
        s.nor[3 * i + 1] = cy / len;
        s.nor[3 * i + 2] = cz / len;
        s.at[i] = std::acos(s.nor[3 * i + 2]);
        s.af[i] = std::atan2(s.nor[3 * i + 1], s.nor[3 * i]);
        s.darea[i] = 0.5 * len;
    }

    // Polynomial coefficients c[n][l][m] of the unnormalised associated
    // Legendre functions P_l^m(cos t) = sin^m t * sum_n c[n][l][m] cos^n t,
    // by the three-term recurrence in l.
    const int L = lmax + 1;
    std::vector<double> c(static_cast<size_t>(L) * L * L, 0.0);
    auto C = [&](int n, int l, int m) -> double & { return c[(static_cast<size_t>(n) * L + l) * L + m]; };
    C(0, 0, 0) = 1;
    if (lmax >= 1) C(1, 1, 0) = 1;
    for (int l = 1; l <= lmax; l++) C(0, l, l) = C(0, l - 1, l - 1) * (2 * l - 1);
    for (int m = 0; m <= mmax; m++)
        for (int l = m + 1; l <= lmax; l++) {
            int lo;
            if (((l - m) % 2) == 0) {
                C(0, l, m) = -(l + m - 1) * C(0, l - 2, m) / (1 * (l - m));
                lo = 2;
            } else {
                lo = 1;
            }
            if (l != 1)
                for (int n = lo; n <= l - m; n += 2)
                    C(n, l, m) = ((2 * l - 1) * C(n - 1, l - 1, m) - (l + m - 1) * C(n, l - 2, m)) / (1 * (l - m));
        }

    s.fc.assign(static_cast<size_t>(s.nfac) * (mmax + 1), 0.0);
    s.fs.assign(static_cast<size_t>(s.nfac) * (mmax + 1), 0.0);
    s.pleg.assign(static_cast<size_t>(s.nfac) * s.npairs, 0.0);
    s.dsph.assign(static_cast<size_t>(s.nfac) * s.ncoef, 0.0);
    std::vector<double> sp(L), cp(L);
    for (int i = 0; i < s.nfac; i++) {
        sp[0] = 1;
        cp[0] = 1;
        if (lmax >= 1) {
            sp[1] = std::sin(s.at[i]);
            cp[1] = std::cos(s.at[i]);
        }
        for (int j = 2; j <= lmax; j++) {
            sp[j] = sp[1] * sp[j - 1];
            cp[j] = cp[1] * cp[j - 1];
        }
        double *fci = &s.fc[static_cast<size_t>(i) * (mmax + 1)];
        double *fsi = &s.fs[static_cast<size_t>(i) * (mmax + 1)];
        fsi[0] = 0;
        fci[0] = 1;
        for (int m = 1; m <= mmax; m++) {
            fsi[m] = std::sin(m * s.af[i]);
            fci[m] = std::cos(m * s.af[i]);
        }
        int q = 0, k = 0;
        for (int m = 0; m <= mmax; m++)
            for (int l = m; l <= lmax; l++, q++) {
                double p = 0;
                for (int n = ((l - m) % 2 == 0) ? 0 : 1; n <= l - m; n += 2) p = p + C(n, l, m) * cp[n] * sp[m];
                s.pleg[static_cast<size_t>(i) * s.npairs + q] = p;
                s.dsph[static_cast<size_t>(i) * s.ncoef + k++] = fci[m] * p;
                if (m != 0) s.dsph[static_cast<size_t>(i) * s.ncoef + k++] = fsi[m] * p;
            }
    }
}

bool ellipsoid_coefficients(const ShapeTables &s, double a, double b, double c, std::vector<double> &cg)
{
    const int nd = s.nfac, nc = s.ncoef;
    // Log-curvature of the ellipsoid at each facet normal.
    std::vector<double> er(nd);
    for (int i = 0; i < nd; i++) {
        double st = std::sin(s.at[i]);
        double u = a * st * std::cos(s.af[i]);
        double v = b * st * std::sin(s.af[i]);
        double w = c * std::cos(s.at[i]);
        double sum = u * u + v * v + w * w;
        er[i] = 2 * (std::log(a * b * c) - std::log(sum));
    }
    // Design matrix: the basis evaluated at the normals (same values as dsph,
    // recomputed with cos/sin of m*af as the reference does).
    std::vector<double> fm(static_cast<size_t>(nd) * nc);
    for (int i = 0; i < nd; i++) {
        int n = 0, q = 0;
        for (int m = 0; m <= s.mmax; m++)
            for (int l = m; l <= s.lmax; l++, q++) {
                double p = s.pleg[static_cast<size_t>(i) * s.npairs + q];
                if (m != 0) {
                    fm[static_cast<size_t>(i) * nc + n++] = p * std::cos(m * s.af[i]);
                    fm[static_cast<size_t>(i) * nc + n++] = p * std::sin(m * s.af[i]);
                } else {
                    fm[static_cast<size_t>(i) * nc + n++] = p;
                }
            }
    }
    std::vector<double> nm(static_cast<size_t>(nc) * nc), rhs(nc);
    for (int i = 0; i < nc; i++) {
        for (int j = 0; j < nc; j++) {
            double acc = 0;
            for (int k = 0; k < nd; k++) acc = acc + fm[static_cast<size_t>(k) * nc + i] * fm[static_cast<size_t>(k) * nc + j];
            nm[static_cast<size_t>(i) * nc + j] = acc;
        }
        double acc = 0;
        for (int k = 0; k < nd; k++) acc = acc + fm[static_cast<size_t>(k) * nc + i] * er[k];
        rhs[i] = acc;
    }
    if (!lu_solve(nm, nc, rhs)) return false;
    cg = rhs;
    return true;
}

ps_status prepare_object(const ps_problem &p, HostObject &o, std::string &err)
{
    const ps_header &h = p.hdr;
    if (p.n_lc < 1 || !p.lc_points || !p.jd || !p.brightness || !p.sun || !p.earth) {
        err = "ps_problem: missing arrays or no lightcurves";
        return PS_ERR_ARG;
    }
    if (p.n_lc > PS_MAX_LC) {
        err = "number of lightcurves exceeds PS_MAX_LC";
        return PS_ERR_LIMIT;
    }
    if (h.lmax < 0 || h.mmax < 0 || h.mmax > h.lmax || h.lmax > PS_MAX_LM || h.nrows < 1) {
        err = "bad Laplace-series degree/order or nrows";
        return PS_ERR_ARG;
    }
    if (8 * h.nrows * h.nrows > PS_MAX_N_FAC) {
        err = "number of facets exceeds PS_MAX_N_FAC";
        return PS_ERR_LIMIT;
    }
    o.hdr = h;
    o.n_lc = p.n_lc;
    o.lc_points.assign(p.n_lc + 1, 0);
    o.lc_rel.assign(p.n_lc + 1, 0);
    o.lc_start.assign(p.n_lc + 1, 0);
    int nd = 0;
    for (int i = 0; i < p.n_lc; i++) {
        int np = p.lc_points[i];
        if (np < 1 || np > PS_POINTS_MAX) {
            err = "lightcurve point count outside 1..PS_POINTS_MAX";
            return PS_ERR_LIMIT;
        }
        o.lc_points[i] = np;
        o.lc_rel[i] = p.lc_calibrated ? (1 - p.lc_calibrated[i]) : 1;
        o.lc_start[i] = nd;
        nd += np;
    }
    if (nd != p.ndata) {
        err = "ndata differs from the sum of lc_points";
        return PS_ERR_ARG;
    }
    if (nd > PS_MAX_N_OBS) {
        err = "number of points exceeds PS_MAX_N_OBS";
        return PS_ERR_LIMIT;
    }
    o.ndata = nd;
    o.lc_points[p.n_lc] = 3;
    o.lc_rel[p.n_lc] = 0;
    o.lc_start[p.n_lc] = nd;
    o.tim.assign(nd + 3, 0.0);
    o.bright.assign(nd + 3, 0.0);
    o.sig.assign(nd + 3, 0.0);
    o.weight.assign(nd + 3, 1.0);
    o.ee.assign(3 * static_cast<size_t>(nd), 0.0);
    o.ee0.assign(3 * static_cast<size_t>(nd), 0.0);

    double al0 = kPi, al0_abs = kPi;
    int ial0 = -1, ial0_abs = -1;
    double jd_min = 1e20, jd_max = -1e40;
    o.onlyrel = true;
    o.max_rel_points = 0;
    for (int i = 0; i < p.n_lc; i++) {
        if (o.lc_rel[i] == 0) o.onlyrel = false;
        else o.max_rel_points = std::max(o.max_rel_points, o.lc_points[i]);
        double ave = 0;
        for (int j = 0; j < o.lc_points[i]; j++) {
            int q = o.lc_start[i] + j;
            const double *e0 = &p.sun[3 * static_cast<size_t>(q)];
            const double *e = &p.earth[3 * static_cast<size_t>(q)];
            o.tim[q] = p.jd[q];
            o.bright[q] = p.brightness[q];
            if (o.tim[q] < jd_min) jd_min = o.tim[q];
            if (o.tim[q] > jd_max) jd_max = o.tim[q];
            double e0len = std::sqrt(e0[0] * e0[0] + e0[1] * e0[1] + e0[2] * e0[2]);
            double elen = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            ave += o.bright[q];
            for (int k = 0; k < 3; k++) {
                o.ee[3 * static_cast<size_t>(q) + k] = e[k] / elen;
                o.ee0[3 * static_cast<size_t>(q) + k] = e0[k] / e0len;
            }
            if (j == 0) {
                // Solar phase angle of the lightcurve's first point.
                double ca = (e[0] * e0[0] + e[1] * e0[1] + e[2] * e0[2]) / (elen * e0len);
                double al = std::acos(ca);
                if (al < al0) {
                    al0 = al;
                    ial0 = q;
                }
                if (al < al0_abs && o.lc_rel[i] == 0) {
                    al0_abs = al;
                    ial0_abs = q;
                }
            }
        }
        ave /= o.lc_points[i];
        for (int j = 0; j < o.lc_points[i]; j++) o.sig[o.lc_start[i] + j] = ave;
    }

    o.jd0 = h.jd00;
    if (o.jd0 <= 0) o.jd0 = static_cast<int>(jd_min);
    for (int q = 0; q < nd; q++) o.tim[q] = o.tim[q] - o.jd0;
    o.phi0 = h.phi0_deg * kDeg2Rad;
    for (int i = 0; i < p.n_lc; i++) {
        double w = p.lc_weight ? p.lc_weight[i] : -1.0;
        for (int j = 0; j < o.lc_points[i]; j++) o.weight[o.lc_start[i] + j] = (w == -1) ? 1 : w;
    }
    for (int j = 0; j < 3; j++) o.weight[nd + j] = 1;
    if (!o.onlyrel) {
        al0 = al0_abs;
        ial0 = ial0_abs;
    }
    if (ial0 < 0) {
        err = "no lightcurve with a defined solar phase angle";
        return PS_ERR_ARG;
    }
    double a = 1.05, b = 1.00, c = 0.95;
    double rfit = std::sqrt(2 * o.sig[ial0] / (0.5 * kPi * (1 + std::cos(al0))));
    double escl = rfit / std::sqrt((a * b + b * c + a * c) / 3);
    if (!o.onlyrel) escl *= 0.8;
    o.escl = escl;
    o.a = a * escl;
    o.b = b * escl;
    o.c = c * escl;
    o.jd_min = jd_min;
    o.jd_max = jd_max;
    o.conw_r0 = h.conw / escl / escl;

    build_shape(o.shape, h.nrows, h.lmax, h.mmax);
    o.ncoef = o.shape.ncoef;
    o.ma = o.ncoef + 5 + kNPhPar;
    if (o.ncoef + 3 + kNPhPar + 1 > PS_MAX_N_PAR) {
        err = "number of parameters exceeds PS_MAX_N_PAR";
        return PS_ERR_LIMIT;
    }
    if (!ellipsoid_coefficients(o.shape, o.a, o.b, o.c, o.cg_first)) {
        err = "singular matrix in the ellipsoid fit";
        return PS_ERR_SINGULAR;
    }
    o.freq_start = 1 / h.per_start;
    o.freq_end = 1 / h.per_end;
    o.freq_step = 0.5 / (jd_max - jd_min) / 24 * h.per_step_coef;
    o.n_max = static_cast<int64_t>((o.freq_start - o.freq_end) / o.freq_step) + 1;

    // Free-parameter mask (period_search_BOINC.cpp:788-802).
    int nc = o.ncoef;
    o.ia.assign(o.ma, 0);
    for (int i = 0; i < nc; i++) o.ia[i] = 1;
    if (o.onlyrel) o.ia[0] = 0;
    o.ia[nc] = 1;
    o.ia[nc + 1] = 1;
    o.ia[nc + 2] = h.ia_prd;
    for (int i = 0; i < kNPhPar; i++) o.ia[nc + 3 + i] = h.ia_par[i];
    o.ia[nc + 3 + kNPhPar] = h.ia_cl;
    o.ia[nc + 4 + kNPhPar] = 0;
    o.free_list.clear();
    for (int l = 0; l < o.ma; l++)
        if (o.ia[l]) o.free_list.push_back(l);
    o.mfit = static_cast<int>(o.free_list.size());
    set_convexity_rows(o, o.conw_r0);
    return PS_OK;
}

ps_status prepare_object_state(const ps_state &st, HostObject &o, std::string &err)
{
    if (st.n_lc < 1 || !st.lc_points || !st.lc_rel || !st.tim || !st.brightness || !st.sig || !st.weight || !st.ee ||
        !st.ee0 || !st.ia || !st.cg_first) {
        err = "ps_state: missing arrays or no lightcurves";
        return PS_ERR_ARG;
    }
    if (st.n_lc > PS_MAX_LC) {
        err = "number of lightcurves exceeds PS_MAX_LC";
        return PS_ERR_LIMIT;
    }
    if (st.lmax < 0 || st.mmax < 0 || st.mmax > st.lmax || st.lmax > PS_MAX_LM || st.nrows < 1) {
        err = "bad Laplace-series degree/order or nrows";
        return PS_ERR_ARG;
    }
    if (8 * st.nrows * st.nrows > PS_MAX_N_FAC) {
        err = "number of facets exceeds PS_MAX_N_FAC";
        return PS_ERR_LIMIT;
    }
    if (!(st.freq_step > 0) || !(st.escl > 0) || !(st.conw_r > 0) || !(st.cl > 0)) {
        err = "ps_state: frequency step, escl, conw_r and cl must be positive";
        return PS_ERR_ARG;
    }
    ps_header h{};
    h.lmax = st.lmax;
    h.mmax = st.mmax;
    h.nrows = st.nrows;
    for (int k = 0; k < 3; k++) h.par[k] = st.par[k];
    h.cl = st.cl;
    h.alamda_start = st.alamda_start;
    h.alamda_incr = st.alamda_incr;
    h.stop_condition = st.stop_condition;
    h.n_iter_min = st.n_iter_min;
    o.hdr = h;
    o.n_lc = st.n_lc;
    o.lc_points.assign(st.n_lc + 1, 0);
    o.lc_rel.assign(st.n_lc + 1, 0);
    o.lc_start.assign(st.n_lc + 1, 0);
    int nd = 0;
    o.onlyrel = true;
    o.max_rel_points = 0;
    for (int i = 0; i < st.n_lc; i++) {
        const int np = st.lc_points[i];
        if (np < 1 || np > PS_POINTS_MAX) {
            err = "lightcurve point count outside 1..PS_POINTS_MAX";
            return PS_ERR_LIMIT;
        }
        o.lc_points[i] = np;
        o.lc_rel[i] = st.lc_rel[i] ? 1 : 0;
        o.lc_start[i] = nd;
        if (!o.lc_rel[i]) o.onlyrel = false;
        else o.max_rel_points = std::max(o.max_rel_points, np);
        nd += np;
    }
    if (nd != st.ndata || nd > PS_MAX_N_OBS) {
        err = "ndata differs from the sum of lc_points or exceeds PS_MAX_N_OBS";
        return PS_ERR_ARG;
    }
    o.ndata = nd;
    o.lc_points[st.n_lc] = 3;
    o.lc_rel[st.n_lc] = 0;
    o.lc_start[st.n_lc] = nd;
    o.tim.assign(st.tim, st.tim + nd);
    o.bright.assign(st.brightness, st.brightness + nd);
    o.sig.assign(st.sig, st.sig + nd);
    o.weight.assign(st.weight, st.weight + nd);
    for (int j = 0; j < 3; j++) {
        o.tim.push_back(0.0);
        o.bright.push_back(0.0);
        o.sig.push_back(0.0);
        o.weight.push_back(1.0);
    }
    o.ee.assign(st.ee, st.ee + 3 * static_cast<size_t>(nd));
    o.ee0.assign(st.ee0, st.ee0 + 3 * static_cast<size_t>(nd));
    o.phi0 = st.phi0;
    o.escl = st.escl;
    o.conw_r0 = st.conw_r;
    o.freq_start = st.freq_start;
    o.freq_end = st.freq_end;
    o.freq_step = st.freq_step;
    o.n_max = static_cast<int64_t>((o.freq_start - o.freq_end) / o.freq_step) + 1;
    build_shape(o.shape, st.nrows, st.lmax, st.mmax);
    o.ncoef = o.shape.ncoef;
    o.ma = o.ncoef + 5 + kNPhPar;
    if (o.ncoef + 3 + kNPhPar + 1 > PS_MAX_N_PAR) {
        err = "number of parameters exceeds PS_MAX_N_PAR";
        return PS_ERR_LIMIT;
    }
    o.cg_first.assign(st.cg_first, st.cg_first + o.ncoef);
    o.ia.assign(st.ia, st.ia + o.ma);
    o.hdr.ia_prd = o.ia[o.ncoef + 2];
    for (int i = 0; i < kNPhPar; i++) o.hdr.ia_par[i] = o.ia[o.ncoef + 3 + i];
    o.hdr.ia_cl = o.ia[o.ncoef + 3 + kNPhPar];
    o.free_list.clear();
    for (int l = 0; l < o.ma; l++)
        if (o.ia[l]) o.free_list.push_back(l);
    o.mfit = static_cast<int>(o.free_list.size());
    set_convexity_rows(o, o.conw_r0);
    return PS_OK;
}

void set_convexity_rows(HostObject &o, double conw_r)
{
    for (int j = 0; j < 3; j++) {
        o.bright[o.ndata + j] = 0;
        o.sig[o.ndata + j] = 1 / conw_r;
    }
}

ps_row best_of_poles(const ps_fit *fits, int ndata)
{
    double per_best_h = 0, dark_best = 0, la_best = 0, be_best = 0, dev_best = 1e40;
    for (int m = 0; m < PS_N_POLES; m++) {
        const ps_fit &f = fits[m];
        if (f.dev < dev_best) {
            dev_best = f.dev;
            per_best_h = f.period_h;
            dark_best = f.dark / f.totarea * 100;
            la_best = f.lambda_deg;
            be_best = f.beta_deg;
        }
    }
    if (la_best < 0) la_best += 360;
    ps_row r;
    r.period_h = per_best_h;
    r.rms = dev_best;
    r.chi2 = dev_best * dev_best * ndata;
    r.dark_or_conw = dark_best;
    r.lambda_deg = la_best;
    r.beta_deg = be_best;
    return r;
}

// ---- period_search_in reader ----------------------------------------------

namespace {

// Token reader with the two operations the reference's parser uses:
// scanf-style numbers (leading whitespace, newlines included, skipped) and
// "discard the rest of the current line".
struct Reader {
    const char *p, *end;
    void skip_ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r' || *p == '\v' || *p == '\f')) ++p;
    }
    bool num(double &v)
    {
        skip_ws();
        if (p >= end) return false;
        char *e = nullptr;
        v = std::strtod(p, &e);
        if (e == p) return false;
        p = e;
        return true;
    }
    bool num(int32_t &v)
    {
        skip_ws();
        if (p >= end) return false;
        char *e = nullptr;
        long x = std::strtol(p, &e, 10);
        if (e == p) return false;
        p = e;
        v = static_cast<int32_t>(x);
        return true;
    }
    void rest_of_line()
    {
        while (p < end && *p != '\n') ++p;
        if (p < end) ++p;
    }
};

}  // namespace

ps_status parse_input_file(const std::string &path, ParsedInput &in, std::string &err)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open input file " + path;
        return PS_ERR_IO;
    }
    std::string text;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    std::fclose(f);
    Reader r{text.data(), text.data() + text.size()};
    ps_header &h = in.hdr;
    bool ok = r.num(h.per_start) && r.num(h.per_step_coef) && r.num(h.per_end) && r.num(h.ia_prd);
    r.rest_of_line();
    ok = ok && r.num(h.jd00);
    r.rest_of_line();
    ok = ok && r.num(h.phi0_deg);
    r.rest_of_line();
    ok = ok && r.num(h.conw);
    r.rest_of_line();
    ok = ok && r.num(h.lmax) && r.num(h.mmax);
    r.rest_of_line();
    ok = ok && r.num(h.nrows);
    r.rest_of_line();
    for (int i = 0; i < 3; i++) {
        ok = ok && r.num(h.par[i]) && r.num(h.ia_par[i]);
        r.rest_of_line();
    }
    ok = ok && r.num(h.cl) && r.num(h.ia_cl);
    r.rest_of_line();
    ok = ok && r.num(h.stop_condition);
    r.rest_of_line();
    ok = ok && r.num(h.n_iter_min);
    r.rest_of_line();
    ok = ok && r.num(h.alamda_incr);
    r.rest_of_line();
    ok = ok && r.num(h.alamda_start);
    r.rest_of_line();
    int32_t lcurves = 0;
    ok = ok && r.num(lcurves);
    if (!ok) {
        err = "malformed period_search_in header";
        return PS_ERR_IO;
    }
    if (lcurves > PS_MAX_LC || lcurves < 1) {
        err = "number of lightcurves outside 1..PS_MAX_LC";
        return PS_ERR_LIMIT;
    }
    int total = 0;
    for (int i = 0; i < lcurves; i++) {
        int32_t np = 0, flag = 0;
        if (!(r.num(np) && r.num(flag))) {
            err = "malformed lightcurve header";
            return PS_ERR_IO;
        }
        r.rest_of_line();
        if (np > PS_POINTS_MAX || np < 1) {
            err = "lightcurve point count outside 1..PS_POINTS_MAX";
            return PS_ERR_LIMIT;
        }
        total += np;
        if (total > PS_MAX_N_OBS) {
            err = "number of points exceeds PS_MAX_N_OBS";
            return PS_ERR_LIMIT;
        }
        in.lc_points.push_back(np);
        in.lc_calibrated.push_back(flag);
        for (int j = 0; j < np; j++) {
            double v[8];
            for (int k = 0; k < 8; k++)
                if (!r.num(v[k])) {
                    err = "truncated lightcurve data";
                    return PS_ERR_IO;
                }
            in.jd.push_back(v[0]);
            in.brightness.push_back(v[1]);
            for (int k = 0; k < 3; k++) in.sun.push_back(v[2 + k]);
            for (int k = 0; k < 3; k++) in.earth.push_back(v[5 + k]);
        }
    }
    // Trailing "lightcurve weight" pairs (period_search_BOINC.cpp:416-427);
    // an incomplete pair at the end is ignored.
    in.lc_weight.assign(lcurves, -1.0);
    for (;;) {
        int32_t lc;
        double w;
        if (!r.num(lc) || !r.num(w)) break;
        if (lc >= 1 && lc <= lcurves) in.lc_weight[lc - 1] = w;
    }
    return PS_OK;
}

}  // namespace psg

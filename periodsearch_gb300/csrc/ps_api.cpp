// ps_api.cpp -- C ABI of the GB300 period-search engine (ps_gb300.h).
//
// A context owns one prepared object: its host copy (HostObject), one device
// allocation holding every table, the per-slot scratch, the result buffers
// and a CUDA stream with timing events.  Scans launch the persistent fit
// kernel once per call; the best-of-poles reduction of the (at most a few
// hundred kB of) per-fit results runs on the host in the reference's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ps_engine.h"
#include "ps_host.h"

struct ps_input {
    psg::ParsedInput data;
};

// Launch plan of one arithmetic form: point-tile size, shared memory, slots.
struct FormPlan {
    bool ready = false;
    int P = 16, dsph_smem = 0, slots = 0;
    int rel_rows = 0;   // relative-lightcurve rows parked in shared memory (0: global scratch)
    size_t smem = 0;
};

struct ps_ctx {
    psg::HostObject obj;
    ps_options opt{};
    FormPlan plan[2];
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    char *d_tables = nullptr;          // one allocation with every table
    psg::DevObject dob{};
    int sm_count = 0, slots = 0, P = 16, dsph_smem = 0, rel_rows = 0;
    int64_t h2d_bytes = 0;
    size_t smem = 0;
    double *d_scratch = nullptr;
    size_t scratch_stride = 0;
    unsigned long long *d_queue = nullptr;
    ps_fit *d_out = nullptr;
    size_t out_cap = 0;
    int64_t *d_pidx = nullptr;
    int *d_pole = nullptr;
    size_t list_cap = 0;
    int64_t launch_total = 0;   // fit-kernel launches since ps_prepare
    double *d_eval = nullptr;          // cg, alpha, beta, chisq, area of ps_eval
    double *d_state = nullptr;         // saved LM states of screened fits (learned scan)
    size_t state_cap = 0;              // fits
    int64_t *d_slot = nullptr;         // state rows of resumed fits
    size_t slot_cap = 0;
    double *d_alpha_g = nullptr;       // per-slot normal matrices of the wide tensor-core path
    size_t alpha_g_slots = 0;
    std::vector<ps_fit> h_fits;
    ps_timing timing{};
    std::string err;
};

namespace {

ps_status cuda_fail(ps_ctx *c, cudaError_t e, const char *what)
{
    if (c) c->err = std::string(what) + ": " + cudaGetErrorString(e);
    return PS_ERR_CUDA;
}

#define PSG_CUDA(ctx, call)                                        \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call); \
    } while (0)

// Packs host arrays into one device allocation, 256-byte aligned each.
struct Packer {
    std::vector<char> bytes;
    template <class T>
    size_t add(const std::vector<T> &v)
    {
        size_t off = (bytes.size() + 255) & ~size_t(255);
        bytes.resize(off + std::max<size_t>(v.size() * sizeof(T), 1));
        if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

psg::FitConfig make_config(const ps_ctx *c, double conw_r)
{
    const psg::HostObject &o = c->obj;
    const ps_header &h = o.hdr;
    psg::FitConfig f{};
    f.phi0 = o.phi0;
    f.alamda_start = h.alamda_start;
    f.alamda_incr = h.alamda_incr;
    f.conw_r = conw_r;
    f.conv_sig = 1 / conw_r;
    f.freq_start = o.freq_start;
    f.freq_step = o.freq_step;
    f.log_cl = std::log(h.cl);
    f.par0 = h.par[0];
    f.par1 = h.par[1];
    f.par2 = h.par[2];
    // Stop rule of period_search_BOINC.cpp:847-860.
    f.n_iter_max = 0;
    f.iter_diff_max = -1;
    f.n_iter_min = h.n_iter_min;
    if (h.stop_condition > 1) {
        f.n_iter_max = static_cast<int>(h.stop_condition);
        f.iter_diff_max = 0;
        f.n_iter_min = 0;
    }
    if (h.stop_condition < 1) {
        f.n_iter_max = 100;  // MAX_N_ITER, period_search/constants.h:6
        f.iter_diff_max = h.stop_condition;
    }
    return f;
}

ps_status ensure_out(ps_ctx *c, size_t nfits)
{
    if (nfits <= c->out_cap) return PS_OK;
    if (c->d_out) cudaFree(c->d_out);
    c->d_out = nullptr;
    size_t cap = std::max(nfits, size_t(1024));
    PSG_CUDA(c, cudaMalloc(&c->d_out, cap * sizeof(ps_fit)));
    c->out_cap = cap;
    return PS_OK;
}

// Plan of one form for a given basis mode and tile size: shared-memory
// layout, kernel attribute and resident slots (at most per_sm_cap per SM when
// positive).  PS_ERR_LIMIT when the slot does not fit.  The rows of the
// relative lightcurves live in shared memory when they fit without costing
// a resident slot (they are re-read by the second pass over each relative
// lightcurve), else in the per-slot global scratch.
ps_status build_plan(ps_ctx *c, int form, int dsph_smem, int P, int per_sm_cap, FormPlan *out)
{
    const psg::HostObject &o = c->obj;
    const int F = o.shape.nfac;
    cudaDeviceProp prop;
    PSG_CUDA(c, cudaGetDeviceProperties(&prop, c->opt.device));
    const size_t smem_max = static_cast<size_t>(prop.sharedMemPerBlockOptin);
    if (dsph_smem == psg::kBasisTensor && !psg::tensor_basis_ok(F, o.ncoef, o.mfit, P)) return PS_ERR_LIMIT;
    if (dsph_smem == psg::kBasisTensorWide && !psg::tensor_wide_ok(F, o.ncoef, o.mfit, P)) return PS_ERR_LIMIT;
    const psg::SlotLayout L = psg::make_layout(form, o.ma, o.mfit, F, o.ncoef, P, dsph_smem);
    if (L.bytes > smem_max) return PS_ERR_LIMIT;
    // A tensor-core slot holds up to 512 Tensor Memory columns for its whole
    // life: request enough shared memory that only one slot fits on an SM.
    const size_t floor_tc = static_cast<size_t>(prop.sharedMemPerMultiprocessor) / 2 + 1024;
    size_t bytes = L.bytes;
    if (psg::basis_on_tensor(dsph_smem)) bytes = std::min(smem_max, std::max(bytes, floor_tc));
    int e = psg::set_kernel_smem(form, bytes, o.ncoef, dsph_smem);
    if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "cudaFuncSetAttribute");
    int per_sm = 0;
    e = psg::occupancy_slots(form, bytes, o.ncoef, dsph_smem, &per_sm);
    if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "occupancy");
    int rel_rows = 0;
    if (o.max_rel_points > 0) {
        const psg::SlotLayout Lr = psg::make_layout(form, o.ma, o.mfit, F, o.ncoef, P, dsph_smem, o.max_rel_points);
        const size_t need = psg::basis_on_tensor(dsph_smem) ? std::max(Lr.bytes, floor_tc) : Lr.bytes;
        if (Lr.bytes <= smem_max) {
            e = psg::set_kernel_smem(form, need, o.ncoef, dsph_smem);
            if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "cudaFuncSetAttribute");
            int per_sm_r = 0;
            e = psg::occupancy_slots(form, need, o.ncoef, dsph_smem, &per_sm_r);
            if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "occupancy");
            const int cap = per_sm_cap > 0 ? per_sm_cap : 1 << 20;
            if (std::min(per_sm_r, cap) >= std::min(per_sm, cap)) {
                rel_rows = o.max_rel_points;
                bytes = need;
                per_sm = per_sm_r;
            } else {
                e = psg::set_kernel_smem(form, bytes, o.ncoef, dsph_smem);
                if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "cudaFuncSetAttribute");
            }
        }
    }
    if (per_sm < 1) return PS_ERR_LIMIT;
    if (per_sm_cap > 0) per_sm = std::min(per_sm, per_sm_cap);
    if (psg::basis_on_tensor(dsph_smem) && per_sm > 1) {
        c->err = "tensor-core fit slots would share an SM";
        return PS_ERR_LIMIT;
    }
    out->P = P;
    out->dsph_smem = dsph_smem;
    out->rel_rows = rel_rows;
    out->smem = bytes;
    out->slots = per_sm * c->sm_count;
    out->ready = true;
    return PS_OK;
}

// Default plan of one form: 32-point tiles (halved until a slot fits); the
// mixed form with the tensor-core contraction where the shape tables allow
// it, else the SIMT contraction with the FP32 basis in shared memory when it
// fits (else in L2).  The FP64 form's results do not depend on the tile
// size (its sums run in data order); 32 points measured fastest.
ps_status make_plan(ps_ctx *c, int form)
{
    FormPlan &pl = c->plan[form];
    if (pl.ready) return PS_OK;
    const psg::HostObject &o = c->obj;
    const bool mixed = form == PS_FORM_MIXED;
    int modes[3], nm = 0;
    if (mixed) {
        if (!(c->opt.flags & PS_FLAG_NO_TENSOR) && psg::tensor_basis_ok(o.shape.nfac, o.ncoef, o.mfit, 32))
            modes[nm++] = psg::kBasisTensor;
        else if (!(c->opt.flags & PS_FLAG_NO_TENSOR) && psg::tensor_wide_ok(o.shape.nfac, o.ncoef, o.mfit, 32))
            modes[nm++] = psg::kBasisTensorWide;
        modes[nm++] = psg::kBasisSmem;
    }
    modes[nm++] = psg::kBasisGlobal;
    for (int P = 32; P >= 2; P /= 2)
        for (int k = 0; k < nm; k++) {
            FormPlan cand;
            const ps_status st = build_plan(c, form, modes[k], P, c->opt.ctas_per_sm, &cand);
            if (st == PS_OK) {
                pl = cand;
                return PS_OK;
            }
            if (st != PS_ERR_LIMIT) return st;
        }
    c->err = "shared-memory plan of a fit slot exceeds the device limit";
    return PS_ERR_LIMIT;
}

// CTAs per fit for a launch: FP64 fits without trajectories, saved states
// or an iteration limit, fewer than the fit slots, are each spread over a
// thread-block cluster of 2 or 4 CTAs (the most that the slots hold).
int split_size(const ps_ctx *c, const psg::FitWork &w, int form)
{
    if (form != PS_FORM_FP64 || w.traj || w.state || w.iter_limit > 0 || w.nfits < 1) return 1;
    const int64_t slots = c->plan[form].slots;
    if (w.nfits * 4 <= slots) return 4;
    if (w.nfits * 2 <= slots) return 2;
    return 1;
}

// Launches the fits described by w in the given form (queue and outputs
// filled in here) and copies the results back into c->h_fits.
ps_status run_fits(ps_ctx *c, double conw_r, psg::FitWork w, int form)
{
    ps_status st = make_plan(c, form);
    if (st != PS_OK) return st;
    const FormPlan &pl = c->plan[form];
    if (pl.slots > c->slots) {
        // a second form with more slots than the scratch was sized for
        cudaFree(c->d_scratch);
        c->d_scratch = nullptr;
        PSG_CUDA(c, cudaMalloc(&c->d_scratch, c->scratch_stride * pl.slots * sizeof(double)));
        c->slots = pl.slots;
    }
    psg::FitConfig cfg = make_config(c, conw_r);
    st = ensure_out(c, static_cast<size_t>(w.nfits));
    if (st != PS_OK) return st;
    w.queue = c->d_queue;
    w.lit = c->d_queue + 1;   // the lit facet-point counter of the FP64 form
    w.scratch = c->d_scratch;
    w.scratch_stride = c->scratch_stride;
    w.rel_rows = pl.rel_rows;
    w.out = c->d_out;
    if (pl.dsph_smem == psg::kBasisTensorWide) {
        // the wide tensor-core path keeps each slot's normal matrix in global memory
        const size_t stride = static_cast<size_t>(c->obj.mfit) * c->obj.mfit;
        if (c->alpha_g_slots < static_cast<size_t>(pl.slots)) {
            cudaFree(c->d_alpha_g);
            c->d_alpha_g = nullptr;
            c->alpha_g_slots = 0;
            PSG_CUDA(c, cudaMalloc(&c->d_alpha_g, stride * pl.slots * sizeof(double)));
            c->alpha_g_slots = static_cast<size_t>(pl.slots);
        }
        w.alpha_g = c->d_alpha_g;
        w.alpha_stride = stride;
    }
    int grid = static_cast<int>(std::min<int64_t>(pl.slots, std::max<int64_t>(w.nfits, 1)));
    // FP64 fits fewer than the slots: each fit spread over a cluster of
    // CTAs (bit-identical results, a shorter launch)
    const int cs = split_size(c, w, form);
    PSG_CUDA(c, cudaMemsetAsync(c->d_queue, 0, 2 * sizeof(unsigned long long), c->stream));
    PSG_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    int e;
    if (cs > 1) {
        int clusters = 0;
        e = psg::split_max_clusters(cs, pl.smem, &clusters);
        if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "cluster occupancy");
        clusters = static_cast<int>(std::min<int64_t>(std::max(clusters, 1), w.nfits));
        e = psg::launch_fits_split(c->dob, cfg, w, clusters, cs, pl.P, pl.smem, c->stream);
    } else {
        e = psg::launch_fits(form, c->dob, cfg, w, grid, pl.P, pl.smem, pl.dsph_smem, c->stream);
    }
    if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "fit kernel launch");
    PSG_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
    c->h_fits.resize(static_cast<size_t>(w.nfits));
    PSG_CUDA(c, cudaMemcpyAsync(c->h_fits.data(), c->d_out, w.nfits * sizeof(ps_fit), cudaMemcpyDeviceToHost,
                                c->stream));
    unsigned long long lit = 0;
    PSG_CUDA(c, cudaMemcpyAsync(&lit, c->d_queue + 1, sizeof(lit), cudaMemcpyDeviceToHost, c->stream));
    PSG_CUDA(c, cudaEventRecord(c->ev[2], c->stream));
    PSG_CUDA(c, cudaStreamSynchronize(c->stream));
    float k_ms = 0, t_ms = 0;
    cudaEventElapsedTime(&k_ms, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&t_ms, c->ev[0], c->ev[2]);
    c->timing.kernel_ms = k_ms;
    c->timing.total_ms = t_ms;
    c->timing.fits = w.nfits;
    int64_t evals = 0;
    for (const ps_fit &f : c->h_fits) evals += f.niter + 1;
    c->timing.evals = evals;
    c->timing.launches = 1;
    c->timing.cluster_size = cs;
    c->timing.lit_facets = static_cast<int64_t>(lit);
    c->launch_total++;
    for (const ps_fit &f : c->h_fits)
        if (f.err_code == 16) {
            c->err = "a tensor-core wait gave up: fit results are incomplete";
            return PS_ERR_TIMEOUT;
        }
    return PS_OK;
}

ps_status scan_rows(ps_ctx *c, double conw_r, int64_t n_lo, int64_t n_hi, ps_row *out, bool prepass)
{
    psg::FitWork w{};
    w.n_lo = n_lo;
    w.nfits = (n_hi - n_lo + 1) * PS_N_POLES;
    // the convexity-weight pre-pass always takes the FP64 form: its decision
    // is a threshold on a mean over few fits, which the mixed form's
    // rounding can move across on an object that sits near it
    ps_status st = run_fits(c, conw_r, w, prepass ? PS_FORM_FP64 : c->opt.form);
    if (st != PS_OK) return st;
    for (int64_t n = n_lo; n <= n_hi; n++) {
        ps_row r = psg::best_of_poles(&c->h_fits[static_cast<size_t>(n - n_lo) * PS_N_POLES], c->obj.ndata);
        if (prepass && std::isnan(r.dark_or_conw)) r.dark_or_conw = 1.0;
        out[n - n_lo] = r;
    }
    return PS_OK;
}

// Fits given as (period index, pole) lists on the host: copied to the
// device and launched in the given form; results in c->h_fits.
ps_status run_list(ps_ctx *c, double conw_r, const int64_t *pidx, const int32_t *pole, int64_t n, int form,
                   int iter_limit = 0, const int64_t *resume_slots = nullptr)
{
    if (static_cast<size_t>(n) > c->list_cap) {
        cudaFree(c->d_pidx);
        cudaFree(c->d_pole);
        c->d_pidx = nullptr;
        c->d_pole = nullptr;
        PSG_CUDA(c, cudaMalloc(&c->d_pidx, n * sizeof(int64_t)));
        PSG_CUDA(c, cudaMalloc(&c->d_pole, n * sizeof(int)));
        c->list_cap = static_cast<size_t>(n);
    }
    PSG_CUDA(c, cudaMemcpyAsync(c->d_pidx, pidx, n * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
    PSG_CUDA(c, cudaMemcpyAsync(c->d_pole, pole, n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    psg::FitWork w{};
    w.n_lo = 1;
    w.nfits = n;
    w.period_index = c->d_pidx;
    w.pole = c->d_pole;
    w.iter_limit = iter_limit;
    if (resume_slots) {
        // continue fits from the states a screening launch saved
        if (static_cast<size_t>(n) > c->slot_cap) {
            cudaFree(c->d_slot);
            c->d_slot = nullptr;
            PSG_CUDA(c, cudaMalloc(&c->d_slot, n * sizeof(int64_t)));
            c->slot_cap = static_cast<size_t>(n);
        }
        PSG_CUDA(c, cudaMemcpyAsync(c->d_slot, resume_slots, n * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
        w.state = c->d_state;
        w.state_slot = c->d_slot;
        w.resume = 1;
    }
    return run_fits(c, conw_r, w, form);
}

// The fits of a scan window on the host: period n_lo + i / 10, pole i % 10 + 1.
struct ScanFits {
    int64_t n_lo = 1, nper = 0;
    std::vector<ps_fit> fits;
    std::vector<char> done;     // run in full (a candidate of its period's row)
    std::vector<char> fp64;     // period refitted in full by the FP64 form

    // The row of period n from its fits run in full; a period none of whose
    // fits ran in full (the learned scan skipped it) gets the row of its
    // screened fits, whose rms after the screening iterations lies above
    // what the full fits would reach.
    ps_row row(int64_t n, int32_t ndata) const
    {
        ps_fit tmp[PS_N_POLES];
        bool any = false;
        for (int m = 0; m < PS_N_POLES; m++) any = any || done[static_cast<size_t>(n * PS_N_POLES + m)];
        for (int m = 0; m < PS_N_POLES; m++) {
            tmp[m] = fits[static_cast<size_t>(n * PS_N_POLES + m)];
            if (any && !done[static_cast<size_t>(n * PS_N_POLES + m)]) tmp[m].dev = NAN;  // not a candidate
        }
        return psg::best_of_poles(tmp, ndata);
    }
    void rows(std::vector<ps_row> &r, int32_t ndata) const
    {
        r.resize(static_cast<size_t>(nper));
        for (int64_t n = 0; n < nper; n++) r[static_cast<size_t>(n)] = row(n, ndata);
    }
    static int64_t best(const std::vector<ps_row> &r)
    {
        int64_t b = 0;
        for (size_t n = 1; n < r.size(); n++)
            if (r[n].rms < r[static_cast<size_t>(b)].rms) b = static_cast<int64_t>(n);
        return b;
    }
};

// Refits in full by the FP64 form every period whose row lies within
// rel (relative) of the best row or within halfwidth periods of it, and
// repeats with the new rows until the set is closed: the best row and its
// neighbourhood then carry FP64 values, and no row outside the set comes
// within rel of it.  A refit launch takes one FP64 fit's time whether it
// fills the device's fit slots or not, so each launch is topped up with the
// next-lowest rows (whole periods) until its last wave of slots is full:
// periods that a later round would likely have needed come at no extra
// time, and fewer rounds run.
ps_status refit_minimum(ps_ctx *c, double conw_r, ScanFits &sf, double rel, int32_t halfwidth, bool fill,
                        double *ms, int64_t *nrefit, int64_t *evals, int32_t *rounds, int64_t *lit)
{
    ps_status st = make_plan(c, PS_FORM_FP64);
    if (st != PS_OK) return st;
    const int64_t slots = std::max(c->plan[PS_FORM_FP64].slots, 1);
    std::vector<ps_row> rows;
    std::vector<int64_t> pidx;
    std::vector<int32_t> pole;
    std::vector<int64_t> per, order;
    std::vector<char> picked;
    for (int round = 0; round < 64; round++) {
        sf.rows(rows, c->obj.ndata);
        const int64_t best = ScanFits::best(rows);
        const double lim = rows[static_cast<size_t>(best)].rms * (1 + rel);
        pidx.clear();
        pole.clear();
        per.clear();
        picked.assign(static_cast<size_t>(sf.nper), 0);
        for (int64_t n = 0; n < sf.nper; n++) {
            if (sf.fp64[static_cast<size_t>(n)]) continue;
            if (!(std::llabs(n - best) <= halfwidth || rows[static_cast<size_t>(n)].rms <= lim)) continue;
            per.push_back(n);
            picked[static_cast<size_t>(n)] = 1;
        }
        if (per.empty()) return PS_OK;
        // top up the last wave with the lowest remaining rows; a set that
        // leaves half (a quarter) of the slots free runs its fits over 2 (4)
        // CTAs each, so its wave holds slots / 2 (slots / 4) fits
        const int64_t need = static_cast<int64_t>(per.size()) * PS_N_POLES;
        const int64_t wave = need * 4 <= slots ? slots / 4 : need * 2 <= slots ? slots / 2 : slots;
        const int64_t cap = (need + wave - 1) / wave * wave;
        if (fill && need + PS_N_POLES <= cap) {
            order.clear();
            for (int64_t n = 0; n < sf.nper; n++)
                if (!sf.fp64[static_cast<size_t>(n)] && !picked[static_cast<size_t>(n)] &&
                    !std::isnan(rows[static_cast<size_t>(n)].rms))
                    order.push_back(n);
            const size_t extra = static_cast<size_t>((cap - need) / PS_N_POLES);
            const size_t k = std::min(extra, order.size());
            std::partial_sort(order.begin(), order.begin() + static_cast<std::ptrdiff_t>(k), order.end(),
                              [&](int64_t a, int64_t b) {
                                  return rows[static_cast<size_t>(a)].rms < rows[static_cast<size_t>(b)].rms;
                              });
            per.insert(per.end(), order.begin(), order.begin() + static_cast<std::ptrdiff_t>(k));
        }
        for (int64_t n : per)
            for (int m = 0; m < PS_N_POLES; m++) {
                pidx.push_back(sf.n_lo + n);
                pole.push_back(m + 1);
            }
        st = run_list(c, conw_r, pidx.data(), pole.data(), static_cast<int64_t>(pidx.size()), PS_FORM_FP64);
        if (st != PS_OK) return st;
        *ms += c->timing.kernel_ms;
        *evals += c->timing.evals;
        *lit += c->timing.lit_facets;
        *nrefit += static_cast<int64_t>(pidx.size());
        *rounds += 1;
        for (size_t k = 0; k < per.size(); k++) {
            const int64_t n = per[k];
            sf.fp64[static_cast<size_t>(n)] = 1;
            for (int m = 0; m < PS_N_POLES; m++) {
                sf.fits[static_cast<size_t>(n * PS_N_POLES + m)] = c->h_fits[k * PS_N_POLES + m];
                sf.done[static_cast<size_t>(n * PS_N_POLES + m)] = 1;
            }
        }
    }
    return PS_OK;
}

}  // namespace

extern "C" {

const char *ps_status_string(ps_status st)
{
    switch (st) {
    case PS_OK: return "ok";
    case PS_ERR_ARG: return "invalid argument";
    case PS_ERR_LIMIT: return "a size limit of the reference is exceeded";
    case PS_ERR_SINGULAR: return "singular matrix in the ellipsoid fit";
    case PS_ERR_IO: return "input/output error";
    case PS_ERR_CUDA: return "CUDA error";
    case PS_ERR_NO_DEVICE: return "no usable CUDA device";
    case PS_ERR_TIMEOUT: return "device wait timed out";
    }
    return "unknown status";
}

int32_t ps_abi_version(void) { return PS_ABI_VERSION; }

ps_status ps_input_read(const char *path, ps_input **out)
{
    if (!path || !out) return PS_ERR_ARG;
    *out = nullptr;
    auto in = std::make_unique<ps_input>();
    std::string err;
    ps_status st = psg::parse_input_file(path, in->data, err);
    if (st != PS_OK) {
        std::fprintf(stderr, "ps_input_read: %s\n", err.c_str());
        return st;
    }
    *out = in.release();
    return PS_OK;
}

ps_status ps_input_problem(const ps_input *in, ps_problem *v)
{
    if (!in || !v) return PS_ERR_ARG;
    const psg::ParsedInput &d = in->data;
    v->hdr = d.hdr;
    v->n_lc = static_cast<int32_t>(d.lc_points.size());
    v->lc_points = d.lc_points.data();
    v->lc_calibrated = d.lc_calibrated.data();
    v->lc_weight = d.lc_weight.data();
    v->ndata = static_cast<int32_t>(d.jd.size());
    v->jd = d.jd.data();
    v->brightness = d.brightness.data();
    v->sun = d.sun.data();
    v->earth = d.earth.data();
    return PS_OK;
}

void ps_input_free(ps_input *in) { delete in; }

}  // extern "C"

namespace {
ps_status upload_object(std::unique_ptr<ps_ctx> &c, ps_ctx **out);
}  // namespace

extern "C" {

ps_status ps_prepare(const ps_problem *prob, const ps_options *opt, ps_ctx **out)
{
    if (!prob || !out) return PS_ERR_ARG;
    *out = nullptr;
    auto c = std::make_unique<ps_ctx>();
    if (opt) c->opt = *opt;
    if (c->opt.form != PS_FORM_FP64 && c->opt.form != PS_FORM_MIXED) return PS_ERR_ARG;
    std::string err;
    ps_status st = psg::prepare_object(*prob, c->obj, err);
    if (st != PS_OK) {
        std::fprintf(stderr, "ps_prepare: %s\n", err.c_str());
        return st;
    }
    return upload_object(c, out);
}

ps_status ps_prepare_state(const ps_state *state, const ps_options *opt, ps_ctx **out)
{
    if (!state || !out) return PS_ERR_ARG;
    *out = nullptr;
    auto c = std::make_unique<ps_ctx>();
    if (opt) c->opt = *opt;
    if (c->opt.form != PS_FORM_FP64 && c->opt.form != PS_FORM_MIXED) return PS_ERR_ARG;
    std::string err;
    ps_status st = psg::prepare_object_state(*state, c->obj, err);
    if (st != PS_OK) {
        std::fprintf(stderr, "ps_prepare_state: %s\n", err.c_str());
        return st;
    }
    return upload_object(c, out);
}

}  // extern "C"

namespace {

// Device side of a prepared object: stream, events, the tables in one
// allocation, the fit plan and the per-slot scratch.
ps_status upload_object(std::unique_ptr<ps_ctx> &c, ps_ctx **out)
{
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= c->opt.device || c->opt.device < 0)
        return PS_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c->opt.device) != cudaSuccess) return PS_ERR_NO_DEVICE;
    if (prop.major < 10) return PS_ERR_NO_DEVICE;
    ps_ctx *cp = c.get();
    PSG_CUDA(cp, cudaSetDevice(c->opt.device));
    c->sm_count = prop.multiProcessorCount;
    PSG_CUDA(cp, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    for (auto &e : c->ev) PSG_CUDA(cp, cudaEventCreate(&e));

    psg::HostObject &o = c->obj;
    const psg::ShapeTables &s = o.shape;
    const int F = s.nfac;
    // Facet-major tables transposed to [index][facet] where threads run over
    // facets, and the Earth/Sun vectors split into coalesced components.
    std::vector<double> nx(F), ny(F), nz(F), pleg(static_cast<size_t>(s.npairs) * F),
        fc(static_cast<size_t>(s.mmax + 1) * F), fs(static_cast<size_t>(s.mmax + 1) * F);
    for (int i = 0; i < F; i++) {
        nx[i] = s.nor[3 * i];
        ny[i] = s.nor[3 * i + 1];
        nz[i] = s.nor[3 * i + 2];
        for (int q = 0; q < s.npairs; q++) pleg[static_cast<size_t>(q) * F + i] = s.pleg[static_cast<size_t>(i) * s.npairs + q];
        for (int m = 0; m <= s.mmax; m++) {
            fc[static_cast<size_t>(m) * F + i] = s.fc[static_cast<size_t>(i) * (s.mmax + 1) + m];
            fs[static_cast<size_t>(m) * F + i] = s.fs[static_cast<size_t>(i) * (s.mmax + 1) + m];
        }
    }
    // Solar phase angle of every point: it depends on the data only, so it is
    // computed once here with the host libm, as the reference computes it in
    // every evaluation (bright.c:30-31: acos of the dot product of the unit
    // vectors, in the same order).
    std::vector<double> ex(o.ndata), ey(o.ndata), ez(o.ndata), sx(o.ndata), sy(o.ndata), sz(o.ndata),
        alpha_pt(o.ndata);
    for (int q = 0; q < o.ndata; q++) {
        ex[q] = o.ee[3 * q];
        ey[q] = o.ee[3 * q + 1];
        ez[q] = o.ee[3 * q + 2];
        sx[q] = o.ee0[3 * q];
        sy[q] = o.ee0[3 * q + 1];
        sz[q] = o.ee0[3 * q + 2];
        alpha_pt[q] = std::acos(ex[q] * sx[q] + ey[q] * sy[q] + ez[q] * sz[q]);
    }
    // FP32 point geometry of the mixed form, two float4 per point: Earth
    // direction and phase angle, Sun direction and time
    std::vector<float> geo_f(static_cast<size_t>(o.ndata) * 8);
    for (int q = 0; q < o.ndata; q++) {
        float *g = &geo_f[static_cast<size_t>(q) * 8];
        g[0] = static_cast<float>(ex[q]);
        g[1] = static_cast<float>(ey[q]);
        g[2] = static_cast<float>(ez[q]);
        g[3] = static_cast<float>(alpha_pt[q]);
        g[4] = static_cast<float>(sx[q]);
        g[5] = static_cast<float>(sy[q]);
        g[6] = static_cast<float>(sz[q]);
        g[7] = static_cast<float>(o.tim[q]);
    }
    std::vector<double> sig2i(o.ndata);
    for (int q = 0; q < o.ndata; q++) sig2i[q] = 1 / (o.sig[q] * o.sig[q]);
    std::vector<float> dsph_f(s.dsph.begin(), s.dsph.end());
    std::vector<float> nx_f(nx.begin(), nx.end()), ny_f(ny.begin(), ny.end()), nz_f(nz.begin(), nz.end()),
        darea_f(s.darea.begin(), s.darea.end());
    Packer pk;
    size_t o_nx = pk.add(nx), o_ny = pk.add(ny), o_nz = pk.add(nz), o_darea = pk.add(s.darea),
           o_dsph = pk.add(s.dsph), o_pleg = pk.add(pleg), o_fc = pk.add(fc), o_fs = pk.add(fs),
           o_pm = pk.add(s.pair_m), o_pn = pk.add(s.pair_n), o_tim = pk.add(o.tim), o_br = pk.add(o.bright),
           o_sig = pk.add(o.sig), o_w = pk.add(o.weight), o_ex = pk.add(ex), o_ey = pk.add(ey), o_ez = pk.add(ez),
           o_sx = pk.add(sx), o_sy = pk.add(sy), o_sz = pk.add(sz), o_ls = pk.add(o.lc_start),
           o_ln = pk.add(o.lc_points), o_lr = pk.add(o.lc_rel), o_fl = pk.add(o.free_list),
           o_cgf = pk.add(o.cg_first), o_dsf = pk.add(dsph_f), o_alp = pk.add(alpha_pt), o_nxf = pk.add(nx_f),
           o_nyf = pk.add(ny_f), o_nzf = pk.add(nz_f), o_daf = pk.add(darea_f), o_s2i = pk.add(sig2i), o_geo = pk.add(geo_f);
    c->h2d_bytes = static_cast<int64_t>(pk.bytes.size());
    PSG_CUDA(cp, cudaMalloc(&c->d_tables, pk.bytes.size()));
    PSG_CUDA(cp, cudaMemcpyAsync(c->d_tables, pk.bytes.data(), pk.bytes.size(), cudaMemcpyHostToDevice, c->stream));
    char *b = c->d_tables;
    psg::DevObject &d = c->dob;
    d.nfac = F;
    d.ncoef = o.ncoef;
    d.ma = o.ma;
    d.mfit = o.mfit;
    d.npairs = s.npairs;
    d.mmax = s.mmax;
    d.n_lc = o.n_lc + 1;
    d.ndata = o.ndata;
    d.max_rel_points = o.max_rel_points;
    d.nx = reinterpret_cast<const double *>(b + o_nx);
    d.ny = reinterpret_cast<const double *>(b + o_ny);
    d.nz = reinterpret_cast<const double *>(b + o_nz);
    d.darea = reinterpret_cast<const double *>(b + o_darea);
    d.dsph = reinterpret_cast<const double *>(b + o_dsph);
    d.pleg = reinterpret_cast<const double *>(b + o_pleg);
    d.fc = reinterpret_cast<const double *>(b + o_fc);
    d.fs = reinterpret_cast<const double *>(b + o_fs);
    d.pair_m = reinterpret_cast<const int *>(b + o_pm);
    d.pair_n = reinterpret_cast<const int *>(b + o_pn);
    d.tim = reinterpret_cast<const double *>(b + o_tim);
    d.bright = reinterpret_cast<const double *>(b + o_br);
    d.sig = reinterpret_cast<const double *>(b + o_sig);
    d.weight = reinterpret_cast<const double *>(b + o_w);
    d.eex = reinterpret_cast<const double *>(b + o_ex);
    d.eey = reinterpret_cast<const double *>(b + o_ey);
    d.eez = reinterpret_cast<const double *>(b + o_ez);
    d.e0x = reinterpret_cast<const double *>(b + o_sx);
    d.e0y = reinterpret_cast<const double *>(b + o_sy);
    d.e0z = reinterpret_cast<const double *>(b + o_sz);
    d.lc_start = reinterpret_cast<const int *>(b + o_ls);
    d.lc_npts = reinterpret_cast<const int *>(b + o_ln);
    d.lc_rel = reinterpret_cast<const int *>(b + o_lr);
    d.free_list = reinterpret_cast<const int *>(b + o_fl);
    d.cg_first = reinterpret_cast<const double *>(b + o_cgf);
    d.dsph_f = reinterpret_cast<const float *>(b + o_dsf);
    d.alpha_pt = reinterpret_cast<const double *>(b + o_alp);
    d.nx_f = reinterpret_cast<const float *>(b + o_nxf);
    d.ny_f = reinterpret_cast<const float *>(b + o_nyf);
    d.nz_f = reinterpret_cast<const float *>(b + o_nzf);
    d.darea_f = reinterpret_cast<const float *>(b + o_daf);
    d.sig2i = reinterpret_cast<const double *>(b + o_s2i);
    d.geo_f = reinterpret_cast<const float4 *>(b + o_geo);

    ps_status pst = make_plan(cp, c->opt.form);
    if (pst != PS_OK) {
        std::fprintf(stderr, "ps_prepare: %s\n", c->err.c_str());
        return pst;
    }
    c->P = c->plan[c->opt.form].P;
    c->dsph_smem = c->plan[c->opt.form].dsph_smem;
    c->rel_rows = c->plan[c->opt.form].rel_rows;
    c->smem = c->plan[c->opt.form].smem;
    c->slots = c->plan[c->opt.form].slots;
    c->scratch_stride = static_cast<size_t>(std::max(o.max_rel_points, 1)) * psg::rel_row_stride(o.ma);
    c->scratch_stride = (c->scratch_stride + 31) & ~size_t(31);
    PSG_CUDA(cp, cudaMalloc(&c->d_scratch, c->scratch_stride * c->slots * sizeof(double)));
    PSG_CUDA(cp, cudaMalloc(&c->d_queue, 256));
    size_t ev_doubles = static_cast<size_t>(o.ma) + static_cast<size_t>(o.mfit) * o.mfit + o.mfit + 1 + F;
    PSG_CUDA(cp, cudaMalloc(&c->d_eval, ev_doubles * sizeof(double)));
    PSG_CUDA(cp, cudaStreamSynchronize(c->stream));
    *out = c.release();
    return PS_OK;
}

}  // namespace

extern "C" {

ps_status ps_get_info(const ps_ctx *c, ps_info *out)
{
    if (!c || !out) return PS_ERR_ARG;
    const psg::HostObject &o = c->obj;
    out->ndata = o.ndata;
    out->n_lc = o.n_lc;
    out->ncoef = o.ncoef;
    out->ma = o.ma;
    out->mfit = o.mfit;
    out->nfac = o.shape.nfac;
    out->n_max = o.n_max;
    out->escl = o.escl;
    out->conw_r0 = o.conw_r0;
    out->freq_start = o.freq_start;
    out->freq_step = o.freq_step;
    out->sm_count = c->sm_count;
    out->slots = c->slots;
    out->h2d_bytes = c->h2d_bytes;
    const FormPlan &pl = c->plan[c->opt.form];
    out->tensor_cores = pl.ready && psg::basis_on_tensor(pl.dsph_smem) ? 1 : 0;
    out->tile_points = pl.ready ? pl.P : 0;
    return PS_OK;
}

ps_status ps_precalc_step(ps_ctx *c, double *conw_r, int32_t *new_conw)
{
    if (!c || !conw_r || !new_conw || !(*conw_r > 0)) return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    const int64_t ntest = std::min<int64_t>(10, c->obj.n_max);
    if (ntest < 1) return PS_ERR_ARG;
    std::vector<ps_row> rows(static_cast<size_t>(ntest));
    ps_status st = scan_rows(c, *conw_r, 1, ntest, rows.data(), true);
    if (st != PS_OK) return st;
    double sum = 0.0;
    for (int64_t n = 0; n < ntest; n++) sum = sum + rows[static_cast<size_t>(n)].dark_or_conw;
    const double ave = sum / ntest;
    if (ave < 1.0) *new_conw = 1;
    if (ave >= 1.0) *conw_r = *conw_r * 2;
    return PS_OK;
}

ps_status ps_precalc_conw(ps_ctx *c, double *conw_r, int32_t *new_conw)
{
    if (!c || !conw_r || !new_conw) return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    const psg::HostObject &o = c->obj;
    double cw = o.conw_r0;
    int32_t nc = 0;
    const int64_t ntest = std::min<int64_t>(10, o.n_max);
    double launches = 0, kms = 0, tms = 0;
    int64_t fits = 0, evals = 0, lit = 0;
    while (nc != 1 && (cw * o.escl * o.escl) < 10.0) {
        if (ntest < 1) break;
        ps_status st = ps_precalc_step(c, &cw, &nc);
        if (st != PS_OK) return st;
        launches += 1;
        kms += c->timing.kernel_ms;
        tms += c->timing.total_ms;
        fits += c->timing.fits;
        evals += c->timing.evals;
        lit += c->timing.lit_facets;
    }
    c->timing.kernel_ms = kms;
    c->timing.total_ms = tms;
    c->timing.fits = fits;
    c->timing.evals = evals;
    c->timing.lit_facets = lit;
    c->timing.launches = static_cast<int32_t>(launches);
    *conw_r = cw;
    *new_conw = nc;
    return PS_OK;
}

ps_status ps_scan(ps_ctx *c, double conw_r, int64_t n_lo, int64_t n_hi, ps_row *out)
{
    if (!c || !out || n_lo < 1 || n_hi < n_lo || !(conw_r > 0)) return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    ps_status st = scan_rows(c, conw_r, n_lo, n_hi, out, false);
    if (st != PS_OK) return st;
    if (n_lo == 1) out[0].dark_or_conw = conw_r * c->obj.escl * c->obj.escl;
    return PS_OK;
}

ps_status ps_fit_batch(ps_ctx *c, double conw_r, int64_t n_fits, const int64_t *period_index, const int32_t *pole,
                       ps_fit *out)
{
    if (!c || !out || !period_index || !pole || n_fits < 1 || !(conw_r > 0)) return PS_ERR_ARG;
    for (int64_t i = 0; i < n_fits; i++)
        if (period_index[i] < 1 || pole[i] < 1 || pole[i] > PS_N_POLES) return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    ps_status st = run_list(c, conw_r, period_index, pole, n_fits, c->opt.form);
    if (st != PS_OK) return st;
    std::memcpy(out, c->h_fits.data(), n_fits * sizeof(ps_fit));
    return PS_OK;
}

// Allocation-free variant of ps_fit_batch for callers that cannot allocate
// device memory at call time (see ps_gb300.h).  Everything it touches is
// either the caller's (work lists, outputs, stream), the context's tables from
// ps_prepare, or the file-scope scratch array of ps_engine.cu.
ps_status ps_fit_batch_noalloc(ps_ctx *c, double conw_r, int64_t n_fits, const int64_t *d_period_index,
                               const int32_t *d_pole, ps_fit *d_out, void *stream)
{
    if (!c || !d_period_index || !d_pole || !d_out || n_fits < 1 || !(conw_r > 0)) return PS_ERR_ARG;
    if (c->opt.form != PS_FORM_FP64) {
        c->err = "ps_fit_batch_noalloc supports the FP64 form only";
        return PS_ERR_ARG;
    }
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    psg::FitConfig cfg = make_config(c, conw_r);
    psg::FitWork w{};
    w.n_lo = 1;
    w.nfits = n_fits;
    w.period_index = d_period_index;
    w.pole = d_pole;
    w.scratch_stride = c->scratch_stride;
    w.rel_rows = c->rel_rows;   // rows in shared memory where the plan put them there
    w.out = d_out;
    int grid = 0;
    int e = psg::launch_fits_noalloc(c->opt.form, c->dob, cfg, w, c->slots, c->P, c->smem, stream, &grid);
    if (e == -1) {
        char msg[256];
        std::snprintf(msg, sizeof msg,
                      "one fit slot needs %zu doubles of scratch; the allocation-free path holds %zu "
                      "(4 MiB minus the work counter)",
                      c->scratch_stride, psg::kStaticScratchDoubles - 32);
        c->err = msg;
        return PS_ERR_LIMIT;
    }
    if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "allocation-free fit launch");
    return PS_OK;
}

ps_status ps_eval(ps_ctx *c, double conw_r, const double *cg, double *alpha, double *beta, double *chisq,
                  double *area)
{
    if (!c || !cg || !alpha || !beta || !chisq || !(conw_r > 0)) return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    const psg::HostObject &o = c->obj;
    const int ma = o.ma, mf = o.mfit, F = o.shape.nfac;
    double *d_cg = c->d_eval, *d_al = d_cg + ma, *d_be = d_al + static_cast<size_t>(mf) * mf, *d_c2 = d_be + mf,
           *d_ar = d_c2 + 1;
    PSG_CUDA(c, cudaMemcpyAsync(d_cg, cg, ma * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    psg::FitConfig cfg = make_config(c, conw_r);
    int e = psg::launch_eval(c->opt.form, c->dob, cfg, d_cg, d_al, d_be, d_c2, d_ar, c->d_scratch, c->P, c->smem,
                             c->dsph_smem, c->rel_rows, c->stream);
    if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "eval kernel launch");
    PSG_CUDA(c, cudaMemcpyAsync(alpha, d_al, static_cast<size_t>(mf) * mf * sizeof(double), cudaMemcpyDeviceToHost,
                                c->stream));
    PSG_CUDA(c, cudaMemcpyAsync(beta, d_be, mf * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PSG_CUDA(c, cudaMemcpyAsync(chisq, d_c2, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (area) PSG_CUDA(c, cudaMemcpyAsync(area, d_ar, F * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PSG_CUDA(c, cudaStreamSynchronize(c->stream));
    return PS_OK;
}

ps_status ps_trajectories(ps_ctx *c, double conw_r, int64_t n_lo, int64_t n_hi, int32_t feat_iters, float *traj)
{
    if (!c || !traj || n_lo < 1 || n_hi < n_lo || !(conw_r > 0) || feat_iters < 4 || feat_iters > 48 ||
        feat_iters % 4)
        return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    const int64_t nfits = (n_hi - n_lo + 1) * PS_N_POLES;
    float *d_traj = nullptr;
    PSG_CUDA(c, cudaMalloc(&d_traj, nfits * psg::kTrajFloats * sizeof(float)));
    PSG_CUDA(c, cudaMemsetAsync(d_traj, 0, nfits * psg::kTrajFloats * sizeof(float), c->stream));
    psg::FitWork w{};
    w.n_lo = n_lo;
    w.nfits = nfits;
    w.traj = d_traj;
    w.screen_iters = feat_iters;
    ps_status st = run_fits(c, conw_r, w, c->opt.form);
    if (st == PS_OK) {
        cudaError_t e = cudaMemcpy(traj, d_traj, nfits * psg::kTrajFloats * sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_fail(c, e, "trajectory copy");
    }
    cudaFree(d_traj);
    return st;
}

ps_status ps_mlp_train(int32_t device, float *weights, const float *x, const float *y, int64_t n, int32_t epochs,
                       int32_t batch, float lr, uint64_t seed, float *loss_history)
{
    if (!weights || !x || !y || n < 1 || epochs < 1 || batch < 1 || n > INT32_MAX) return PS_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return PS_ERR_NO_DEVICE;
    int e = psg::mlp_train(weights, x, y, static_cast<int>(n), epochs, batch, lr, seed, loss_history);
    return e == 0 ? PS_OK : PS_ERR_CUDA;
}

ps_status ps_mlp_predict(int32_t device, const float *weights, const float *x, int64_t n, float *y)
{
    if (!weights || !x || !y || n < 1 || n > INT32_MAX) return PS_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return PS_ERR_NO_DEVICE;
    int e = psg::mlp_predict(weights, x, static_cast<int>(n), y);
    return e == 0 ? PS_OK : PS_ERR_CUDA;
}

ps_status ps_mlp_grad(int32_t device, const float *weights, const float *x, const float *y, int64_t n, float *loss,
                      float *grad)
{
    if (!weights || !x || !y || !loss || !grad || n < 1 || n > INT32_MAX) return PS_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return PS_ERR_NO_DEVICE;
    int e = psg::mlp_grad(weights, x, y, static_cast<int>(n), loss, grad);
    return e == 0 ? PS_OK : PS_ERR_CUDA;
}

namespace {

// Screening launch: screen_iters iterations of every fit of n_lo..n_hi in
// the mixed form with the in-kernel predictor; results in c->h_fits.  With
// save_state every fit's LM state is kept on the device (c->d_state, fit f
// in row f) for a later resume.
ps_status screen_fits(ps_ctx *c, double conw_r, int64_t n_lo, int64_t n_hi, const float *weights, int screen_iters,
                      bool save_state)
{
    const int64_t nfits = (n_hi - n_lo + 1) * PS_N_POLES;
    if (save_state && static_cast<size_t>(nfits) > c->state_cap) {
        cudaFree(c->d_state);
        c->d_state = nullptr;
        c->state_cap = 0;
        PSG_CUDA(c, cudaMalloc(&c->d_state, nfits * psg::state_stride(c->obj.ma) * sizeof(double)));
        c->state_cap = static_cast<size_t>(nfits);
    }
    float *d_w = nullptr;
    PSG_CUDA(c, cudaMalloc(&d_w, psg::kMlpFloats * sizeof(float)));
    cudaError_t ce = cudaMemcpy(d_w, weights, psg::kMlpFloats * sizeof(float), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        cudaFree(d_w);
        return cuda_fail(c, ce, "predictor weights copy");
    }
    psg::FitWork w{};
    w.n_lo = n_lo;
    w.nfits = nfits;
    w.iter_limit = screen_iters;
    w.screen_iters = screen_iters;
    w.mlp = d_w;
    if (save_state) w.state = c->d_state;
    ps_status st = run_fits(c, conw_r, w, PS_FORM_MIXED);
    cudaFree(d_w);
    return st;
}

bool screen_iters_ok(int k) { return k >= 4 && k <= 48 && k % 4 == 0; }

}  // namespace

ps_status ps_screen(ps_ctx *c, double conw_r, int64_t n_lo, int64_t n_hi, int32_t screen_iters, const float *weights,
                    ps_fit *out)
{
    if (!c || !weights || !out || n_lo < 1 || n_hi < n_lo || !(conw_r > 0) || !screen_iters_ok(screen_iters))
        return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    ps_status st = screen_fits(c, conw_r, n_lo, n_hi, weights, screen_iters, false);
    if (st != PS_OK) return st;
    std::memcpy(out, c->h_fits.data(), c->h_fits.size() * sizeof(ps_fit));
    return PS_OK;
}

ps_status ps_scan_learned(ps_ctx *c, double conw_r, int64_t n_lo, int64_t n_hi, const float *weights,
                          const ps_learned_opts *opts, ps_row *out, ps_learned_stats *stats)
{
    ps_learned_opts o{8, 0.02, 0, 2, 0.005, 2, 1};
    if (opts) o = *opts;
    if (!c || !weights || !out || n_lo < 1 || n_hi < n_lo || !(conw_r > 0) || !screen_iters_ok(o.screen_iters) ||
        !(o.margin >= 0) || o.batch_periods < 0 || o.region_halfwidth < 0 || !(o.refit_rel >= 0) ||
        o.refit_halfwidth < 0)
        return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    ScanFits sf;
    sf.n_lo = n_lo;
    sf.nper = n_hi - n_lo + 1;
    const int64_t nfits = sf.nper * PS_N_POLES;
    ps_learned_stats stt{};
    stt.fits_total = nfits;
    const int64_t launch0 = c->launch_total;
    // (1) screening: screen_iters iterations of every fit, the predicted
    // final rms, the LM states kept for the completion
    ps_status st = screen_fits(c, conw_r, n_lo, n_hi, weights, o.screen_iters, true);
    if (st != PS_OK) return st;
    stt.screen_ms = c->timing.kernel_ms;
    stt.evals += c->timing.evals;
    stt.evals_screen = c->timing.evals;
    sf.fits = c->h_fits;
    sf.done.assign(static_cast<size_t>(nfits), 0);
    sf.fp64.assign(static_cast<size_t>(sf.nper), 0);
    // predicted row of every period: the lowest predicted final rms of its poles
    std::vector<double> pred(static_cast<size_t>(sf.nper));
    for (int64_t n = 0; n < sf.nper; n++) {
        double p = INFINITY;
        for (int m = 0; m < PS_N_POLES; m++) {
            const double v = sf.fits[static_cast<size_t>(n * PS_N_POLES + m)].pred_dev;
            if (v > 0 && v < p) p = v;
        }
        pred[static_cast<size_t>(n)] = p;
    }
    std::vector<int64_t> order(static_cast<size_t>(sf.nper));
    for (int64_t n = 0; n < sf.nper; n++) order[static_cast<size_t>(n)] = n;
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t a, int64_t b) { return pred[static_cast<size_t>(a)] < pred[static_cast<size_t>(b)]; });
    std::vector<char> period_done(static_cast<size_t>(sf.nper), 0);
    std::vector<int64_t> pidx, slot;
    std::vector<int32_t> pole;
    // completes every pole of the listed periods from its saved state
    auto complete = [&](const std::vector<int64_t> &periods) -> ps_status {
        pidx.clear();
        pole.clear();
        slot.clear();
        for (int64_t n : periods) {
            period_done[static_cast<size_t>(n)] = 1;
            stt.region_periods++;
            for (int m = 0; m < PS_N_POLES; m++) {
                const int64_t i = n * PS_N_POLES + m;
                sf.done[static_cast<size_t>(i)] = 1;
                // a fit that the screening already ended (stop rule) is final
                if (!sf.fits[static_cast<size_t>(i)].screened) continue;
                pidx.push_back(n_lo + n);
                pole.push_back(m + 1);
                slot.push_back(i);
            }
        }
        const int64_t k = static_cast<int64_t>(pidx.size());
        if (k == 0) return PS_OK;
        ps_status r = run_list(c, conw_r, pidx.data(), pole.data(), k, PS_FORM_MIXED, 0, slot.data());
        if (r != PS_OK) return r;
        stt.complete_ms += c->timing.kernel_ms;
        stt.evals += c->timing.evals;
        stt.evals_complete += c->timing.evals;
        for (int64_t q = 0; q < k; q++)
            sf.fits[static_cast<size_t>(slot[static_cast<size_t>(q)])] = c->h_fits[static_cast<size_t>(q)];
        return PS_OK;
    };
    auto best_done = [&]() {
        double b = INFINITY;
        int64_t bn = -1;
        for (int64_t n = 0; n < sf.nper; n++) {
            if (!period_done[static_cast<size_t>(n)]) continue;
            const double r = sf.row(n, c->obj.ndata).rms;
            if (r < b) {
                b = r;
                bn = n;
            }
        }
        return std::make_pair(b, bn);
    };
    // (2) completion in the order of the predicted rows, a device's worth
    // of periods per launch, until the next period's predicted row, lowered
    // by the margin, cannot beat the best completed row
    const int64_t batch = o.batch_periods > 0 ? o.batch_periods : std::max<int64_t>(1, c->slots / PS_N_POLES);
    const double shrink = std::exp(-o.margin);
    size_t next = 0;
    std::vector<int64_t> group;
    for (;;) {
        const double best = best_done().first;
        group.clear();
        while (next < order.size() && static_cast<int64_t>(group.size()) < batch) {
            const int64_t n = order[next];
            if (!(pred[static_cast<size_t>(n)] * shrink <= best)) break;
            group.push_back(n);
            next++;
        }
        if (group.empty()) break;
        st = complete(group);
        if (st != PS_OK) return st;
    }
    // (3) every period within region_halfwidth of the best completed row,
    // until the best row no longer moves
    for (int round = 0; round < 16; round++) {
        const int64_t bn = best_done().second;
        if (bn < 0) break;
        group.clear();
        for (int64_t n = std::max<int64_t>(0, bn - o.region_halfwidth);
             n <= std::min<int64_t>(sf.nper - 1, bn + o.region_halfwidth); n++)
            if (!period_done[static_cast<size_t>(n)]) group.push_back(n);
        if (group.empty()) break;
        st = complete(group);
        if (st != PS_OK) return st;
    }
    for (char d : sf.done) stt.fits_completed += d;
    stt.fits_screened_out = nfits - stt.fits_completed;
    // (4) FP64 refit of the periods nearest the best row
    const int64_t ev0 = stt.evals;
    int64_t lit = 0;
    st = refit_minimum(c, conw_r, sf, o.refit_rel, o.refit_halfwidth, o.fill_refit_waves != 0, &stt.refit_ms,
                       &stt.fits_refit, &stt.evals, &stt.refit_rounds, &lit);
    if (st != PS_OK) return st;
    stt.evals_refit = stt.evals - ev0;
    std::vector<ps_row> rows;
    sf.rows(rows, c->obj.ndata);
    const int64_t best = ScanFits::best(rows);
    for (int64_t n = 0; n < sf.nper; n++) out[n] = rows[static_cast<size_t>(n)];
    if (n_lo == 1) out[0].dark_or_conw = conw_r * c->obj.escl * c->obj.escl;
    stt.best_index = n_lo + best;
    c->timing.kernel_ms = stt.screen_ms + stt.complete_ms + stt.refit_ms;
    c->timing.fits = nfits;
    c->timing.evals = stt.evals;
    c->timing.lit_facets = lit;   // the FP64 refit's
    c->timing.launches = static_cast<int32_t>(c->launch_total - launch0);
    stt.launches = c->timing.launches;
    if (stats) *stats = stt;
    return PS_OK;
}

ps_status ps_scan_refined(ps_ctx *c, double conw_r, int64_t n_lo, int64_t n_hi, double refit_rel,
                          int32_t refit_halfwidth, ps_row *out, ps_learned_stats *stats)
{
    if (!c || !out || n_lo < 1 || n_hi < n_lo || !(conw_r > 0) || !(refit_rel >= 0) || refit_halfwidth < 0)
        return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    ScanFits sf;
    sf.n_lo = n_lo;
    sf.nper = n_hi - n_lo + 1;
    const int64_t nfits = sf.nper * PS_N_POLES;
    ps_learned_stats stt{};
    stt.fits_total = nfits;
    const int64_t launch0 = c->launch_total;
    psg::FitWork w{};
    w.n_lo = n_lo;
    w.nfits = nfits;
    ps_status st = run_fits(c, conw_r, w, c->opt.form);
    if (st != PS_OK) return st;
    stt.complete_ms = c->timing.kernel_ms;
    stt.evals = c->timing.evals;
    stt.evals_complete = c->timing.evals;
    stt.fits_completed = nfits;
    sf.fits = c->h_fits;
    sf.done.assign(static_cast<size_t>(nfits), 1);
    sf.fp64.assign(static_cast<size_t>(sf.nper), c->opt.form == PS_FORM_FP64 ? 1 : 0);
    int64_t lit = c->opt.form == PS_FORM_FP64 ? c->timing.lit_facets : 0;
    st = refit_minimum(c, conw_r, sf, refit_rel, refit_halfwidth, true, &stt.refit_ms, &stt.fits_refit,
                       &stt.evals, &stt.refit_rounds, &lit);
    if (st != PS_OK) return st;
    stt.evals_refit = stt.evals - stt.evals_complete;
    std::vector<ps_row> rows;
    sf.rows(rows, c->obj.ndata);
    for (int64_t n = 0; n < sf.nper; n++) out[n] = rows[static_cast<size_t>(n)];
    if (n_lo == 1) out[0].dark_or_conw = conw_r * c->obj.escl * c->obj.escl;
    stt.best_index = n_lo + ScanFits::best(rows);
    c->timing.kernel_ms = stt.complete_ms + stt.refit_ms;
    c->timing.fits = nfits;
    c->timing.evals = stt.evals;
    c->timing.lit_facets = lit;   // the FP64 form's
    c->timing.launches = static_cast<int32_t>(c->launch_total - launch0);
    stt.launches = c->timing.launches;
    if (stats) *stats = stt;
    return PS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner
// ---------------------------------------------------------------------------
extern "C" ps_status ps_autotune(ps_ctx *c, double conw_r, int32_t sample_fits, int32_t sample_iters,
                                 ps_tune_report *rep)
{
    if (!c || !rep || !(conw_r > 0) || sample_fits < 0 || sample_iters < 0) return PS_ERR_ARG;
    PSG_CUDA(c, cudaSetDevice(c->opt.device));
    const int form = c->opt.form;
    const bool mixed = form == PS_FORM_MIXED;
    const psg::HostObject &o = c->obj;
    ps_status st = make_plan(c, form);
    if (st != PS_OK) return st;
    const FormPlan dflt = c->plan[form];
    *rep = ps_tune_report{};
    const int64_t nfit = sample_fits > 0 ? sample_fits : 2 * static_cast<int64_t>(dflt.slots);
    const int iters = sample_iters > 0 ? sample_iters : 6;
    rep->sample_fits = static_cast<int32_t>(nfit);
    rep->sample_iters = iters;
    // sample: periods spread over the scan, all poles in turn
    std::vector<int64_t> pidx(static_cast<size_t>(nfit));
    std::vector<int32_t> pole(static_cast<size_t>(nfit));
    for (int64_t k = 0; k < nfit; k++) {
        pidx[static_cast<size_t>(k)] = 1 + (k / PS_N_POLES * 7919) % std::max<int64_t>(o.n_max, 1);
        pole[static_cast<size_t>(k)] = static_cast<int32_t>(k % PS_N_POLES) + 1;
    }
    std::vector<int> modes;
    if (mixed) {
        if (!(c->opt.flags & PS_FLAG_NO_TENSOR)) {
            modes.push_back(psg::kBasisTensor);
            modes.push_back(psg::kBasisTensorWide);
        }
        modes.push_back(psg::kBasisSmem);
    }
    modes.push_back(psg::kBasisGlobal);
    const int tiles_mixed[] = {32, 16}, tiles_fp64[] = {32, 16, 8};
    std::vector<FormPlan> plans;
    double best = -1;
    int chosen = -1;
    for (int mode : modes) {
        const int *tiles = mixed ? tiles_mixed : tiles_fp64;
        const int ntiles = mixed ? 2 : 3;
        for (int t = 0; t < ntiles; t++) {
            for (int cap : {0, 1}) {
                if (rep->n >= PS_TUNE_MAX) break;
                FormPlan cand;
                st = build_plan(c, form, mode, tiles[t], cap, &cand);
                if (st == PS_ERR_LIMIT) continue;
                if (st != PS_OK) return st;
                bool dup = false;
                for (const FormPlan &q : plans)
                    dup |= q.P == cand.P && q.dsph_smem == cand.dsph_smem && q.slots == cand.slots;
                if (dup) continue;
                c->plan[form] = cand;
                st = run_list(c, conw_r, pidx.data(), pole.data(), nfit, form, iters);   // warm-up
                if (st == PS_OK) st = run_list(c, conw_r, pidx.data(), pole.data(), nfit, form, iters);
                if (st != PS_OK) {
                    c->plan[form] = dflt;
                    return st;
                }
                ps_tune_candidate &r = rep->cand[rep->n];
                r.basis = cand.dsph_smem;
                r.tile_points = cand.P;
                r.ctas_per_sm = cand.slots / std::max(c->sm_count, 1);
                r.slots = cand.slots;
                r.fits_per_s = c->timing.kernel_ms > 0 ? nfit / (c->timing.kernel_ms * 1e-3) : 0;
                if (r.fits_per_s > best) {
                    best = r.fits_per_s;
                    chosen = rep->n;
                }
                plans.push_back(cand);
                rep->n++;
            }
        }
    }
    if (chosen < 0) {
        c->plan[form] = dflt;
        c->err = "no kernel configuration could be measured";
        return PS_ERR_LIMIT;
    }
    c->plan[form] = plans[static_cast<size_t>(chosen)];
    const FormPlan &pl = c->plan[form];
    const int e = psg::set_kernel_smem(form, pl.smem, o.ncoef, pl.dsph_smem);
    if (e != 0) return cuda_fail(c, static_cast<cudaError_t>(e), "cudaFuncSetAttribute");
    c->P = pl.P;
    c->dsph_smem = pl.dsph_smem;
    c->rel_rows = pl.rel_rows;
    c->smem = pl.smem;
    rep->chosen = chosen;
    return PS_OK;
}

// ---------------------------------------------------------------------------
// Multi-object packing
// ---------------------------------------------------------------------------
struct ps_pack {
    std::vector<ps_ctx *> ctx;
    int form = PS_FORM_FP64;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    psg::DevObject *d_objs = nullptr;
    psg::FitConfig *d_cfgs = nullptr;
    double *d_scratch = nullptr;
    size_t scratch_stride = 0;
    double *d_alpha_g = nullptr;       // per-slot normal matrices of the wide tensor-core path
    int slots = 0, P = 0, dsph_smem = 0;
    size_t smem = 0;
    unsigned long long *d_queue = nullptr;
    int *d_obj = nullptr, *d_pole = nullptr;
    int64_t *d_pidx = nullptr;
    ps_fit *d_out = nullptr;
    size_t cap = 0;
    ps_timing timing{};
    std::string err;
};

namespace {

ps_status pack_fail(ps_pack *k, cudaError_t e, const char *what)
{
    k->err = std::string(what) + ": " + cudaGetErrorString(e);
    return PS_ERR_CUDA;
}

#define PSG_PACK_CUDA(pk, call)                                    \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return pack_fail((pk), e_, #call);  \
    } while (0)

bool same_shape(const psg::HostObject &a, const psg::HostObject &b)
{
    return a.shape.nfac == b.shape.nfac && a.ncoef == b.ncoef && a.ma == b.ma && a.mfit == b.mfit &&
           a.shape.npairs == b.shape.npairs && a.shape.mmax == b.shape.mmax && a.free_list == b.free_list &&
           a.shape.dsph == b.shape.dsph && a.shape.nor == b.shape.nor;
}

}  // namespace

extern "C" {

ps_status ps_pack_create(ps_ctx *const *ctxs, int32_t n, int32_t form, ps_pack **out)
{
    if (!ctxs || n < 1 || !out || (form != PS_FORM_FP64 && form != PS_FORM_MIXED)) return PS_ERR_ARG;
    *out = nullptr;
    for (int32_t i = 0; i < n; i++) {
        if (!ctxs[i]) return PS_ERR_ARG;
        if (ctxs[i]->opt.device != ctxs[0]->opt.device || !same_shape(ctxs[i]->obj, ctxs[0]->obj)) return PS_ERR_ARG;
    }
    std::unique_ptr<ps_pack> k(new ps_pack());
    k->ctx.assign(ctxs, ctxs + n);
    k->form = form;
    k->device = ctxs[0]->opt.device;
    ps_ctx *c0 = ctxs[0];
    PSG_PACK_CUDA(k.get(), cudaSetDevice(k->device));
    ps_status st = make_plan(c0, form);
    if (st != PS_OK) {
        k->err = c0->err;
        return st;
    }
    const FormPlan &pl = c0->plan[form];
    k->P = pl.P;
    k->dsph_smem = pl.dsph_smem;
    k->smem = pl.smem;
    k->slots = pl.slots;
    int e = psg::set_pack_smem(form, k->smem, c0->obj.ncoef, k->dsph_smem);
    if (e != 0) return pack_fail(k.get(), static_cast<cudaError_t>(e), "cudaFuncSetAttribute");
    for (ps_ctx *c : k->ctx) k->scratch_stride = std::max(k->scratch_stride, c->scratch_stride);
    PSG_PACK_CUDA(k.get(), cudaStreamCreateWithFlags(&k->stream, cudaStreamNonBlocking));
    PSG_PACK_CUDA(k.get(), cudaEventCreate(&k->ev[0]));
    PSG_PACK_CUDA(k.get(), cudaEventCreate(&k->ev[1]));
    PSG_PACK_CUDA(k.get(), cudaMalloc(&k->d_objs, sizeof(psg::DevObject) * n));
    PSG_PACK_CUDA(k.get(), cudaMalloc(&k->d_cfgs, sizeof(psg::FitConfig) * n));
    PSG_PACK_CUDA(k.get(), cudaMalloc(&k->d_scratch, k->scratch_stride * k->slots * sizeof(double)));
    PSG_PACK_CUDA(k.get(), cudaMalloc(&k->d_queue, 2 * sizeof(unsigned long long)));
    if (k->dsph_smem == psg::kBasisTensorWide)
        PSG_PACK_CUDA(k.get(), cudaMalloc(&k->d_alpha_g, static_cast<size_t>(c0->obj.mfit) * c0->obj.mfit *
                                                            k->slots * sizeof(double)));
    std::vector<psg::DevObject> objs(static_cast<size_t>(n));
    for (int32_t i = 0; i < n; i++) objs[static_cast<size_t>(i)] = ctxs[i]->dob;
    PSG_PACK_CUDA(k.get(), cudaMemcpy(k->d_objs, objs.data(), sizeof(psg::DevObject) * n, cudaMemcpyHostToDevice));
    *out = k.release();
    return PS_OK;
}

}  // extern "C"

namespace {

// One packed launch.  iter_limit > 0 stops every fit after that many LM
// iterations (screening, with the predictor `weights` when given); traj
// (host, [n_fits][kTrajFloats]) receives the fits' trajectory records.
ps_status pack_run(ps_pack *k, const double *conw_r, int64_t n_fits, const int32_t *object,
                   const int64_t *period_index, const int32_t *pole, int iter_limit, int screen_iters,
                   const float *weights, float *traj, ps_fit *out)
{
    if (!k || !conw_r || n_fits < 1 || !object || !period_index || !pole || !out) return PS_ERR_ARG;
    const int32_t nobj = static_cast<int32_t>(k->ctx.size());
    for (int32_t o = 0; o < nobj; o++)
        if (!(conw_r[o] > 0)) return PS_ERR_ARG;
    for (int64_t i = 0; i < n_fits; i++)
        if (object[i] < 0 || object[i] >= nobj || period_index[i] < 1 || pole[i] < 1 || pole[i] > PS_N_POLES)
            return PS_ERR_ARG;
    PSG_PACK_CUDA(k, cudaSetDevice(k->device));
    // largest objects first: the queue then ends on short fits
    std::vector<int64_t> order(static_cast<size_t>(n_fits));
    for (int64_t i = 0; i < n_fits; i++) order[static_cast<size_t>(i)] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return k->ctx[static_cast<size_t>(object[a])]->obj.ndata > k->ctx[static_cast<size_t>(object[b])]->obj.ndata;
    });
    std::vector<int> h_obj(static_cast<size_t>(n_fits)), h_pole(static_cast<size_t>(n_fits));
    std::vector<int64_t> h_pidx(static_cast<size_t>(n_fits));
    for (int64_t i = 0; i < n_fits; i++) {
        const int64_t u = order[static_cast<size_t>(i)];
        h_obj[static_cast<size_t>(i)] = object[u];
        h_pidx[static_cast<size_t>(i)] = period_index[u];
        h_pole[static_cast<size_t>(i)] = pole[u];
    }
    std::vector<psg::FitConfig> cfgs(static_cast<size_t>(nobj));
    for (int32_t o = 0; o < nobj; o++) cfgs[static_cast<size_t>(o)] = make_config(k->ctx[static_cast<size_t>(o)], conw_r[o]);
    if (static_cast<size_t>(n_fits) > k->cap) {
        cudaFree(k->d_obj);
        cudaFree(k->d_pole);
        cudaFree(k->d_pidx);
        cudaFree(k->d_out);
        k->d_obj = k->d_pole = nullptr;
        k->d_pidx = nullptr;
        k->d_out = nullptr;
        k->cap = 0;
        PSG_PACK_CUDA(k, cudaMalloc(&k->d_obj, sizeof(int) * n_fits));
        PSG_PACK_CUDA(k, cudaMalloc(&k->d_pole, sizeof(int) * n_fits));
        PSG_PACK_CUDA(k, cudaMalloc(&k->d_pidx, sizeof(int64_t) * n_fits));
        PSG_PACK_CUDA(k, cudaMalloc(&k->d_out, sizeof(ps_fit) * n_fits));
        k->cap = static_cast<size_t>(n_fits);
    }
    PSG_PACK_CUDA(k, cudaMemcpyAsync(k->d_cfgs, cfgs.data(), sizeof(psg::FitConfig) * nobj, cudaMemcpyHostToDevice,
                                     k->stream));
    PSG_PACK_CUDA(k, cudaMemcpyAsync(k->d_obj, h_obj.data(), sizeof(int) * n_fits, cudaMemcpyHostToDevice, k->stream));
    PSG_PACK_CUDA(k, cudaMemcpyAsync(k->d_pole, h_pole.data(), sizeof(int) * n_fits, cudaMemcpyHostToDevice, k->stream));
    PSG_PACK_CUDA(k, cudaMemcpyAsync(k->d_pidx, h_pidx.data(), sizeof(int64_t) * n_fits, cudaMemcpyHostToDevice,
                                     k->stream));
    PSG_PACK_CUDA(k, cudaMemsetAsync(k->d_queue, 0, 2 * sizeof(unsigned long long), k->stream));
    psg::FitWork w{};
    w.n_lo = 1;
    w.nfits = n_fits;
    w.period_index = k->d_pidx;
    w.pole = k->d_pole;
    w.queue = k->d_queue;
    w.lit = k->d_queue + 1;
    w.scratch = k->d_scratch;
    w.scratch_stride = k->scratch_stride;
    w.out = k->d_out;
    w.objs = k->d_objs;
    w.cfgs = k->d_cfgs;
    w.object = k->d_obj;
    w.alpha_g = k->d_alpha_g;
    w.alpha_stride = static_cast<size_t>(k->ctx[0]->obj.mfit) * k->ctx[0]->obj.mfit;
    w.iter_limit = iter_limit;
    w.screen_iters = screen_iters;
    // predictor weights and trajectory records: launch-local device buffers
    struct Tmp {
        float *p = nullptr;
        ~Tmp() { cudaFree(p); }
    } d_w, d_traj;
    const size_t traj_bytes = static_cast<size_t>(n_fits) * psg::kTrajFloats * sizeof(float);
    if (weights) {
        PSG_PACK_CUDA(k, cudaMalloc(&d_w.p, psg::kMlpFloats * sizeof(float)));
        PSG_PACK_CUDA(k, cudaMemcpyAsync(d_w.p, weights, psg::kMlpFloats * sizeof(float), cudaMemcpyHostToDevice,
                                         k->stream));
        w.mlp = d_w.p;
    }
    if (traj) {
        PSG_PACK_CUDA(k, cudaMalloc(&d_traj.p, traj_bytes));
        PSG_PACK_CUDA(k, cudaMemsetAsync(d_traj.p, 0, traj_bytes, k->stream));
        w.traj = d_traj.p;
    }
    const int grid = static_cast<int>(std::min<int64_t>(k->slots, n_fits));
    PSG_PACK_CUDA(k, cudaEventRecord(k->ev[0], k->stream));
    int e = psg::launch_pack(k->form, w, k->ctx[0]->obj.ncoef, grid, k->P, k->smem, k->dsph_smem, k->stream);
    if (e != 0) return pack_fail(k, static_cast<cudaError_t>(e), "packed fit kernel launch");
    PSG_PACK_CUDA(k, cudaEventRecord(k->ev[1], k->stream));
    std::vector<ps_fit> sorted(static_cast<size_t>(n_fits));
    PSG_PACK_CUDA(k, cudaMemcpyAsync(sorted.data(), k->d_out, sizeof(ps_fit) * n_fits, cudaMemcpyDeviceToHost,
                                     k->stream));
    std::vector<float> traj_sorted(traj ? static_cast<size_t>(n_fits) * psg::kTrajFloats : 0);
    if (traj)
        PSG_PACK_CUDA(k, cudaMemcpyAsync(traj_sorted.data(), d_traj.p, traj_bytes, cudaMemcpyDeviceToHost, k->stream));
    unsigned long long lit = 0;
    PSG_PACK_CUDA(k, cudaMemcpyAsync(&lit, k->d_queue + 1, sizeof(lit), cudaMemcpyDeviceToHost, k->stream));
    PSG_PACK_CUDA(k, cudaStreamSynchronize(k->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, k->ev[0], k->ev[1]);
    int64_t evals = 0;
    for (int64_t i = 0; i < n_fits; i++) {
        const ps_fit &f = sorted[static_cast<size_t>(i)];
        const int64_t u = order[static_cast<size_t>(i)];
        out[u] = f;
        if (traj)
            std::memcpy(traj + u * psg::kTrajFloats, traj_sorted.data() + i * psg::kTrajFloats,
                        psg::kTrajFloats * sizeof(float));
        evals += f.niter + 1;
        if (f.err_code == 16) {
            k->err = "a tensor-core wait gave up: fit results are incomplete";
            return PS_ERR_TIMEOUT;
        }
    }
    k->timing = ps_timing{};
    k->timing.kernel_ms = ms;
    k->timing.total_ms = ms;
    k->timing.fits = n_fits;
    k->timing.evals = evals;
    k->timing.launches = 1;
    k->timing.lit_facets = static_cast<int64_t>(lit);
    return PS_OK;
}

}  // namespace

extern "C" {

ps_status ps_pack_fit(ps_pack *k, const double *conw_r, int64_t n_fits, const int32_t *object,
                      const int64_t *period_index, const int32_t *pole, ps_fit *out)
{
    return pack_run(k, conw_r, n_fits, object, period_index, pole, 0, 0, nullptr, nullptr, out);
}

ps_status ps_pack_screen(ps_pack *k, const double *conw_r, int64_t n_fits, const int32_t *object,
                         const int64_t *period_index, const int32_t *pole, int32_t screen_iters,
                         const float *weights, ps_fit *out)
{
    if (!weights || !screen_iters_ok(screen_iters)) return PS_ERR_ARG;
    return pack_run(k, conw_r, n_fits, object, period_index, pole, screen_iters, screen_iters, weights, nullptr,
                    out);
}

ps_status ps_pack_trajectories(ps_pack *k, const double *conw_r, int64_t n_fits, const int32_t *object,
                               const int64_t *period_index, const int32_t *pole, int32_t feat_iters, float *traj,
                               ps_fit *out)
{
    if (!traj || !screen_iters_ok(feat_iters)) return PS_ERR_ARG;
    return pack_run(k, conw_r, n_fits, object, period_index, pole, 0, feat_iters, nullptr, traj, out);
}

ps_status ps_pack_timing(const ps_pack *k, ps_timing *out)
{
    if (!k || !out) return PS_ERR_ARG;
    *out = k->timing;
    return PS_OK;
}

const char *ps_pack_last_error(const ps_pack *k) { return k ? k->err.c_str() : "null pack"; }

void ps_pack_destroy(ps_pack *k)
{
    if (!k) return;
    cudaSetDevice(k->device);
    if (k->stream) cudaStreamSynchronize(k->stream);
    cudaFree(k->d_objs);
    cudaFree(k->d_cfgs);
    cudaFree(k->d_scratch);
    cudaFree(k->d_alpha_g);
    cudaFree(k->d_queue);
    cudaFree(k->d_obj);
    cudaFree(k->d_pole);
    cudaFree(k->d_pidx);
    cudaFree(k->d_out);
    if (k->ev[0]) cudaEventDestroy(k->ev[0]);
    if (k->ev[1]) cudaEventDestroy(k->ev[1]);
    if (k->stream) cudaStreamDestroy(k->stream);
    delete k;
}

}  // extern "C"

extern "C" {

ps_status ps_last_timing(const ps_ctx *c, ps_timing *out)
{
    if (!c || !out) return PS_ERR_ARG;
    *out = c->timing;
    return PS_OK;
}

const char *ps_last_error(const ps_ctx *c) { return c ? c->err.c_str() : ""; }

void ps_destroy(ps_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->opt.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->d_tables);
    cudaFree(c->d_scratch);
    cudaFree(c->d_queue);
    cudaFree(c->d_out);
    cudaFree(c->d_pidx);
    cudaFree(c->d_pole);
    cudaFree(c->d_eval);
    cudaFree(c->d_state);
    cudaFree(c->d_slot);
    cudaFree(c->d_alpha_g);
    for (auto &e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

ps_status ps_device_fma_peaks(int32_t device, double *fp64_tflops, double *fp32_tflops)
{
    if (!fp64_tflops || !fp32_tflops) return PS_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return PS_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return PS_ERR_NO_DEVICE;
    int e = psg::measure_fma_peaks(fp64_tflops, fp32_tflops, nullptr);
    return e == 0 ? PS_OK : PS_ERR_CUDA;
}

ps_status ps_rows_from_fits(const ps_fit *fits, int64_t n_periods, int32_t ndata, ps_row *out)
{
    if (!fits || !out || n_periods < 0 || ndata < 1) return PS_ERR_ARG;
    for (int64_t n = 0; n < n_periods; n++) out[n] = psg::best_of_poles(fits + n * PS_N_POLES, ndata);
    return PS_OK;
}

int32_t ps_format_row(const ps_row *r, char *buf, size_t len)
{
    if (!r || !buf) return -1;
    return std::snprintf(buf, len, "%.8f  %.6f  %.6f %4.1f %4.0f %4.0f\n", r->period_h, r->rms, r->chi2,
                         r->dark_or_conw, r->lambda_deg, r->beta_deg);
}

ps_status ps_shape_tables(int32_t nrows, int32_t lmax, int32_t mmax, int32_t *nfac, int32_t *ncoef, double *nor,
                          double *darea, double *dsph)
{
    if (nrows < 1 || lmax < 0 || mmax < 0 || mmax > lmax || lmax > PS_MAX_LM || 8 * nrows * nrows > PS_MAX_N_FAC)
        return PS_ERR_ARG;
    psg::ShapeTables s;
    psg::build_shape(s, nrows, lmax, mmax);
    if (nfac) *nfac = s.nfac;
    if (ncoef) *ncoef = s.ncoef;
    if (nor) std::memcpy(nor, s.nor.data(), s.nor.size() * sizeof(double));
    if (darea) std::memcpy(darea, s.darea.data(), s.darea.size() * sizeof(double));
    if (dsph) std::memcpy(dsph, s.dsph.data(), s.dsph.size() * sizeof(double));
    return PS_OK;
}

// Process-level drop-in (period_search_BOINC.cpp:218-954): resume from the
// state file, run the convexity pre-pass, scan, append rows, checkpoint by
// writing "temp" next to the state file and renaming it (do_checkpoint,
// :85-101).
ps_status ps_run_files(const char *in_path, const char *out_path, const char *state_path, const ps_options *opt,
                       int32_t checkpoint_rows)
{
    if (!in_path || !out_path) return PS_ERR_ARG;
    ps_input *in = nullptr;
    ps_status st = ps_input_read(in_path, &in);
    if (st != PS_OK) return st;
    ps_problem prob;
    ps_input_problem(in, &prob);
    int64_t n_start_from = 1;
    bool resume = false;
    if (state_path) {
        FILE *sf = std::fopen(state_path, "r");
        if (sf) {
            int nlines = 0;
            if (std::fscanf(sf, "%d", &nlines) == 1) {
                n_start_from = nlines + 1;
                resume = true;
            }
            std::fclose(sf);
        }
    }
    ps_ctx *c = nullptr;
    st = ps_prepare(&prob, opt, &c);
    if (st != PS_OK) {
        ps_input_free(in);
        return st;
    }
    double conw_r = 0;
    int32_t new_conw = 0;
    st = ps_precalc_conw(c, &conw_r, &new_conw);
    FILE *f = nullptr;
    if (st == PS_OK) {
        f = std::fopen(out_path, resume ? "a" : "w");
        if (!f) st = PS_ERR_IO;
    }
    const int64_t n_max = c->obj.n_max;
    const int64_t chunk = std::max<int64_t>(checkpoint_rows > 0 ? checkpoint_rows : n_max, 1);
    std::vector<ps_row> rows;
    for (int64_t n0 = n_start_from; st == PS_OK && n0 <= n_max; n0 += chunk) {
        int64_t n1 = std::min(n_max, n0 + chunk - 1);
        rows.resize(static_cast<size_t>(n1 - n0 + 1));
        st = ps_scan(c, conw_r, n0, n1, rows.data());
        if (st != PS_OK) break;
        char line[256];
        for (const ps_row &r : rows) {
            ps_format_row(&r, line, sizeof line);
            std::fputs(line, f);
        }
        std::fflush(f);
        if (state_path && checkpoint_rows > 0) {
            std::string tmp = std::string(state_path) + ".temp";
            FILE *t = std::fopen(tmp.c_str(), "w");
            if (!t) {
                st = PS_ERR_IO;
                break;
            }
            std::fprintf(t, "%lld", static_cast<long long>(n1));
            std::fclose(t);
            if (std::rename(tmp.c_str(), state_path) != 0) st = PS_ERR_IO;
        }
    }
    if (f) std::fclose(f);
    ps_destroy(c);
    ps_input_free(in);
    return st;
}

}  // extern "C"

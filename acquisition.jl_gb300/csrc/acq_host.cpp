// acq_host.cpp — host-side plan geometry, validation, codes, patterns and CFAR.
//
// Compiled with -ffp-contract=off so that double-precision expressions round exactly as
// the reference's Julia (which never contracts a*b+c into an FMA) on both x86-64 and
// aarch64 hosts.
#include "acq_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <sstream>

namespace acq {

namespace {

// NH10 as +-1 (bits 0000110101, 0 -> +1); pinned by test/sign_patterns.jl:45-46.
const int8_t kNH10[10] = {1, 1, 1, 1, -1, -1, 1, -1, 1, -1};

// IS-GPS-200 phase-selector taps (G2 stages, 1-based) for PRN 1..32.
const int kL1Taps[32][2] = {{2, 6}, {3, 7}, {4, 8}, {5, 9}, {1, 9}, {2, 10}, {1, 8}, {2, 9},
                            {3, 10}, {2, 3}, {3, 4}, {5, 6}, {6, 7}, {7, 8}, {8, 9}, {9, 10},
                            {1, 4}, {2, 5}, {3, 6}, {4, 7}, {5, 8}, {6, 9}, {1, 3}, {4, 6},
                            {5, 7}, {6, 8}, {7, 9}, {8, 10}, {1, 6}, {2, 7}, {3, 8}, {4, 9}};

// IS-GPS-705 XB code advance (chips) for the I5 code, PRN 1..37.
const int kL5XbAdvance[37] = {266,  365,  804,  1138, 1509, 1559, 1756, 2084, 2170, 2303, 2527, 2687, 2930,
                              3471, 3940, 4132, 4332, 4924, 5343, 5443, 5641, 5816, 5898, 5918, 5955, 6243,
                              6345, 6477, 6518, 6875, 7168, 7187, 7329, 7577, 7720, 7777, 8057};

const SystemInfo kSystems[3] = {
    {ACQ_GPS_L1CA, "GPSL1CA", 1023, 1.023e6, 1575.42e6, 50.0, 1, nullptr, false, 32},
    {ACQ_GPS_L5I, "GPSL5I", 10230, 10.23e6, 1176.45e6, 100.0, 10, kNH10, false, 37},
    {ACQ_GALILEO_E1B, "GalileoE1B", 4092, 1.023e6, 1575.42e6, 250.0, 1, nullptr, true, 50},
};

std::string fmt_g(double v) {
    // Julia prints whole floats like "7000.0"; integers go through std::to_string.
    std::ostringstream o;
    o.precision(17);
    o << v;
    return o.str();
}

std::vector<int8_t> l1ca_chips(int prn) {
    int s1 = kL1Taps[prn - 1][0], s2 = kL1Taps[prn - 1][1];
    int g1[10], g2[10];
    for (int i = 0; i < 10; ++i) g1[i] = g2[i] = 1;
    std::vector<int8_t> out(1023);
    for (int i = 0; i < 1023; ++i) {
        int bit = g1[9] ^ g2[s1 - 1] ^ g2[s2 - 1];
        out[i] = static_cast<int8_t>(1 - 2 * bit);
        int f1 = g1[2] ^ g1[9];
        int f2 = g2[1] ^ g2[2] ^ g2[5] ^ g2[7] ^ g2[8] ^ g2[9];
        for (int k = 9; k > 0; --k) { g1[k] = g1[k - 1]; g2[k] = g2[k - 1]; }
        g1[0] = f1;
        g2[0] = f2;
    }
    return out;
}

void l5_xa_step(int* r) {
    int f = r[8] ^ r[9] ^ r[11] ^ r[12];
    for (int k = 12; k > 0; --k) r[k] = r[k - 1];
    r[0] = f;
}

void l5_xb_step(int* r) {
    int f = r[0] ^ r[2] ^ r[3] ^ r[5] ^ r[6] ^ r[7] ^ r[11] ^ r[12];
    for (int k = 12; k > 0; --k) r[k] = r[k - 1];
    r[0] = f;
}

std::vector<int8_t> l5i_primary_chips(int prn) {
    int xa[13], xb[13];
    for (int i = 0; i < 13; ++i) xa[i] = xb[i] = 1;
    for (int i = 0; i < kL5XbAdvance[prn - 1]; ++i) l5_xb_step(xb);
    std::vector<int8_t> out(10230);
    for (int i = 0; i < 10230; ++i) {
        if (i == 8190)  // XA short cycle
            for (int k = 0; k < 13; ++k) xa[k] = 1;
        out[i] = static_cast<int8_t>(1 - 2 * (xa[12] ^ xb[12]));
        l5_xa_step(xa);
        l5_xb_step(xb);
    }
    return out;
}

uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

std::vector<int8_t> e1b_synthetic_chips(int prn) {
    std::vector<int8_t> out(4092);
    for (int k = 0; k < 4092; ++k) {
        uint64_t h = splitmix64((static_cast<uint64_t>(prn) << 32) | static_cast<uint64_t>(k));
        out[k] = (h >> 63) ? -1 : 1;
    }
    return out;
}

bool is_whole(double x) { return std::floor(x) == x && std::fabs(x) < 4503599627370496.0; }

// ---- regularized incomplete gamma (Numerical-Recipes style series / Lentz continued fraction)
double log_gamma_q(double a, double x) {
    // log Q(a, x), accurate in the far upper tail.
    if (x <= 0) return 0.0;
    double lg = std::lgamma(a);
    if (x < a + 1.0) {
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 0; n < 100000; ++n) {
            ap += 1.0;
            del *= x / ap;
            sum += del;
            if (std::fabs(del) < std::fabs(sum) * 1e-17) break;
        }
        double logp = -x + a * std::log(x) - lg + std::log(sum);
        double p = std::exp(logp);
        return std::log1p(-p);
    }
    const double fpmin = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / fpmin, dd = 1.0 / b, h = dd;
    for (int i = 1; i < 100000; ++i) {
        double an = -i * (i - a);
        b += 2.0;
        dd = an * dd + b;
        if (std::fabs(dd) < fpmin) dd = fpmin;
        c = b + an / c;
        if (std::fabs(c) < fpmin) c = fpmin;
        dd = 1.0 / dd;
        double del = dd * c;
        h *= del;
        if (std::fabs(del - 1.0) < 1e-17) break;
    }
    return -x + a * std::log(x) - lg + std::log(h);
}

// Inverse standard normal upper tail via Acklam's rational approximation + one Halley step.
double norm_isf(double q) {
    static const double a[] = {-3.969683028665376e+01, 2.209460984245205e+02, -2.759285104469687e+02,
                               1.383577518672690e+02, -3.066479806614716e+01, 2.506628277459239e+00};
    static const double b[] = {-5.447609879822406e+01, 1.615858368580409e+02, -1.556989798598866e+02,
                               6.680131188771972e+01, -1.328068155288572e+01};
    static const double c[] = {-7.784894002430293e-03, -3.223964580411365e-01, -2.400758277161838e+00,
                               -2.549732539343734e+00, 4.374664141464968e+00, 2.938163982698783e+00};
    static const double d[] = {7.784695709041462e-03, 3.224671290700398e-01, 2.445134137142996e+00,
                               3.754408661907416e+00};
    double p = 1.0 - q;  // lower-tail probability of the quantile we want
    double x;
    if (q < 0.02425) {
        double t = std::sqrt(-2.0 * std::log(q));
        x = -(((((c[0] * t + c[1]) * t + c[2]) * t + c[3]) * t + c[4]) * t + c[5]) /
            ((((d[0] * t + d[1]) * t + d[2]) * t + d[3]) * t + 1.0);
        x = -x;
    } else if (p < 0.02425) {
        double t = std::sqrt(-2.0 * std::log(p));
        x = (((((c[0] * t + c[1]) * t + c[2]) * t + c[3]) * t + c[4]) * t + c[5]) /
            ((((d[0] * t + d[1]) * t + d[2]) * t + d[3]) * t + 1.0);
    } else {
        double t = p - 0.5, r = t * t;
        x = (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * t /
            (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1.0);
    }
    return x;
}

}  // namespace

const SystemInfo& system_info(int id) {
    if (id < 0 || id > 2) throw AcqError(ACQ_ERR_ARGUMENT, "unknown system id " + std::to_string(id));
    return kSystems[id];
}

int nextprod_2357(int n) {
    for (int m = std::max(n, 1);; ++m) {
        int k = m;
        for (int p : {2, 3, 5, 7})
            while (k % p == 0) k /= p;
        if (k == 1) return m;
    }
}

std::vector<int> fft_radices(int n) {
    std::vector<int> r;
    while (n % 4 == 0) { r.push_back(4); n /= 4; }
    while (n % 2 == 0) { r.push_back(2); n /= 2; }
    for (int p : {3, 5, 7})
        while (n % p == 0) { r.push_back(p); n /= p; }
    for (int p = 11; n > 1; p += 2)
        while (n % p == 0) { r.push_back(p); n /= p; }
    return r;
}

Geometry compute_geometry(const acq_plan_desc& d) {
    const SystemInfo& s = system_info(d.system);
    const int n_nc = d.num_noncoherent_accumulations;
    const int n_coh = d.num_coherently_integrated_code_periods;
    const int n_be = d.bit_edge_search_steps;
    auto arg = [](const std::string& m) { return AcqError(ACQ_ERR_ARGUMENT, m); };
    // src/plan.jl:325-330
    if (n_nc < 1) throw arg("num_noncoherent_accumulations must be >= 1, got " + std::to_string(n_nc));
    if (n_coh < 1) throw arg("num_coherently_integrated_code_periods must be >= 1");
    if (n_be < 1) throw arg("bit_edge_search_steps must be >= 1, got " + std::to_string(n_be));
    if (n_coh == 1 && n_be > 1)
        throw arg("bit_edge_search_steps must be 1 when num_coherently_integrated_code_periods == 1 "
                  "(sub-bit mode; no bit boundary search applies), got " + std::to_string(n_be));
    if (!(d.sampling_freq_hz > 0) || !std::isfinite(d.sampling_freq_hz))
        throw arg("sampling_freq must be positive and finite, got " + fmt_g(d.sampling_freq_hz));
    if (!(d.min_doppler_coverage_hz >= 0) || !std::isfinite(d.min_doppler_coverage_hz))
        throw arg("min_doppler_coverage must be >= 0 and finite, got " + fmt_g(d.min_doppler_coverage_hz));
    if (d.noise_estimator != ACQ_NOISE_OPPOSITE_ROW && d.noise_estimator != ACQ_NOISE_GLOBAL_MEAN)
        throw arg("unknown noise estimator " + std::to_string(d.noise_estimator));
    // src/plan.jl:335-383
    const int L = s.secondary_length;
    const bool use_sec = d.use_secondary_code != 0;
    if (use_sec && L > 1 && n_coh > 1 && L > d.max_secondary_code_rotations)
        throw arg(std::string("Secondary-code rotation search size exceeds the per-plan cap for ") + s.name +
                  ": get_secondary_code_length(system)=" + std::to_string(L) +
                  " > max_secondary_code_rotations=" + std::to_string(d.max_secondary_code_rotations) +
                  " at num_coherently_integrated_code_periods=" + std::to_string(n_coh) +
                  ". Remedies (in order): (1) reduce num_coherently_integrated_code_periods; "
                  "(2) raise max_secondary_code_rotations to at least " + std::to_string(L) +
                  "; or (3) set use_secondary_code = false to opt out of the rotation search.");
    if (use_sec && L > 1 && n_coh > 1 && n_coh % L != 0)
        throw arg("Secondary-code rotation search requires num_coherently_integrated_code_periods to be a whole "
                  "multiple of the secondary-code length L=" + std::to_string(L) +
                  ", got num_coherently_integrated_code_periods=" + std::to_string(n_coh) +
                  ". A partial secondary-code period makes the rotation search produce a +-Doppler sign "
                  "ambiguity — a near-equal mirror peak at -f whose sign flips at random under noise "
                  "(issue #68). Remedies (in order): (1) set num_coherently_integrated_code_periods to a "
                  "multiple of " + std::to_string(L) + " (e.g. " + std::to_string(L) +
                  " for one full secondary-code period); (2) set num_coherently_integrated_code_periods = 1 "
                  "and raise num_noncoherent_accumulations for a robust sign at coarser Doppler resolution; "
                  "or (3) set use_secondary_code = false to opt out of the rotation search.");
    Geometry g{};
    const double fs = d.sampling_freq_hz;
    // src/plan.jl:386 — same float64 op order: code_length / code_freq * fs
    const double spc_f = static_cast<double>(s.code_length) / s.code_freq * fs;
    if (spc_f > 2.0e9) throw arg("samples_per_code too large");
    g.spc = static_cast<int>(std::ceil(spc_f));
    // src/plan.jl:389-397
    const bool has_data = std::isfinite(s.data_freq) && s.data_freq > 0;
    if (has_data) {
        long long bit_samples = static_cast<long long>(std::ceil(fs / s.data_freq));
        g.bit_period_codes = static_cast<int>(bit_samples / g.spc);
    } else {
        g.bit_period_codes = n_coh;
    }
    // src/plan.jl:413-432
    const double bin_width = fs / g.spc;
    const double mnb_f = std::ceil(2 * d.min_doppler_coverage_hz / bin_width + 2.0 / n_coh);
    long long min_num_blocks = static_cast<long long>(mnb_f);
    int nb = 0;
    for (long long c = std::max(1LL, min_num_blocks); c <= g.spc; ++c)
        if (g.spc % c == 0) { nb = static_cast<int>(c); break; }
    if (nb == 0)
        throw arg("No valid num_blocks found: samples_per_code=" + std::to_string(g.spc) +
                  " has no divisor >= min_num_blocks=" + std::to_string(min_num_blocks) +
                  ". This should not happen for standard GNSS sampling frequencies — please file a bug.");
    // src/plan.jl:440-446
    if (has_data && n_coh >= g.bit_period_codes) {
        if (g.bit_period_codes <= 0 || n_coh % g.bit_period_codes != 0)
            throw arg("num_coherently_integrated_code_periods=" + std::to_string(n_coh) +
                      " must be divisible by bit_period_codes=" + std::to_string(g.bit_period_codes) +
                      " (code periods per data bit).");
        if (g.bit_period_codes % n_be != 0)
            throw arg("bit_edge_search_steps=" + std::to_string(n_be) + " must divide bit_period_codes=" +
                      std::to_string(g.bit_period_codes) + ".");
    }
    g.nb = nb;
    g.bs = g.spc / nb;
    g.fft_size = nextprod_2357(2 * g.bs);
    g.fft_tile = g.fft_size;
    g.ndb = (has_data && n_coh >= g.bit_period_codes) ? n_coh / g.bit_period_codes : 1;
    g.n_coh = n_coh;
    g.n_be = n_be;
    g.n_nc = n_nc;
    g.ndop = n_coh * nb;
    // src/plan.jl:493-495
    g.coverage = nb * fs / g.spc;
    g.doppler_step = g.coverage / g.ndop;
    g.doppler_first = -g.coverage / 2;
    g.doppler_freqs.resize(g.ndop);
    for (int i = 0; i < g.ndop; ++i) g.doppler_freqs[i] = g.doppler_first + i * g.doppler_step;
    // src/plan.jl:511-525, :534-535
    const bool rot = use_sec && L > 1 && n_coh > 1;
    g.R = rot ? L : 1;
    g.spc_eff = g.spc * g.R;
    const bool sign = g.ndb > 1 || n_be > 1 || rot;
    g.path = rot ? 2 : (sign ? 1 : 0);
    if (g.path != 0) {
        const int bpc_k = n_coh / g.ndb;
        if ((long long)bpc_k * nb / n_be < 1)
            throw arg("bit_edge_search_steps=" + std::to_string(n_be) + " leaves no whole edge step");
    }
    if (g.path == 1 && (1 << (g.ndb - 1)) > 4096) throw arg("too many data-bit combinations");
    if ((long long)g.ndop * g.spc_eff > 2000000000LL) throw arg("search grid too large");
    g.noise_estimator = d.noise_estimator;
    g.use_secondary_code = use_sec ? 1 : 0;
    g.cfar_thr = cfar_threshold(0.01, (int64_t)g.ndop * g.spc * g.R, n_nc);
    return g;
}

std::vector<int8_t> full_chips(int system, int prn) {
    const SystemInfo& s = system_info(system);
    if (prn < 1 || prn > s.max_prn)
        throw AcqError(ACQ_ERR_ARGUMENT, std::string(s.name) + " PRN must be in 1:" + std::to_string(s.max_prn) +
                                             ", got " + std::to_string(prn));
    std::vector<int8_t> p = system == ACQ_GPS_L1CA ? l1ca_chips(prn)
                          : system == ACQ_GPS_L5I  ? l5i_primary_chips(prn)
                                                   : e1b_synthetic_chips(prn);
    if (s.secondary_length <= 1) return p;
    std::vector<int8_t> full(static_cast<size_t>(p.size()) * s.secondary_length);
    for (int k = 0; k < s.secondary_length; ++k)
        for (size_t i = 0; i < p.size(); ++i) full[k * p.size() + i] = static_cast<int8_t>(p[i] * s.secondary[k]);
    return full;
}

void gen_code(int system, int prn, int64_t n, double fs, double fc, double start_phase, int8_t* out) {
    const SystemInfo& s = system_info(system);
    if (fc <= 0) fc = s.code_freq;
    std::vector<int8_t> chips = full_chips(system, prn);
    const int64_t L = static_cast<int64_t>(chips.size());
    double sp = std::fmod(start_phase, static_cast<double>(L));
    if (sp < 0) sp += L;
    if (sp == 0.0 && is_whole(fs) && is_whole(fc)) {
        const int64_t fsi = static_cast<int64_t>(fs), fci = static_cast<int64_t>(fc);
        for (int64_t i = 0; i < n; ++i) {
            __int128 num = static_cast<__int128>(i) * fci;
            int64_t idx = static_cast<int64_t>(num / fsi);
            int64_t rem = static_cast<int64_t>(num - static_cast<__int128>(idx) * fsi);
            int8_t v = chips[idx % L];
            if (s.boc11 && 2 * rem >= fsi) v = static_cast<int8_t>(-v);
            out[i] = v;
        }
        return;
    }
    const double ratio = fc / fs;
    for (int64_t i = 0; i < n; ++i) {
        double ph = sp + static_cast<double>(i) * ratio;
        double fl = std::floor(ph);
        int64_t idx = static_cast<int64_t>(fl);
        int8_t v = chips[((idx % L) + L) % L];
        if (s.boc11 && (ph - fl) >= 0.5) v = static_cast<int8_t>(-v);
        out[i] = v;
    }
}

std::vector<float> sign_patterns(int system, int prn, int ndb, int R, int n_coh, bool use_secondary) {
    const SystemInfo& s = system_info(system);
    const int combos = 1 << (ndb - 1);
    const bool sec_active = use_secondary && R > 1;
    const int num_sec = sec_active ? R : 1;
    const int coh_per_bit = n_coh / ndb;
    const int L = sec_active ? R : 1;
    std::vector<float> pat(static_cast<size_t>(n_coh) * combos * num_sec);
    int col = 0;
    for (int r = 0; r < num_sec; ++r)
        for (int dd = 0; dd < combos; ++dd, ++col)
            for (int k = 0; k < n_coh; ++k) {
                int bit_idx = k / coh_per_bit;
                float data_sign = bit_idx == 0 ? 1.0f : (((dd >> (bit_idx - 1)) & 1) == 0 ? 1.0f : -1.0f);
                float sec_sign = sec_active ? static_cast<float>(s.secondary[(k + r) % L]) : 1.0f;
                pat[static_cast<size_t>(col) * n_coh + k] = data_sign * sec_sign;
            }
    return pat;
}

bool code_drift_shifts(const Geometry& g, const SystemInfo& s, double fs, int step, int32_t* out) {
    if (step == 0) {
        for (int r = 0; r < g.ndop; ++r) out[r] = 0;
        return false;
    }
    const double carrier = s.center_freq;
    const double dur = static_cast<double>(g.n_coh) * g.spc / fs;
    bool any = false;
    for (int r = 0; r < g.ndop; ++r) {
        // src/noncoherent_integration.jl:612 — same left-to-right float64 ops, round half to even
        double v = g.doppler_freqs[r] * step * dur * fs / carrier;
        long long raw = static_cast<long long>(std::nearbyint(v));
        if (raw != 0) any = true;
        long long m = raw % g.spc;
        if (m < 0) m += g.spc;
        out[r] = static_cast<int32_t>(m);
    }
    return any;
}

double cfar_threshold(double pfa, int64_t num_cells, int M) {
    if (!(pfa > 0 && pfa < 1)) throw AcqError(ACQ_ERR_ARGUMENT, "pfa must be in (0, 1), got " + fmt_g(pfa));
    if (num_cells <= 0)
        throw AcqError(ACQ_ERR_ARGUMENT, "num_cells must be positive, got " + std::to_string(num_cells));
    if (M <= 0) throw AcqError(ACQ_ERR_ARGUMENT, "num_noncoherent_integrations must be positive");
    // src/cfar.jl:70: identical float64 expression
    const double pfa_cell = 1 - std::pow(1 - pfa, 1 / static_cast<double>(num_cells));
    const double a = static_cast<double>(M);
    if (!(pfa_cell > 0)) throw AcqError(ACQ_ERR_ARGUMENT, "per-cell false-alarm probability underflows to 0");
    const double logq = std::log(pfa_cell);
    double x;
    if (M == 1) {
        x = -logq;  // Q(1, x) = exp(-x)
    } else {
        // Wilson-Hilferty start, then Newton on log Q (DiDonato-Morris style refinement).
        double z = norm_isf(pfa_cell);
        double t = 1.0 - 1.0 / (9.0 * a) + z / (3.0 * std::sqrt(a));
        x = a * t * t * t;
        if (!(x > 0)) x = std::max(1e-3, -logq);
        for (int it = 0; it < 200; ++it) {
            double lq = log_gamma_q(a, x);
            // d/dx log Q = -x^{a-1} e^{-x} / (Gamma(a) Q)
            double logdens = (a - 1) * std::log(x) - x - std::lgamma(a);
            double dlog = -std::exp(logdens - lq);
            double step = (lq - logq) / dlog;
            double xn = x - step;
            if (!(xn > 0)) xn = x / 2;
            if (std::fabs(xn - x) <= 1e-15 * x) { x = xn; break; }
            x = xn;
        }
    }
    return x / a;
}

// src/plot.jl:16-20 (_fmdbzp_column_to_tau) and :35-57 (_fmdbzp_sort_by_chip): chip phase
// mod(-tau * fc / fs, code_length) per column with Julia's floating-point mod, then a stable
// sort (Julia's sortperm keeps equal keys in index order).
bool is_whole_freq(double x) { return is_whole(x); }

void chip_order(int num_blocks, int block_size, int64_t width, double code_freq, double fs, int32_t* perm,
                double* axis) {
    if (num_blocks < 1 || block_size < 1 || width < 1 || !(code_freq > 0) || !(fs > 0))
        throw AcqError(ACQ_ERR_ARGUMENT, "chip order needs positive num_blocks, block_size, width and frequencies");
    const double code_length = static_cast<double>(width) * code_freq / fs;
    std::vector<double> chip(static_cast<size_t>(width));
    for (int64_t c = 0; c < width; ++c) {
        const int64_t block_row = c / block_size, within = c % block_size;
        const int64_t tau = (((num_blocks - block_row) % num_blocks + num_blocks) % num_blocks) * block_size + within;
        const double x = -static_cast<double>(tau) * code_freq / fs;
        double r = std::fmod(x, code_length);
        if (r == 0.0) r = 0.0;                  // copysign(r, code_length)
        else if ((r > 0) != (code_length > 0)) r += code_length;
        chip[static_cast<size_t>(c)] = r;
    }
    std::vector<int32_t> idx(static_cast<size_t>(width));
    for (int64_t i = 0; i < width; ++i) idx[static_cast<size_t>(i)] = static_cast<int32_t>(i);
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return chip[a] < chip[b]; });
    for (int64_t i = 0; i < width; ++i) {
        perm[i] = idx[static_cast<size_t>(i)];
        if (axis) axis[i] = chip[static_cast<size_t>(idx[static_cast<size_t>(i)])];
    }
}

}  // namespace acq

// vpf_tables.cu -- host side of the library: error state, parameter defaults, numpy-exact
// grids and the per-grid device lookup tables used by every kernel.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

static thread_local std::string t_last_error;

int set_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return code;
}

int check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return ABM_OK;
    return set_error(ABM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int allow_dynamic_smem(const void *func, int bytes, const char *what) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> done;   // (device, kernel) -> bytes
    int dev = 0;
    int st = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    std::lock_guard<std::mutex> lk(mu);
    auto it = done.find({dev, func});
    if (it != done.end() && it->second >= bytes) return ABM_OK;
    st = check_cuda(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                    what);
    if (!st) done[{dev, func}] = bytes;
    return st;
}

// np.linspace(-pi, pi, n) (numpy 2.x: arange(n) * step + start, last element = stop).
void np_linspace_pi(int n, std::vector<double> &out) {
    out.resize(n);
    if (n == 1) {
        out[0] = -kPi;
        return;
    }
    const double delta = kPi - (-kPi);
    const double step = delta / (double)(n - 1);
    for (int k = 0; k < n; ++k) {
        double y = (double)k * step;
        out[k] = y + (-kPi);
    }
    out[n - 1] = kPi;
}

// np.arange(-pi, pi, 2*pi/rv): length ceil((stop - start) / step); a[i] = start + i * delta
// with delta = (start + step) - start (numpy's DOUBLE_fill).
int np_arange_phi(int rv, std::vector<double> *out) {
    const double start = -kPi, stop = kPi, step = (2 * kPi) / (double)rv;
    const double len_d = std::ceil((stop - start) / step);
    const int len = len_d > 0 ? (int)len_d : 0;
    if (out) {
        out->resize(len);
        const double a1 = start + step;
        const double delta = a1 - start;
        for (int i = 0; i < len; ++i)
            (*out)[i] = (i == 0) ? start : (i == 1 ? a1 : start + (double)i * delta);
    }
    return len;
}

int find_nearest(const std::vector<double> &a, double v) {  // supcalc.py:8-11
    if (std::isnan(v)) return 0;
    int best = 0;
    double bv = std::fabs(a[0] - v);
    for (size_t k = 1; k < a.size(); ++k) {
        double d = std::fabs(a[k] - v);
        if (d < bv) {
            bv = d;
            best = (int)k;
        }
    }
    return best;
}

// Trapezoid prefix sums and point values of cos/sin over an integration grid, fixed point.
static void integral_tables(const std::vector<double> &phi, int rv,
                            std::vector<long long> &q, std::vector<long long> &cpt,
                            long long &qc_total, long long &qs_total) {
    q.assign(2 * (size_t)(rv + 1), 0);
    cpt.assign(2 * (size_t)rv, 0);
    long double qc = 0, qs = 0;
    for (int k = 0; k < rv; ++k) {
        const double c = std::cos(phi[k]), s = std::sin(phi[k]);
        q[2 * k] = llroundl(qc * (long double)kFix);
        q[2 * k + 1] = llroundl(qs * (long double)kFix);
        cpt[2 * k] = llroundl((long double)c * (long double)kFix);
        cpt[2 * k + 1] = llroundl((long double)s * (long double)kFix);
        long double dl = (k > 0) ? (long double)(phi[k] - phi[k - 1]) : 0.0L;
        long double dr = (k + 1 < rv) ? (long double)(phi[k + 1] - phi[k]) : 0.0L;
        long double w = (dl + dr) / 2;   // trapezoid weight of sample k (scipy trapz over phi)
        qc += w * c;
        qs += w * s;
    }
    q[2 * rv] = llroundl(qc * (long double)kFix);
    q[2 * rv + 1] = llroundl(qs * (long double)kFix);
    qc_total = q[2 * rv];
    qs_total = q[2 * rv + 1];
}

struct GridEntry {
    GridDev g;
    void *mem = nullptr;
};

static std::mutex g_mu;
static std::map<std::tuple<int, int, double, double>, GridEntry> g_grids;
static std::map<std::tuple<int, int, std::string>, GridEntry> g_phi_grids;

static int upload(const std::vector<std::pair<const void *, size_t>> &parts, void **mem,
                  std::vector<void *> &ptrs) {
    size_t total = 0;
    std::vector<size_t> offs;
    for (auto &p : parts) {
        offs.push_back(total);
        total += (p.second + 255) & ~size_t(255);
    }
    void *d = nullptr;
    int st = check_cuda(cudaMalloc(&d, total > 0 ? total : 256), "cudaMalloc(grid tables)");
    if (st) return st;
    for (size_t i = 0; i < parts.size(); ++i) {
        char *dst = (char *)d + offs[i];
        ptrs.push_back(dst);
        if (parts[i].second) {
            st = check_cuda(cudaMemcpy(dst, parts[i].first, parts[i].second,
                                       cudaMemcpyHostToDevice),
                            "cudaMemcpy(grid tables)");
            if (st) {
                cudaFree(d);
                return st;
            }
        }
    }
    *mem = d;
    return ABM_OK;
}

int build_grid_host(int rv, double fov0, double fov1, GridHostTables &t) {
    std::vector<double> phis;
    np_linspace_pi(rv, phis);
    GridDev &g = t.g;
    memset(&g, 0, sizeof(g));
    g.rv = rv;
    g.words = (rv + 31) / 32;
    g.f0 = find_nearest(phis, fov0);
    g.f1 = find_nearest(phis, fov1);
    g.kmax = (rv + 3) / 4;
    g.full_fov = (g.f0 == 0 && g.f1 == rv - 1 && rv >= 3) ? 1 : 0;
    const double inv_delta = (double)(rv - 1) / (2 * kPi);
    g.inv_delta = (float)inv_delta;
    g.half_rm1 = (float)(0.5 * (rv - 1));
    g.rvm1 = (float)(rv - 1);
    g.ps2_scale = (float)((double)rv / (2 * kPi));
    // FP32 bearing error <= 1e-6 rad (atan2 + inputs) plus the rounding of u (~2^-22 u).
    g.band_t = (float)(1e-6 * inv_delta + 2.4e-7 * rv);
    g.band_h = 2e-6f;
    if (rv > 4) {
        const double tn = std::tan(2 * kPi / rv);
        g.cull = (float)((1.0 / (tn * tn)) * (1.0 + 1e-5));
    } else {
        g.cull = 0.f;
    }
    t.mid.resize(4 * (size_t)std::max(rv - 1, 1));
    for (int k = 0; k + 1 < rv; ++k) {
        const double m = 0.5 * (phis[k] + phis[k + 1]);
        const double c = std::cos(m), s = std::sin(m);
        const float ch = (float)c, sh = (float)s;
        t.mid[4 * k] = ch;
        t.mid[4 * k + 1] = (float)(c - (double)ch);
        t.mid[4 * k + 2] = sh;
        t.mid[4 * k + 3] = (float)(s - (double)sh);
    }
    t.cot2.assign(2 * (size_t)std::max(g.kmax, 1), 0.f);
    t.cot2[0] = INFINITY;
    for (int k = 1; k < g.kmax; ++k) {
        const double tn = std::tan(2 * kPi * k / rv);
        const double c2 = 1.0 / (tn * tn);
        const float hi = (float)c2;
        t.cot2[2 * k] = hi;
        t.cot2[2 * k + 1] = (float)(c2 - (double)hi);
    }
    std::vector<double> phi;
    const int len = np_arange_phi(rv, &phi);
    g.phi_ok = (len == rv);
    if (len < rv) phi.resize(rv, phi.empty() ? -kPi : phi.back());
    integral_tables(phi, rv, t.q, t.cpt, g.qc_total, g.qs_total);
    return ABM_OK;
}

const GridDev *grid_for(int rv, double fov0, double fov1, int *status) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_tuple(dev, rv, fov0, fov1);
    auto it = g_grids.find(key);
    if (it != g_grids.end()) {
        *status = ABM_OK;
        return &it->second.g;
    }
    GridHostTables t;
    build_grid_host(rv, fov0, fov1, t);
    GridEntry e;
    e.g = t.g;
    std::vector<void *> ptrs;
    int st = upload({{t.mid.data(), t.mid.size() * sizeof(float)},
                     {t.cot2.data(), t.cot2.size() * sizeof(float)},
                     {t.q.data(), t.q.size() * sizeof(long long)},
                     {t.cpt.data(), t.cpt.size() * sizeof(long long)}},
                    &e.mem, ptrs);
    if (st) {
        *status = st;
        return nullptr;
    }
    e.g.mid = (const float4 *)ptrs[0];
    e.g.cot2 = (const float2 *)ptrs[1];
    e.g.q = (const longlong2 *)ptrs[2];
    e.g.cpt = (const longlong2 *)ptrs[3];
    auto res = g_grids.emplace(key, e);
    *status = ABM_OK;
    return &res.first->second.g;
}

const GridDev *grid_for_phi(int rv, const double *phi, int *status) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::string blob((const char *)phi, sizeof(double) * (size_t)rv);
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_tuple(dev, rv, blob);
    auto it = g_phi_grids.find(key);
    if (it != g_phi_grids.end()) {
        *status = ABM_OK;
        return &it->second.g;
    }
    std::vector<double> ph(phi, phi + rv);
    std::vector<long long> q, cpt;
    GridEntry e;
    memset(&e.g, 0, sizeof(e.g));
    e.g.rv = rv;
    e.g.words = (rv + 31) / 32;
    e.g.phi_ok = 1;
    integral_tables(ph, rv, q, cpt, e.g.qc_total, e.g.qs_total);
    std::vector<void *> ptrs;
    int st = upload({{q.data(), q.size() * sizeof(long long)},
                     {cpt.data(), cpt.size() * sizeof(long long)}},
                    &e.mem, ptrs);
    if (st) {
        *status = st;
        return nullptr;
    }
    e.g.q = (const longlong2 *)ptrs[0];
    e.g.cpt = (const longlong2 *)ptrs[1];
    auto res = g_phi_grids.emplace(key, e);
    *status = ABM_OK;
    return &res.first->second.g;
}

void sincos_table_host(std::vector<float> &tab) {
    tab.assign(4 * (size_t)kSinCosTab, 0.f);
    for (int k = 0; k < kSinCosTab; ++k) {
        const long double a = (long double)k * 2.0L * 3.14159265358979323846264338327950288L /
                              (long double)kSinCosTab;
        const long double c = cosl(a), sn = sinl(a);
        const float ch = (float)c, sh = (float)sn;
        tab[4 * k] = ch;
        tab[4 * k + 1] = (float)(c - (long double)ch);
        tab[4 * k + 2] = sh;
        tab[4 * k + 3] = (float)(sn - (long double)sh);
    }
}

// cos/sin(k 2pi / kSinCosTab) as double-float pairs in global memory (per device), for
// kernels outside the translation unit that holds the __constant__ copy.
const float4 *sincos_table_dev(int *status) {
    static std::mutex mu;
    static std::map<int, const float4 *> tabs;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = tabs.find(dev);
    if (it != tabs.end()) {
        *status = ABM_OK;
        return it->second;
    }
    std::vector<float> tab;
    sincos_table_host(tab);
    void *mem = nullptr;
    std::vector<void *> ptrs;
    int st = upload({{tab.data(), tab.size() * sizeof(float)}}, &mem, ptrs);
    if (st) {
        *status = st;
        return nullptr;
    }
    tabs[dev] = (const float4 *)ptrs[0];
    *status = ABM_OK;
    return (const float4 *)ptrs[0];
}

}  // namespace abm

using namespace abm;

extern "C" {

int abm_vpf_abi_version(void) { return ABM_VPF_ABI_VERSION; }

const char *abm_last_error_string(void) { return t_last_error.c_str(); }

int abm_vf_params_default(abm_vf_params *p) {
    if (!p) return set_error(ABM_ERR_INVALID_ARG, "abm_vf_params_default: p is NULL");
    memset(p, 0, sizeof(*p));
    p->gam = 0.1;     // vf_params.py:12 (key VF_GAMMA, unset in the shipped .env files)
    p->v0 = 1.0;
    p->alp0 = 1.0;
    p->alp1 = 0.09;
    p->alp2 = 0.0;
    p->bet0 = 1.0;
    p->bet1 = 0.09;
    p->bet2 = 0.0;
    p->boundary = ABM_BOUNDARY_WALLS;
    p->limit_movement = 0;
    p->max_vel = 3.0;
    p->max_th = 0.1;
    p->width = 600.0;  // sims.py:60
    p->height = 480.0;
    p->window_pad = 30.0;
    p->fov0 = -kPi;
    p->fov1 = kPi;
    p->rv = 800;
    p->radius = 10.0;
    p->dt = 1.0;
    return ABM_OK;
}

int abm_phi_table(int32_t rv, double *phi_host, int32_t cap) {
    if (rv < 2 || rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "abm_phi_table: rv=%d", rv);
    std::vector<double> phi;
    const int len = np_arange_phi(rv, &phi);
    if (phi_host)
        for (int i = 0; i < len && i < cap; ++i) phi_host[i] = phi[i];
    return len;
}

int abm_vpf_words(int32_t rv) {
    if (rv < 1 || rv > ABM_MAX_RV) return set_error(ABM_ERR_RV, "abm_vpf_words: rv=%d", rv);
    return (rv + 31) / 32;
}

}  // extern "C"

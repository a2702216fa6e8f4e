// Error reporting, version and argument checks shared by all entry points.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <string>

#include "smx_internal.cuh"

namespace smx {

static thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};

void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int set_error(int status, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

void clear_error() { g_last_error.clear(); }

int check_cuda(cudaError_t e, const char *what) {
    return set_error(SMX_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

int validate_potential(const smx_potential *p) {
    if (!p) return set_error(SMX_ERR_ARGUMENT, "potential is NULL");
    const double v[] = {p->halo_M, p->halo_Rs, p->halo_qa, p->halo_qb, p->halo_qc, p->disc_M,
                        p->disc_a, p->disc_b, p->bar_M, p->bar_a, p->bar_b, p->bar_L,
                        p->bar_gamma, p->bulge_M, p->bulge_a, p->bulge_b, p->bulge_L,
                        p->bulge_gamma};
    for (double x : v)
        if (!std::isfinite(x)) return set_error(SMX_ERR_NONFINITE, "non-finite potential parameter");
    if (p->halo_Rs <= 0 || p->halo_qa <= 0 || p->halo_qb <= 0 || p->halo_qc <= 0)
        return set_error(SMX_ERR_ARGUMENT, "NFW scale radius and axis ratios must be > 0");
    if (p->bar_L <= 0 || p->bulge_L <= 0)
        return set_error(SMX_ERR_UNSUPPORTED,
                         "needle half-length L must be > 0 (axisymmetric Dehnen models are not built)");
    if (p->bar_a + p->bar_b <= 0 || p->bulge_a + p->bulge_b <= 0 || p->disc_a + p->disc_b <= 0)
        return set_error(SMX_ERR_ARGUMENT, "scale lengths must be > 0");
    for (int t : {p->bar_type, p->bulge_type})
        if (!(t == 0 || (t >= 1 && t <= 4) || (t >= 11 && t <= 14)))
            return set_error(SMX_ERR_UNSUPPORTED, "Dehnen model type %d is not built (T1-T4, V1-V4)", t);
    if (p->cyl_n_modes != 0) {
        if (p->cyl_n_modes < 0 || p->cyl_n_modes > 64 || p->cyl_n_r < 4 || p->cyl_n_z < 4)
            return set_error(SMX_ERR_ARGUMENT, "cylindrical spline: 1..64 modes and at least 4 grid points per axis");
        if (!(p->cyl_r0 > 0) || !std::isfinite(p->cyl_r0))
            return set_error(SMX_ERR_ARGUMENT, "cylindrical spline: r0 must be finite and > 0");
        if (!p->cyl_r_grid || !p->cyl_z_grid || !p->cyl_coef)
            return set_error(SMX_ERR_ARGUMENT, "cylindrical spline: NULL table");
    }
    return SMX_OK;
}

}  // namespace smx

extern "C" {

int smx_version(void) { return 100; }

unsigned long long smx_kernel_launches(void) { return smx::g_launches.load(std::memory_order_relaxed); }

const char *smx_status_string(int s) {
    switch (s) {
        case SMX_OK: return "ok";
        case SMX_ERR_ARGUMENT: return "invalid argument";
        case SMX_ERR_UNSUPPORTED: return "unsupported";
        case SMX_ERR_NONFINITE: return "non-finite value";
        case SMX_ERR_ITERATION_CAP: return "iteration cap reached";
        case SMX_ERR_CUDA: return "CUDA error";
        case SMX_ERR_WORKSPACE: return "workspace too small";
        case SMX_ERR_NUMERIC: return "numerical failure";
        default: return "unknown status";
    }
}

size_t smx_last_error(char *buf, size_t len) {
    const std::string &e = smx::g_last_error;
    if (buf && len) {
        size_t k = e.size() < len - 1 ? e.size() : len - 1;
        memcpy(buf, e.data(), k);
        buf[k] = 0;
    }
    return e.size();
}

}  // extern "C"

// Host build of the device L-BFGS-B state machine (botorch_gb300/csrc/lbfgsb_core.cuh)
// with one thread per restart, for tests that step it in lock-step with scipy's
// routine on the CPU. Test infrastructure: the library never calls it.
#define LB_HOST_EMU 1
#include <math.h>
#include <stdint.h>

#include <vector>

#include "lbfgsb_core.cuh"

using namespace bgb_lb;

extern "C" {

long long emu_workspace_bytes(long long R, long long n, int m) { return make_layout(R, n, m).total; }

void emu_init(long long R, int n, int m, double* X, const double* lo, const double* hi, char* ws) {
    InitArgs a;
    a.L = make_layout(R, n, m);
    a.R = R;
    a.n = n;
    a.m = m;
    a.ws = ws;
    a.X = X;
    a.lo = lo;
    a.hi = hi;
    std::vector<Shm> sh(1);
    for (long long r = 0; r < R; ++r) init_restart(a, (int)r, sh[0]);
}

void emu_step(long long R, int n, int m, int maxls, long long maxiter, long long maxfun, double factr,
              double pgtol, double* X, const double* value, double sign, const double* grad, const int* status,
              int ignore_status, char* ws, int* summary) {
    StepArgs a;
    a.L = make_layout(R, n, m);
    a.R = R;
    a.n = n;
    a.m = m;
    a.maxls = maxls;
    a.maxiter = maxiter;
    a.maxfun = maxfun;
    a.factr = factr;
    a.pgtol = pgtol;
    a.ws = ws;
    a.X = X;
    a.value = value;
    a.sign = sign;
    a.grad = grad;
    a.status = status;
    a.ignore_status = ignore_status;
    const int n2 = sort_len(n);
    std::vector<double> dyn((step_dyn_bytes(n2) + 7) / 8);
    std::vector<Shm> sh(1);
    for (long long r = 0; r < R; ++r)
        step_restart(a, (int)r, sh[0], reinterpret_cast<unsigned char*>(dyn.data()), n2);
    if (summary) summarize(a.L, ws, R, sh[0], summary);
}

void emu_results(long long R, int n, int m, const char* ws, double* f, long long* nit, long long* nfev, int* code) {
    const Layout L = make_layout(R, n, m);
    const State* st = reinterpret_cast<const State*>(ws + L.states);
    for (long long r = 0; r < R; ++r) {
        f[r] = st[r].f;
        nit[r] = st[r].nit;
        nfev[r] = st[r].nfev;
        code[r] = st[r].code;
    }
}

}  // extern "C"

/* ORACLE (test infrastructure; also the CPU baseline of the fused log-areas
 * benchmark): plain-C restatement of the reference's fused qLogEHVI kernel,
 * botorch/csrc/logei_fused.cpp:
 *   safe_softplus / safe_sigmoid / cauchy            logei_fused.cpp:38-66
 *   Pareto value and derivative                      logei_fused.cpp:68-82
 *   log_fatplus forward, forward + backward          logei_fused.cpp:84-111
 *   compute_fatmin (with gradient weights)           logei_fused.cpp:113-172
 *   fused_log_areas_forward                          logei_fused.cpp:184-264
 *   fused_log_areas_backward                         logei_fused.cpp:266-374
 * Same loops, branches and summation order; the parallel loop of the
 * reference (at::parallel_for over B * n_sub) is the [lo, hi) range of each
 * call, so that a caller can split the range over threads. Only tests and the
 * benchmark's CPU baseline use it. Built by oracle/build.py. */
#include <math.h>
#include <stdint.h>

#define LA_MAX_I 32
#define LA_MAX_M 8

#define LA_DEFINE(T, SUF, EXP, LOG, LOG1P, CLAMP)                                              \
    static T softplus_##SUF(T y) {                                                             \
        if (y > (T)20) return y;                                                               \
        if (y < (T)-20) return EXP(y);                                                         \
        return LOG1P(EXP(y));                                                                  \
    }                                                                                          \
    static T sigmoid_##SUF(T y) {                                                              \
        if (y >= (T)0) {                                                                       \
            T e = EXP(-y);                                                                     \
            return (T)1 / ((T)1 + e);                                                          \
        }                                                                                      \
        T e = EXP(y);                                                                          \
        return e / ((T)1 + e);                                                                 \
    }                                                                                          \
    static T cauchy_##SUF(T y) { return (T)1 / ((T)1 + y * y); }                               \
    static void pareto_vd_##SUF(T z, T* val, T* deriv) {                                       \
        T d = (T)2 + (T)2 * z + z * z;                                                         \
        *val = (T)2 / d;                                                                       \
        *deriv = (T)-2 * ((T)2 + (T)2 * z) / (d * d);                                          \
    }                                                                                          \
    static T pareto_v_##SUF(T z) {                                                             \
        T d = (T)2 + (T)2 * z + z * z;                                                         \
        return (T)2 / d;                                                                       \
    }                                                                                          \
    static T log_fatplus_##SUF(T x, T tau, T inv_tau) {                                        \
        T y = x * inv_tau;                                                                     \
        T f = softplus_##SUF(y) + (T)0.1 * cauchy_##SUF(y);                                    \
        T val = tau * f;                                                                       \
        return val > (T)0 ? LOG(val) : (T)-1e30;                                               \
    }                                                                                          \
    static void log_fatplus_vg_##SUF(T x, T tau, T inv_tau, T* val, T* grad) {                 \
        T y = x * inv_tau;                                                                     \
        T cy = cauchy_##SUF(y);                                                                \
        T sp = softplus_##SUF(y);                                                              \
        T f = sp + (T)0.1 * cy;                                                                \
        T tf = tau * f;                                                                        \
        if (tf <= (T)0) {                                                                      \
            *val = (T)-1e30;                                                                   \
            *grad = (T)0;                                                                      \
            return;                                                                            \
        }                                                                                      \
        *val = LOG(tf);                                                                        \
        T sg = sigmoid_##SUF(y);                                                               \
        T fp = sg - (T)2 * (T)0.1 * y * cy * cy;                                               \
        *grad = fp / (tau * f);                                                                \
    }                                                                                          \
    static T fatmin_##SUF(const T* x, int n, T tau, T inv_tau, T* gw) {                        \
        if (n == 1) {                                                                          \
            if (gw) gw[0] = (T)1;                                                              \
            return x[0];                                                                       \
        }                                                                                      \
        T mn = x[0];                                                                           \
        int ami = 0;                                                                           \
        for (int j = 1; j < n; j++)                                                            \
            if (x[j] < mn) {                                                                   \
                mn = x[j];                                                                     \
                ami = j;                                                                       \
            }                                                                                  \
        if (mn < (T)-1e29) {                                                                   \
            if (gw)                                                                            \
                for (int j = 0; j < n; j++) gw[j] = (j == ami) ? (T)1 : (T)0;                  \
            return mn;                                                                         \
        }                                                                                      \
        T S = 0, S_pd = 0, pd[LA_MAX_I];                                                       \
        for (int j = 0; j < n; j++) {                                                          \
            T zj = (x[j] - mn) * inv_tau;                                                      \
            if (gw) {                                                                          \
                T pv, pder;                                                                    \
                pareto_vd_##SUF(zj, &pv, &pder);                                               \
                S += pv;                                                                       \
                pd[j] = pder;                                                                  \
                S_pd += pder;                                                                  \
            } else {                                                                           \
                S += pareto_v_##SUF(zj);                                                       \
            }                                                                                  \
        }                                                                                      \
        T result = mn - tau * LOG(S);                                                          \
        if (gw)                                                                                \
            for (int j = 0; j < n; j++)                                                        \
                gw[j] = (j == ami) ? (T)1 + (S_pd - (T)-1) / S : -pd[j] / S;                   \
        return result;                                                                         \
    }                                                                                          \
    static T lcl_##SUF(T lo, T up) { return LOG(((CLAMP) < up ? (CLAMP) : up) - lo); }          \
    void oracle_log_areas_forward_##SUF(const T* obj, int64_t B, int64_t n_sub, int64_t isz,   \
                                        int64_t m, const T* cl, const T* cu, int64_t B_cells,  \
                                        int64_t nc, double tau_relu, double tau_max, T* out,   \
                                        int64_t lo, int64_t hi) {                              \
        const T tr = (T)tau_relu, tm = (T)tau_max;                                             \
        const T inv_tr = (T)1 / tr, inv_tm = (T)1 / tm;                                        \
        (void)B;                                                                               \
        for (int64_t idx = lo; idx < hi; idx++) {                                              \
            const int64_t b = idx / n_sub, s = idx % n_sub;                                    \
            const int64_t bc = B_cells == 1 ? 0 : b;                                           \
            for (int64_t c = 0; c < nc; c++) {                                                 \
                T li[LA_MAX_M][LA_MAX_I];                                                      \
                for (int j = 0; j < isz; j++)                                                  \
                    for (int k = 0; k < m; k++)                                                \
                        li[k][j] = log_fatplus_##SUF(                                          \
                            obj[((b * n_sub + s) * isz + j) * m + k] - cl[(bc * nc + c) * m + k], \
                            tr, inv_tr);                                                       \
                T area = 0;                                                                    \
                for (int k = 0; k < m; k++) {                                                  \
                    T lim = fatmin_##SUF(li[k], (int)isz, tm, inv_tm, 0);                      \
                    T pair[2] = {lim, lcl_##SUF(cl[(bc * nc + c) * m + k],                     \
                                                cu[(bc * nc + c) * m + k])};                   \
                    area += fatmin_##SUF(pair, 2, tm, inv_tm, 0);                              \
                }                                                                              \
                out[(b * nc + c) * n_sub + s] = area;                                          \
            }                                                                                  \
        }                                                                                      \
    }                                                                                          \
    void oracle_log_areas_backward_##SUF(const T* go, const T* obj, int64_t B, int64_t n_sub,  \
                                         int64_t isz, int64_t m, const T* cl, const T* cu,     \
                                         int64_t B_cells, int64_t nc, double tau_relu,         \
                                         double tau_max, T* g_obj, int64_t lo, int64_t hi) {   \
        const T tr = (T)tau_relu, tm = (T)tau_max;                                             \
        const T inv_tr = (T)1 / tr, inv_tm = (T)1 / tm;                                        \
        (void)B;                                                                               \
        for (int64_t idx = lo; idx < hi; idx++) {                                              \
            const int64_t b = idx / n_sub, s = idx % n_sub;                                    \
            const int64_t bc = B_cells == 1 ? 0 : b;                                           \
            T g_buf[LA_MAX_I][LA_MAX_M];                                                       \
            for (int j = 0; j < LA_MAX_I; j++)                                                 \
                for (int k = 0; k < LA_MAX_M; k++) g_buf[j][k] = 0;                            \
            for (int64_t c = 0; c < nc; c++) {                                                 \
                const T g_out = go[(b * nc + c) * n_sub + s];                                  \
                T li[LA_MAX_M][LA_MAX_I], lg[LA_MAX_M][LA_MAX_I];                              \
                for (int j = 0; j < isz; j++)                                                  \
                    for (int k = 0; k < m; k++)                                                \
                        log_fatplus_vg_##SUF(                                                  \
                            obj[((b * n_sub + s) * isz + j) * m + k] - cl[(bc * nc + c) * m + k], \
                            tr, inv_tr, &li[k][j], &lg[k][j]);                                 \
                for (int k = 0; k < m; k++) {                                                  \
                    T fmg[LA_MAX_I], fm2g[2];                                                  \
                    T lim = fatmin_##SUF(li[k], (int)isz, tm, inv_tm, fmg);                    \
                    T pair[2] = {lim, lcl_##SUF(cl[(bc * nc + c) * m + k],                     \
                                                cu[(bc * nc + c) * m + k])};                   \
                    fatmin_##SUF(pair, 2, tm, inv_tm, fm2g);                                   \
                    T g_lim = g_out * fm2g[0];                                                 \
                    for (int j = 0; j < isz; j++) g_buf[j][k] += g_lim * fmg[j] * lg[k][j];    \
                }                                                                              \
            }                                                                                  \
            for (int j = 0; j < isz; j++)                                                      \
                for (int k = 0; k < m; k++) g_obj[((b * n_sub + s) * isz + j) * m + k] = g_buf[j][k]; \
        }                                                                                      \
    }

LA_DEFINE(double, f64, exp, log, log1p, 1e10)
LA_DEFINE(float, f32, expf, logf, log1pf, 1e8f)

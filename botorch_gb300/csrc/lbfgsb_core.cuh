// Batched L-BFGS-B: one restart's optimiser, advanced by one CTA.
//
// The per-restart optimiser of the reference's batched driver
// (botorch/optim/batched_lbfgs_b.py:169-636, which steps scipy's L-BFGS-B
// routine once per restart and round, botorch/generation/gen.py:226-247)
// restated as a state machine that a CTA advances on the device: consume the
// objective value and gradient the restart asked for, run the algorithm until it
// next needs them (or stops), and write the point to evaluate.
//
// The algorithm is L-BFGS-B 3.0 as published: Byrd, Lu, Nocedal and Zhu, "A
// limited memory algorithm for bound constrained optimization" (SIAM J. Sci.
// Comput. 16, 1995): the compact form B = theta I - W M W^T with W = [Y, theta S],
// the generalized Cauchy point by a walk over the sorted breakpoints of the
// projected steepest-descent path, and the subspace minimisation by the direct
// primal method; Zhu, Byrd, Lu and Nocedal, "Algorithm 778" (ACM TOMS 23, 1997):
// the driver logic (memory refresh after a singular factor or a failed line
// search, the skipped update when s^T y <= eps * (-g^T s), the stopping tests
// on the projected gradient and on the relative reduction of f); Morales and
// Nocedal, "Remark on Algorithm 778" (ACM TOMS 38, 2011): the subspace step is
// first projected onto the box and kept when it is a descent direction, else
// backtracked to the box; and the line search of More and Thuente, "Line search
// algorithms with guaranteed sufficient decrease" (ACM TOMS 20, 1994), with
// ftol = 1e-3, gtol = 0.9, xtol = 0.1 and the step bounded by the box.
//
// Arithmetic differs from scipy's compiled routine only in summation order and
// rounding: the O(m n) dot products are CTA reductions, the small factors are
// applied with reciprocal pivots, and the Gram blocks of the subspace matrix
// are formed from their definition (rather than updated by the variables that
// changed sides) after a memory refresh or when more than an eighth of the
// variables changed sides. Ties between equal breakpoints are taken in index
// order.
//
// The same source compiles for the host with LB_HOST_EMU (one thread, all
// barriers no-ops): the host build exists only so that tests can step it in
// lock-step with scipy's routine on the CPU.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(LB_HOST_EMU)
#define LB_FN static inline
#define LB_SYNC() ((void)0)
#define LB_SYNCWARP() ((void)0)
#define LB_NT 1
#define LB_NW 1
#define LB_WARP 1
#define LB_HD inline
#else
#define LB_FN __device__ __forceinline__
#define LB_SYNC() __syncthreads()
#define LB_SYNCWARP() __syncwarp()
#define LB_NT 256
#define LB_NW 8
#define LB_WARP 32
#define LB_HD __host__ __device__ inline
#endif

namespace bgb_lb {

constexpr int kMaxM = 20;      // largest history (scipy's default maxcor is 10)
constexpr int kMaxN = 8192;    // largest number of variables per restart
constexpr double kEpsMch = 2.220446049250313e-16;
constexpr double kBig = 1e10;
constexpr double kFtol = 1e-3, kGtol = 0.9, kXtol = 0.1;

// What a restart waits for.
enum : int { kStopped = 0, kWaitFgStart = 1, kWaitFgLn = 2 };
// Line-search task.
enum : int { kLsStart = 0, kLsFg = 1, kLsConv = 2, kLsWarn = 3, kLsError = 4 };
// Control labels of the state machine.
enum : int { kLIter = 0, kLNewX = 1, kLExit = 2 };

// Stop codes (mirror the include file's BGB_LBFGSB_*).
enum : int {
    kRunning = 0,
    kConvPgtol = 1,
    kConvFtol = 2,
    kAbnormal = 3,
    kMaxIter = 4,
    kMaxFun = 5,
    kNonFinite = 6,
};

// Per-restart scalars; kept in the workspace between launches.
struct State {
    double f, fold, gd, gdold, stp, stpmx, dnorm, dtd, theta, sbgnrm;
    double ls_finit, ls_ginit, ls_gtest, ls_fx, ls_gx, ls_fy, ls_gy;
    double ls_stx, ls_sty, ls_stmin, ls_stmax, ls_width, ls_width1;
    int ls_brackt, ls_stage, ls_task;
    int col, head, itail, iupdat, updatd, iter, ifun, iback, nfgv, nfree, nskip, info, wrk;
    int wait, code, held, wn1_valid;  // wn1_valid: the Gram blocks of the subspace matrix are current
    long long nit, nfev;
};

// Problem-wide inputs (identical for every restart).
struct Problem {
    int n, m, maxls, boxed, cnstnd;
    long long maxiter, maxfun;
    double factr, pgtol;
    const double* lo;
    const double* hi;
    const int8_t* nbd;  // 0 unbounded, 1 lower only, 2 both, 3 upper only
};

// One restart's arrays.
struct Arrays {
    double* x;     // the point (the row evaluated by the caller)
    double* g;     // gradient at x
    double* xold;  // point at the start of the line search
    double* gold;  // gradient there; y = g - gold after the search
    double* z;     // Cauchy point, then the subspace minimiser
    double* d;     // Cauchy direction, then the search direction
    double* r;     // reduced gradient, then the Newton direction (free entries)
    double* xp;    // subspace point before projection
    double* ws;    // S, n x m column-major, circular in the column
    double* wy;    // Y, likewise
    double* sy;    // S^T Y (m x m, column-major), logical order oldest first
    double* ss;    // S^T S
    double* wt;    // Cholesky factor of theta S^T S + L D^-1 L^T (upper)
    double* wn;    // factor of the subspace middle matrix (2m x 2m, upper)
    double* wn1;   // its Gram blocks (2m x 2m, lower): Y^T Z Z^T Y, S^T A A^T S, S^T Y split
    int8_t* iwhere;
    int8_t* wasfree;
};

// CTA-shared scratch. The small matrices are loaded here for a launch.
struct Shm {
    State s;
    double sy[kMaxM * kMaxM], ss[kMaxM * kMaxM], wt[kMaxM * kMaxM];
    double wn[4 * kMaxM * kMaxM];
    double wn1[4 * kMaxM * kMaxM];
    double p[2 * kMaxM], c[2 * kMaxM], v[2 * kMaxM], wbp[2 * kMaxM], wv[2 * kMaxM];
    double dots[kMaxM * (2 * kMaxM + 1)];
    double rd[2 * kMaxM], dinv[kMaxM], rsq[kMaxM], rwt[kMaxM];
    int red_i2[LB_NW];
    int nenter, nleave;
    double red_d[LB_NW];
    int red_i[LB_NW];
    double f1, f2, f2_org, dtm, tsum, dr;
    int need_walk, to999, info, label, trial;
};

struct Ctx {
    Problem P;
    Arrays A;
    Shm* sh;
    double* key;  // breakpoint sort scratch (n2 entries)
    int* idx;
    int n2;
    double* tile;   // row tiles of S and Y for the Gram sums (kTileRows + 1) x kTileCols
    int8_t* tmask;  // free flags of the tile's rows
    int* elist;     // variables that entered / left the free set (free_set -> form_k)
    int* llist;
};

constexpr int kTileRows = 64;
constexpr int kTileCols = 2 * kMaxM;
// Dynamic shared memory of the step launch: breakpoint sort scratch, then the tile.


// ---------------------------------------------------------------------------
// Thread-level helpers.

#if defined(LB_HOST_EMU)
LB_FN int lb_tid() { return 0; }
LB_FN double warp_sum(double v) { return v; }
LB_FN int warp_sum_i(int v) { return v; }
LB_FN double warp_max(double v) { return v; }
LB_FN void warp_argmin(double&, int&) {}
LB_FN double group_sum(double v, int) { return v; }
#else
LB_FN int lb_tid() { return threadIdx.x; }
LB_FN double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
LB_FN int warp_sum_i(int v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
LB_FN double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
// Sum over aligned groups of g lanes (g a power of two <= 32); every lane of the
// warp calls it.
LB_FN double group_sum(double v, int g) {
    for (int o = g / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
LB_FN void warp_argmin(double& v, int& i) {
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_xor_sync(0xffffffffu, v, o);
        int j = __shfl_xor_sync(0xffffffffu, i, o);
        if (w < v || (w == v && j < i)) {
            v = w;
            i = j;
        }
    }
}
#endif

LB_FN int lane_of(int t) { return t & 31; }
LB_FN int warp_of(int t) { return t >> 5; }

// Sum over the CTA; every thread gets the same value (fixed order).
LB_FN double block_sum(Shm& sh, double v) {
    const int t = lb_tid();
    v = warp_sum(v);
    if (lane_of(t) == 0) sh.red_d[warp_of(t)] = v;
    LB_SYNC();
    double s = 0.0;
    for (int w = 0; w < LB_NW; ++w) s += sh.red_d[w];
    LB_SYNC();
    return s;
}

LB_FN int block_sum_i(Shm& sh, int v) {
    const int t = lb_tid();
    v = warp_sum_i(v);
    if (lane_of(t) == 0) sh.red_i[warp_of(t)] = v;
    LB_SYNC();
    int s = 0;
    for (int w = 0; w < LB_NW; ++w) s += sh.red_i[w];
    LB_SYNC();
    return s;
}

LB_FN double block_max(Shm& sh, double v) {
    const int t = lb_tid();
    v = warp_max(v);
    if (lane_of(t) == 0) sh.red_d[warp_of(t)] = v;
    LB_SYNC();
    double s = sh.red_d[0];
    for (int w = 1; w < LB_NW; ++w) s = sh.red_d[w] > s ? sh.red_d[w] : s;
    LB_SYNC();
    return s;
}

// Lexicographic minimum of (v, i) over the CTA.
LB_FN void block_argmin(Shm& sh, double& v, int& i) {
    const int t = lb_tid();
    warp_argmin(v, i);
    if (lane_of(t) == 0) {
        sh.red_d[warp_of(t)] = v;
        sh.red_i[warp_of(t)] = i;
    }
    LB_SYNC();
    v = sh.red_d[0];
    i = sh.red_i[0];
    for (int w = 1; w < LB_NW; ++w) {
        if (sh.red_d[w] < v || (sh.red_d[w] == v && sh.red_i[w] < i)) {
            v = sh.red_d[w];
            i = sh.red_i[w];
        }
    }
    LB_SYNC();
}

constexpr int kLaneStride = LB_NT >= 32 ? 32 : 1;

// out[j] = sum_k a_j[k] b_j[k] for j < J, one warp per output with the lanes
// over k. setup(j, a, b, mode) names the two columns; mode 0 sums over every
// k, 1 over the free variables (iwhere <= 0), 2 over the active ones.
template <class Setup>
LB_FN void warp_dots(int J, int n, const int8_t* iwhere, Setup setup, double* out) {
    const int t = lb_tid();
    for (int j = warp_of(t); j < J; j += LB_NW) {
        const double* a;
        const double* b;
        int mode;
        setup(j, a, b, mode);
        double acc = 0.0;
        if (mode == 0) {
            for (int k = lane_of(t); k < n; k += kLaneStride) acc += a[k] * b[k];
        } else {
            const bool want_free = mode == 1;
            for (int k = lane_of(t); k < n; k += kLaneStride)
                if ((iwhere[k] <= 0) == want_free) acc += a[k] * b[k];
        }
        acc = warp_sum(acc);
        if (lane_of(t) == 0) out[j] = acc;
    }
    LB_SYNC();
}

// out[o] = sum_k a_o[k] b_o[k] over the free (mode 1) or active (mode 2) k, for
// o < J, where a_o and b_o are among ncols <= kTileCols columns (column c at
// col(c)) staged tile by tile in shared memory, so that each column is read
// from memory once per 4 * LB_NT outputs: pair(o, ia, ib, mode) names them.
// With few outputs (the newest pair's products) g consecutive lanes share one,
// each summing every g-th row of a tile, and their sums are added at the end:
// the chain of dependent float64 adds per thread is n / g long instead of n.
template <class Col, class Pair>
LB_FN void tiled_gram(int J, int n, int ncols, Col col, const int8_t* iwhere, Pair pair, double* tile,
                      int8_t* tmask, double* out) {
    const int t = lb_tid();
    constexpr int ld = kTileRows + 1;  // (odd stride: the columns start in different banks)
    int g = 1;
    while (g < LB_WARP && 2 * J * g <= LB_NT) g *= 2;
    const int sub = t % g, tg = t / g, ng = LB_NT / g;
    for (int o0 = 0; o0 < J; o0 += 4 * ng) {
        int ia[4], ib[4], md[4];
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int q = 0; q < 4; ++q) {
            const int o = o0 + tg + q * ng;
            ia[q] = ib[q] = md[q] = -1;
            if (o < J) pair(o, ia[q], ib[q], md[q]);
        }
        for (int k0 = 0; k0 < n; k0 += kTileRows) {
            const int rows = n - k0 < kTileRows ? n - k0 : kTileRows;
            for (int e = t; e < ncols * kTileRows; e += LB_NT) {
                const int c = e / kTileRows, r = e - c * kTileRows;
                tile[c * ld + r] = r < rows ? col(c)[k0 + r] : 0.0;
            }
            for (int r = t; r < kTileRows; r += LB_NT) tmask[r] = (r < rows && iwhere[k0 + r] <= 0) ? 1 : 0;
            LB_SYNC();
            for (int q = 0; q < 4; ++q) {
                if (ia[q] < 0) continue;
                const double* a = tile + ia[q] * ld;
                const double* b = tile + ib[q] * ld;
                const int8_t want = md[q] == 1 ? 1 : 0;
                double sum = 0.0;
                for (int r = sub; r < rows; r += g)
                    if (tmask[r] == want) sum += a[r] * b[r];
                acc[q] += sum;
            }
            LB_SYNC();
        }
        for (int q = 0; q < 4; ++q) {
            acc[q] = group_sum(acc[q], g);  // (every lane: g divides the warp)
            if (sub == 0 && ia[q] >= 0) out[o0 + tg + q * ng] = acc[q];
        }
    }
    LB_SYNC();
}

// Column of S or Y holding logical pair j (0 = oldest).
LB_FN int colptr(const State& s, int m, int j) { return (s.head + j) % m; }

// ---------------------------------------------------------------------------
// Small dense kernels, run by the first warp of the CTA (all its lanes call
// them; results are in shared memory after the call). Column-major, leading
// dimension ld; n <= 2 * kMaxM.

LB_FN int lane_id() { return lb_tid() & (LB_WARP - 1); }

// sum_i a[i] b[i] over i < n, every lane gets it.
LB_FN double warp_dot(const double* a, const double* b, int n) {
    double acc = 0.0;
    for (int i = lane_id(); i < n; i += LB_WARP) acc += a[i] * b[i];
    return warp_sum(acc);
}

// Upper Cholesky factor R (A = R^T R) in place, right-looking; rdiag = 1 / diag(R).
// Returns 0 or the 1-based column whose pivot is not positive.
LB_FN int warp_chol_upper(double* a, int ld, int n, double* rdiag) {
    const int l = lane_id();
    for (int k = 0; k < n; ++k) {
        const double akk = a[k + k * ld];
        if (!(akk > 0.0)) return k + 1;
        const double rkk = sqrt(akk);
        const double inv = 1.0 / rkk;
        for (int j = k + 1 + l; j < n; j += LB_WARP) a[k + j * ld] *= inv;
        LB_SYNCWARP();
        if (l == 0) {
            a[k + k * ld] = rkk;
            rdiag[k] = inv;
        }
        for (int j = k + 1 + l; j < n; j += LB_WARP) {
            const double rkj = a[k + j * ld];
            for (int i = k + 1; i <= j; ++i) a[i + j * ld] -= a[k + i * ld] * rkj;
        }
        LB_SYNCWARP();
    }
    return 0;
}

// rdiag = 1 / diag(T); 0, or the 1-based index of a zero diagonal entry.
LB_FN int warp_rdiag(const double* t, int ld, int n, double* rdiag) {
    for (int i = lane_id(); i < n; i += LB_WARP) rdiag[i] = 1.0 / t[i + i * ld];
    LB_SYNCWARP();
    for (int i = 0; i < n; ++i)
        if (t[i + i * ld] == 0.0) return i + 1;
    return 0;
}

// Solve T^T x = b in place, T upper triangular.
LB_FN void warp_solve_upper_t(const double* t, int ld, int n, const double* rdiag, double* b) {
    const int l = lane_id();
    for (int j = 0; j < n; ++j) {
        const double xj = b[j] * rdiag[j];
        LB_SYNCWARP();
        if (l == 0) b[j] = xj;
        for (int i = j + 1 + l; i < n; i += LB_WARP) b[i] -= t[j + i * ld] * xj;
        LB_SYNCWARP();
    }
}

// Solve T x = b in place, T upper triangular.
LB_FN void warp_solve_upper(const double* t, int ld, int n, const double* rdiag, double* b) {
    const int l = lane_id();
    for (int j = n - 1; j >= 0; --j) {
        const double xj = b[j] * rdiag[j];
        LB_SYNCWARP();
        if (l == 0) b[j] = xj;
        for (int i = l; i < j; i += LB_WARP) b[i] -= t[i + j * ld] * xj;
        LB_SYNCWARP();
    }
}

// Solve T^T X = B for nrhs columns (column c at B + c * ldb), one lane per column.
LB_FN void warp_solve_upper_t_multi(const double* t, int ld, int n, const double* rdiag, double* B, int ldb,
                                    int nrhs) {
    for (int c = lane_id(); c < nrhs; c += LB_WARP) {
        double* b = B + c * ldb;
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            for (int i = 0; i < j; ++i) acc += t[i + j * ld] * b[i];
            b[j] = (b[j] - acc) * rdiag[j];
        }
    }
    LB_SYNCWARP();
}

// p = M v for the 2col x 2col middle matrix M of the compact form, through the
// factor of T = theta S^T S + L D^-1 L^T (Byrd et al. 1995, section 3); p and v distinct.
LB_FN int middle_times(Shm& sh, int m, int col, const double* v, double* p) {
    if (col == 0) return 0;
    const int l = lane_id();
    const double* sy = sh.sy;
    for (int i = l; i < col; i += LB_WARP) {
        const double di = sy[i + i * m];
        sh.dinv[i] = 1.0 / di;
        sh.rsq[i] = 1.0 / sqrt(di);
    }
    const int info = warp_rdiag(sh.wt, m, col, sh.rwt);
    if (info) return info;
    for (int i = l; i < col; i += LB_WARP) {
        double acc = 0.0;
        for (int k = 0; k < i; ++k) acc += sy[i + k * m] * v[k] * sh.dinv[k];
        p[col + i] = v[col + i] + acc;
        p[i] = v[i] * sh.rsq[i];
    }
    LB_SYNCWARP();
    warp_solve_upper_t(sh.wt, m, col, sh.rwt, p + col);
    warp_solve_upper(sh.wt, m, col, sh.rwt, p + col);
    for (int i = l; i < col; i += LB_WARP) {
        double acc = 0.0;
        for (int k = i + 1; k < col; ++k) acc += sy[k + i * m] * p[col + k];
        p[i] = -p[i] * sh.rsq[i] + acc * sh.dinv[i];
    }
    LB_SYNCWARP();
    return 0;
}

// ---------------------------------------------------------------------------
// CTA-wide steps.

// Infinity norm of the projected gradient.
LB_FN double proj_grad_norm(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    double v = 0.0;
    for (int k = lb_tid(); k < P.n; k += LB_NT) {
        double gi = A.g[k];
        const int nb = P.nbd[k];
        if (nb != 0) {
            if (gi < 0.0) {
                if (nb >= 2) gi = fmax(A.x[k] - P.hi[k], gi);
            } else {
                if (nb <= 2) gi = fmin(A.x[k] - P.lo[k], gi);
            }
        }
        gi = fabs(gi);
        v = gi > v ? gi : v;
    }
    return block_max(*c.sh, v);
}

LB_FN void reset_memory(State& s) {
    s.wn1_valid = 0;
    s.info = 0;
    s.col = 0;
    s.head = 0;
    s.theta = 1.0;
    s.iupdat = 0;
    s.updatd = 0;
}

// Bitonic sort of (key, idx) pairs, ascending and lexicographic, n2 a power of two.
LB_FN void sort_breakpoints(Ctx& c) {
    const int n2 = c.n2;
    double* key = c.key;
    int* idx = c.idx;
    for (int size = 2; size <= n2; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = lb_tid(); i < (n2 >> 1); i += LB_NT) {
                const int lo = 2 * stride * (i / stride) + (i % stride);
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const double a = key[lo], b = key[hi];
                const int ia = idx[lo], ib = idx[hi];
                const bool gt = a > b || (a == b && ia > ib);
                if (gt == up) {
                    key[lo] = b;
                    key[hi] = a;
                    idx[lo] = ib;
                    idx[hi] = ia;
                }
            }
            LB_SYNC();
        }
    }
}

// Generalized Cauchy point z along the projected steepest-descent path; on
// return sh.c = W^T (z - x). Returns nonzero when a triangular factor is singular.
LB_FN int cauchy(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    State& s = sh.s;
    const int n = P.n, m = P.m, col = s.col, col2 = 2 * s.col;
    const double theta = s.theta;
    const int t = lb_tid();
    const double inf = (double)INFINITY;
    if (s.sbgnrm <= 0.0) {
        for (int k = t; k < n; k += LB_NT) A.z[k] = A.x[k];
        if (t == 0)
            for (int j = 0; j < col2; ++j) sh.c[j] = 0.0;
        LB_SYNC();
        return 0;
    }
    double f1p = 0.0, bk = inf;
    int nbrk = 0, nfd = 0, unb = 0, bki = 0x7fffffff;
    for (int k = t; k < c.n2; k += LB_NT) {
        if (k >= n) {
            c.key[k] = inf;
            c.idx[k] = k;
            continue;
        }
        const double neggi = -A.g[k];
        const int nb = P.nbd[k];
        int iw = A.iwhere[k];
        double tl = 0.0, tu = 0.0;
        if (iw != 3 && iw != -1) {
            if (nb <= 2) tl = A.x[k] - P.lo[k];
            if (nb >= 2) tu = P.hi[k] - A.x[k];
            const bool xlower = nb <= 2 && tl <= 0.0;
            const bool xupper = nb >= 2 && tu <= 0.0;
            iw = 0;
            if (xlower) {
                if (neggi <= 0.0) iw = 1;
            } else if (xupper) {
                if (neggi >= 0.0) iw = 2;
            } else {
                if (fabs(neggi) <= 0.0) iw = -3;
            }
            A.iwhere[k] = (int8_t)iw;
        }
        double kk = inf;
        if (iw != 0 && iw != -1) {
            A.d[k] = 0.0;
        } else {
            A.d[k] = neggi;
            f1p -= neggi * neggi;
            if (nb <= 2 && nb != 0 && neggi < 0.0) {
                kk = tl / (-neggi);
                ++nbrk;
            } else if (nb >= 2 && neggi > 0.0) {
                kk = tu / neggi;
                ++nbrk;
            } else {
                ++nfd;
                if (fabs(neggi) > 0.0) ++unb;
            }
        }
        c.key[k] = kk;
        c.idx[k] = k;
        if (kk < bk) {
            bk = kk;
            bki = k;
        }
        A.z[k] = A.x[k];
    }
    const double f1 = block_sum(sh, f1p);
    const int nbreak = block_sum_i(sh, nbrk);
    const int nfree_dec = block_sum_i(sh, nfd);
    const int unbnded = block_sum_i(sh, unb);
    block_argmin(sh, bk, bki);
    if (nbreak == 0 && nfree_dec == 0) {  // d = 0: x is the Cauchy point
        if (t == 0)
            for (int j = 0; j < col2; ++j) sh.c[j] = 0.0;
        LB_SYNC();
        return 0;
    }
    // p = W^T d
    warp_dots(col2, n, A.iwhere,
              [&](int j, const double*& a, const double*& b, int& mode) {
                  const size_t pj = (size_t)colptr(s, m, j < col ? j : j - col) * n;
                  a = (j < col ? A.wy : A.ws) + pj;
                  b = A.d;
                  mode = 0;
              },
              sh.p);
    if (t < LB_WARP) {
        for (int j = lane_id(); j < col; j += LB_WARP) sh.p[col + j] *= theta;
        for (int j = lane_id(); j < col2; j += LB_WARP) sh.c[j] = 0.0;
        LB_SYNCWARP();
        double f2 = -theta * f1;
        const double f2_org = f2;
        int info = 0;
        if (col > 0) {
            info = middle_times(sh, m, col, sh.p, sh.v);
            if (!info) f2 -= warp_dot(sh.v, sh.p, col2);
        }
        if (t == 0) {
            sh.f2_org = f2_org;
            sh.info = info;
            sh.f1 = f1;
            sh.f2 = f2;
            sh.dtm = -f1 / f2;
            sh.tsum = 0.0;
            sh.need_walk = (nbreak > 0 && !(-f1 / f2 < bk)) ? 1 : 0;
            sh.to999 = 0;
        }
    }
    LB_SYNC();
    if (sh.info) return sh.info;
    if (sh.need_walk) {
        sort_breakpoints(c);
        if (t < LB_WARP) {
            const int l = lane_id();
            const bool bnded = unbnded == 0;
            int nleft = nbreak, it = 0, info = 0, to999 = 0;
            double tj = 0.0, f1w = sh.f1, f2w = sh.f2, dtm = sh.dtm, tsum = 0.0;
            const double f2_org = sh.f2_org;
            while (true) {
                const double tj0 = tj;
                tj = c.key[it];
                const int ibp = c.idx[it];
                const double dt = tj - tj0;
                if (dtm < dt || ibp >= n) break;  // (an overflowed breakpoint sorts among the padding)
                tsum += dt;
                --nleft;
                ++it;
                const double dibp = A.d[ibp];
                const double zibp = (dibp > 0.0 ? P.hi[ibp] : P.lo[ibp]) - A.x[ibp];
                LB_SYNCWARP();
                if (l == 0) {
                    A.d[ibp] = 0.0;
                    A.z[ibp] = dibp > 0.0 ? P.hi[ibp] : P.lo[ibp];
                    A.iwhere[ibp] = dibp > 0.0 ? 2 : 1;
                }
                if (nleft == 0 && nbreak == n) {
                    dtm = dt;
                    to999 = 1;
                    break;
                }
                const double dibp2 = dibp * dibp;
                f1w = f1w + dt * f2w + dibp2 - theta * dibp * zibp;
                f2w = f2w - theta * dibp2;
                if (col > 0) {
                    for (int j = l; j < col2; j += LB_WARP) {
                        sh.c[j] += dt * sh.p[j];
                        const size_t pj = (size_t)colptr(s, m, j < col ? j : j - col) * n;
                        sh.wbp[j] = j < col ? A.wy[pj + ibp] : theta * A.ws[pj + ibp];
                    }
                    LB_SYNCWARP();
                    info = middle_times(sh, m, col, sh.wbp, sh.v);
                    if (info) break;
                    const double wmc = warp_dot(sh.c, sh.v, col2);
                    const double wmp = warp_dot(sh.p, sh.v, col2);
                    const double wmw = warp_dot(sh.wbp, sh.v, col2);
                    for (int j = l; j < col2; j += LB_WARP) sh.p[j] -= dibp * sh.wbp[j];
                    LB_SYNCWARP();
                    f1w += dibp * wmc;
                    f2w += 2.0 * dibp * wmp - dibp2 * wmw;
                }
                f2w = fmax(kEpsMch * f2_org, f2w);
                if (nleft > 0) {
                    dtm = -f1w / f2w;
                    continue;
                } else if (bnded) {
                    f1w = 0.0;
                    f2w = 0.0;
                    dtm = 0.0;
                } else {
                    dtm = -f1w / f2w;
                }
                break;
            }
            if (l == 0) {
                sh.info = info;
                sh.dtm = dtm;
                sh.tsum = tsum;
                sh.to999 = to999;
            }
        }
        LB_SYNC();
        if (sh.info) return sh.info;
    }
    if (t == 0 && !sh.to999) {
        if (sh.dtm <= 0.0) sh.dtm = 0.0;
        sh.tsum += sh.dtm;
    }
    LB_SYNC();
    if (!sh.to999) {
        const double tsum = sh.tsum;
        for (int k = t; k < n; k += LB_NT) A.z[k] += tsum * A.d[k];
    }
    if (t == 0 && col > 0)
        for (int j = 0; j < col2; ++j) sh.c[j] += sh.dtm * sh.p[j];
    LB_SYNC();
    return 0;
}

// Appends, in increasing k, the k < n with fe(k) to le and those with fl(k)
// to ll (tile by tile over the CTA, warp ballots for the offsets).
template <class FE, class FL>
LB_FN void block_append2(Shm& sh, int n, FE fe, FL fl, int* le, int* ll, int& ne, int& nl) {
    const int t = lb_tid();
    int be = 0, bl = 0;
    for (int k0 = 0; k0 < n; k0 += LB_NT) {
        const int k = k0 + t;
        const bool e = k < n && fe(k), l = k < n && fl(k);
#if defined(LB_HOST_EMU)
        if (e) le[be] = k;
        if (l) ll[bl] = k;
        be += e ? 1 : 0;
        bl += l ? 1 : 0;
#else
        const unsigned me = __ballot_sync(0xffffffffu, e), ml = __ballot_sync(0xffffffffu, l);
        const unsigned below = (1u << lane_of(t)) - 1u;
        if (lane_of(t) == 0) {
            sh.red_i[warp_of(t)] = __popc(me);
            sh.red_i2[warp_of(t)] = __popc(ml);
        }
        LB_SYNC();
        int oe = be, ol = bl, te = 0, tl = 0;
        for (int w = 0; w < LB_NW; ++w) {
            if (w < warp_of(t)) {
                oe += sh.red_i[w];
                ol += sh.red_i2[w];
            }
            te += sh.red_i[w];
            tl += sh.red_i2[w];
        }
        if (e) le[oe + __popc(me & below)] = k;
        if (l) ll[ol + __popc(ml & below)] = k;
        be += te;
        bl += tl;
        LB_SYNC();
#endif
    }
    ne = be;
    nl = bl;
}

// Free set at the Cauchy point; sets s.nfree and s.wrk (the set changed or
// the memory was updated), and the lists of the variables that entered and
// left it (used to update the subspace matrix's Gram blocks).
LB_FN void free_set(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    const bool count = sh.s.iter > 0 && P.cnstnd;
    int ne = 0, nl = 0, nf = 0;
    if (count)
        block_append2(
            sh, P.n, [&](int k) { return A.iwhere[k] <= 0 && A.wasfree[k] == 0; },
            [&](int k) { return A.iwhere[k] > 0 && A.wasfree[k] != 0; }, c.elist, c.llist, ne, nl);
    for (int k = lb_tid(); k < P.n; k += LB_NT) {
        const bool fr = A.iwhere[k] <= 0;
        A.wasfree[k] = fr ? 1 : 0;
        nf += fr ? 1 : 0;
    }
    nf = block_sum_i(sh, nf);
    if (lb_tid() == 0) {
        sh.s.wrk = (ne + nl > 0 || sh.s.updatd) ? 1 : 0;
        sh.s.nfree = nf;
        sh.nenter = ne;
        sh.nleave = nl;
    }
    LB_SYNC();
}

// Factor of the middle matrix of the subspace step,
//   K = [ D + Y^T Z Z^T Y / theta      -L_a^T + R_z^T ]
//       [ -L_a + R_z            theta S^T A A^T S     ]
// (Z the free, A the active variables; L_a the strictly lower part of S^T A A^T Y,
// R_z the upper part of S^T Z Z^T Y), as [[R11, R12], [0, R22]] upper in sh.wn.
// The Gram blocks are kept in wn1 (2m x 2m, column-major, lower):
//   wn1(i, j)         = y_i^T Z Z^T y_j         (j <= i)
//   wn1(m + i, m + j) = s_i^T A A^T s_j         (j <= i)
//   wn1(m + i, j)     = s_i^T A A^T y_j (i > j), s_i^T Z Z^T y_j (i <= j)
// and, as in the published algorithm, updated from the previous iteration's
// blocks: the newest pair's row and column over all variables, and the old
// entries by the variables that entered or left the free set. They are formed
// from their definition after a memory refresh, when the previous blocks are
// stale, or when more than an eighth of the variables changed sides.
LB_FN int form_k(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    State& s = sh.s;
    const int n = P.n, m = P.m, col = s.col, ld = 2 * P.m;
    double* wn1 = sh.wn1;
    auto wcol = [&](int q) {  // staged columns: Y (logical order) then S
        return (q < col ? A.wy : A.ws) + (size_t)colptr(s, m, q < col ? q : q - col) * n;
    };
    const bool incremental = s.wn1_valid && 8 * (sh.nenter + sh.nleave) <= n;
    if (!incremental) {
        const int J1 = col * (col + 1) / 2;
        const int J = 2 * J1 + col * col;
        tiled_gram(J, n, 2 * col, wcol, A.iwhere,
                   [&](int o, int& a, int& b, int& mode) {
                       if (o < 2 * J1) {  // lower triangles of Y^T Z Z^T Y, then S^T A A^T S
                           const int oo = o < J1 ? o : o - J1;
                           int i = 0;
                           while ((i + 1) * (i + 2) / 2 <= oo) ++i;
                           const int j = oo - i * (i + 1) / 2;
                           const int base = o < J1 ? 0 : col;
                           a = base + i;
                           b = base + j;
                           mode = o < J1 ? 1 : 2;
                       } else {  // S^T Y split: active below the diagonal, free on and above
                           const int oo = o - 2 * J1;
                           const int i = oo / col, j = oo % col;
                           a = col + i;
                           b = j;
                           mode = i > j ? 2 : 1;
                       }
                   },
                   c.tile, c.tmask, sh.dots);
        for (int o = lb_tid(); o < J; o += LB_NT) {
            if (o < 2 * J1) {
                const int oo = o < J1 ? o : o - J1;
                int i = 0;
                while ((i + 1) * (i + 2) / 2 <= oo) ++i;
                const int j = oo - i * (i + 1) / 2;
                const int off = o < J1 ? 0 : m;
                wn1[(off + i) + (off + j) * ld] = sh.dots[o];
            } else {
                const int oo = o - 2 * J1;
                wn1[(m + oo / col) + (oo % col) * ld] = sh.dots[o];
            }
        }
        LB_SYNC();
    } else {
        int upcl = col;
        if (s.updatd) {
            if (s.iupdat > m && lb_tid() < LB_WARP) {  // drop the oldest pair's rows and columns
                for (int jy = 0; jy < m - 1; ++jy) {
                    for (int i = lane_id(); i < m - 1; i += LB_WARP) {
                        if (i < m - 1 - jy) {
                            wn1[(jy + i) + jy * ld] = wn1[(jy + 1 + i) + (jy + 1) * ld];
                            wn1[(m + jy + i) + (m + jy) * ld] = wn1[(m + jy + 1 + i) + (m + jy + 1) * ld];
                        }
                        wn1[(m + i) + jy * ld] = wn1[(m + 1 + i) + (jy + 1) * ld];
                    }
                    LB_SYNCWARP();
                }
            }
            LB_SYNC();
            // the newest pair (logical col - 1) against every pair, over all variables
            const int nw = col - 1;
            tiled_gram(4 * col, n, 2 * col, wcol, A.iwhere,
                       [&](int o, int& a, int& b, int& mode) {
                           const int j = o % col;
                           switch (o / col) {
                               case 0: a = nw; b = j; mode = 1; break;               // y_new^T Z Z^T y_j
                               case 1: a = col + nw; b = col + j; mode = 2; break;   // s_new^T A A^T s_j
                               case 2: a = col + nw; b = j; mode = 2; break;         // s_new^T A A^T y_j
                               default: a = col + j; b = nw; mode = 1; break;        // s_j^T Z Z^T y_new
                           }
                       },
                       c.tile, c.tmask, sh.dots);
            if (lb_tid() < LB_WARP) {
                for (int j = lane_id(); j < col; j += LB_WARP) {
                    wn1[nw + j * ld] = sh.dots[j];
                    wn1[(m + nw) + (m + j) * ld] = sh.dots[col + j];
                    if (j < nw) wn1[(m + nw) + j * ld] = sh.dots[2 * col + j];
                    wn1[(m + j) + nw * ld] = sh.dots[3 * col + j];
                }
            }
            LB_SYNC();
            upcl = col - 1;
        }
        // the old entries: add the entering variables' products, remove the leaving ones'
        const int np = upcl * (upcl + 1) / 2;
        const int ne = sh.nenter, nl = sh.nleave;
        for (int o = lb_tid(); o < 2 * np + upcl * upcl; o += LB_NT) {
            int i, j;
            const double *u, *w;
            double sgn = 1.0;
            int row, cl;
            if (o < 2 * np) {
                const int oo = o < np ? o : o - np;
                i = 0;
                while ((i + 1) * (i + 2) / 2 <= oo) ++i;
                j = oo - i * (i + 1) / 2;
                const bool ys = o < np;
                u = (ys ? A.wy : A.ws) + (size_t)colptr(s, m, i) * n;
                w = (ys ? A.wy : A.ws) + (size_t)colptr(s, m, j) * n;
                sgn = ys ? 1.0 : -1.0;  // free-set Gram of Y grows with the entering set, S^T A A^T S shrinks
                row = ys ? i : m + i;
                cl = ys ? j : m + j;
            } else {
                const int oo = o - 2 * np;
                i = oo / upcl;
                j = oo % upcl;
                u = A.ws + (size_t)colptr(s, m, i) * n;
                w = A.wy + (size_t)colptr(s, m, j) * n;
                sgn = i <= j ? 1.0 : -1.0;  // R_z: free set; L_a: active set
                row = m + i;
                cl = j;
            }
            double te = 0.0, tl = 0.0;
            for (int e = 0; e < ne; ++e) te += u[c.elist[e]] * w[c.elist[e]];
            for (int e = 0; e < nl; ++e) tl += u[c.llist[e]] * w[c.llist[e]];
            wn1[row + cl * ld] += sgn * (te - tl);
        }
        LB_SYNC();
    }
    if (lb_tid() < LB_WARP) {
        const int l = lane_id();
        const double theta = s.theta;
        double* wn = sh.wn;
        for (int iy = l; iy < col; iy += LB_WARP) {
            const int is = col + iy;
            for (int jy = 0; jy <= iy; ++jy) {
                const int js = col + jy;
                wn[jy + iy * ld] = wn1[iy + jy * ld] / theta;
                wn[js + is * ld] = wn1[(m + iy) + (m + jy) * ld] * theta;
            }
            for (int jy = 0; jy < iy; ++jy) wn[jy + is * ld] = -wn1[(m + iy) + jy * ld];
            for (int jy = iy; jy < col; ++jy) wn[jy + is * ld] = wn1[(m + iy) + jy * ld];
            wn[iy + iy * ld] += sh.sy[iy + iy * m];
        }
        LB_SYNCWARP();
        int info = warp_chol_upper(wn, ld, col, sh.rd) ? -1 : 0;
        if (!info) {
            warp_solve_upper_t_multi(wn, ld, col, sh.rd, wn + col * ld, ld, col);
            const int ne2 = col * (col + 1) / 2;
            for (int e = l; e < ne2; e += LB_WARP) {
                int jj = 0;
                while ((jj + 1) * (jj + 2) / 2 <= e) ++jj;
                const int ii = e - jj * (jj + 1) / 2;
                const int is = col + ii, js = col + jj;
                double acc = 0.0;
                for (int k = 0; k < col; ++k) acc += wn[k + is * ld] * wn[k + js * ld];
                wn[is + js * ld] += acc;
            }
            LB_SYNCWARP();
            if (warp_chol_upper(wn + col + col * ld, ld, col, sh.rd + col)) info = -2;
        }
        if (l == 0) {
            sh.info = info;
            s.wn1_valid = info == 0 ? 1 : 0;
        }
    }
    LB_SYNC();
    return sh.info;
}

// Reduced gradient r = -Z^T (B (z - x) + g) on the free entries (0 elsewhere).
LB_FN int reduced_gradient(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    const State& s = sh.s;
    const int n = P.n, m = P.m, col = s.col;
    if (!P.cnstnd && col > 0) {
        for (int k = lb_tid(); k < n; k += LB_NT) A.r[k] = -A.g[k];
        LB_SYNC();
        return 0;
    }
    if (lb_tid() < LB_WARP) {
        const int info = middle_times(sh, m, col, sh.c, sh.v) ? -8 : 0;
        if (lb_tid() == 0) sh.info = info;
    }
    LB_SYNC();
    if (sh.info) return sh.info;
    const double theta = s.theta;
    for (int k = lb_tid(); k < n; k += LB_NT) {
        if (A.iwhere[k] > 0) {
            A.r[k] = 0.0;
            continue;
        }
        double rk = -theta * (A.z[k] - A.x[k]) - A.g[k];
        for (int j = 0; j < col; ++j) {
            const size_t pj = (size_t)colptr(s, m, j) * n;
            rk = rk + A.wy[pj + k] * sh.v[j] + A.ws[pj + k] * (theta * sh.v[col + j]);
        }
        A.r[k] = rk;
    }
    LB_SYNC();
    return 0;
}

// Subspace minimisation from the Cauchy point: Newton step on the free
// variables, projected onto the box and kept if it is a descent direction,
// else backtracked to the box (Morales and Nocedal 2011).
LB_FN int subspace_min(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    const State& s = sh.s;
    const int n = P.n, m = P.m, col = s.col, col2 = 2 * s.col, ld = 2 * P.m;
    const double theta = s.theta;
    const int t = lb_tid();
    warp_dots(col2, n, A.iwhere,
              [&](int j, const double*& a, const double*& b, int& mode) {
                  const size_t pj = (size_t)colptr(s, m, j < col ? j : j - col) * n;
                  a = (j < col ? A.wy : A.ws) + pj;
                  b = A.r;
                  mode = 0;
              },
              sh.wv);
    if (t < LB_WARP) {
        for (int j = lane_id(); j < col; j += LB_WARP) sh.wv[col + j] *= theta;
        const int info = warp_rdiag(sh.wn, ld, col2, sh.rd);
        if (!info) {
            warp_solve_upper_t(sh.wn, ld, col2, sh.rd, sh.wv);
            for (int j = lane_id(); j < col; j += LB_WARP) sh.wv[j] = -sh.wv[j];
            LB_SYNCWARP();
            warp_solve_upper(sh.wn, ld, col2, sh.rd, sh.wv);
        }
        if (t == 0) sh.info = info;
    }
    LB_SYNC();
    if (sh.info) return sh.info;
    const double inv_theta = 1.0 / theta;
    int iw = 0;
    for (int k = t; k < n; k += LB_NT) {
        A.xp[k] = A.z[k];
        if (A.iwhere[k] > 0) continue;
        double dk = A.r[k];
        for (int j = 0; j < col; ++j) {
            const size_t pj = (size_t)colptr(s, m, j) * n;
            dk = dk + A.wy[pj + k] * sh.wv[j] / theta + A.ws[pj + k] * sh.wv[col + j];
        }
        dk *= inv_theta;
        A.r[k] = dk;
        const double xk = A.z[k];
        const int nb = P.nbd[k];
        double zk;
        if (nb == 0) {
            zk = xk + dk;
        } else if (nb == 1) {
            zk = fmax(P.lo[k], xk + dk);
            if (zk == P.lo[k]) iw = 1;
        } else if (nb == 2) {
            zk = fmin(P.hi[k], fmax(P.lo[k], xk + dk));
            if (zk == P.lo[k] || zk == P.hi[k]) iw = 1;
        } else {
            zk = fmin(P.hi[k], xk + dk);
            if (zk == P.hi[k]) iw = 1;
        }
        A.z[k] = zk;
    }
    if (block_sum_i(sh, iw) == 0) return 0;
    double ddp = 0.0;
    for (int k = t; k < n; k += LB_NT) ddp += (A.z[k] - A.x[k]) * A.g[k];
    ddp = block_sum(sh, ddp);
    if (!(ddp > 0.0)) return 0;
    // the projected step is not a descent direction: backtrack from the Cauchy point
    double alpha = 1.0;
    int ibd = 0x7fffffff;
    for (int k = t; k < n; k += LB_NT) {
        const double zk = A.xp[k];
        A.z[k] = zk;
        if (A.iwhere[k] > 0) continue;
        const double dk = A.r[k];
        const int nb = P.nbd[k];
        if (nb == 0) continue;
        double cand = 2.0;
        if (dk < 0.0 && nb <= 2) {
            const double t2 = P.lo[k] - zk;
            if (t2 >= 0.0)
                cand = 0.0;
            else if (dk * alpha < t2)
                cand = t2 / dk;
        } else if (dk > 0.0 && nb >= 2) {
            const double t2 = P.hi[k] - zk;
            if (t2 <= 0.0)
                cand = 0.0;
            else if (dk * alpha > t2)
                cand = t2 / dk;
        }
        if (cand < alpha) {
            alpha = cand;
            ibd = k;
        }
    }
    block_argmin(sh, alpha, ibd);
    if (t == 0 && alpha < 1.0) {
        const double dk = A.r[ibd];
        if (dk > 0.0) {
            A.z[ibd] = P.hi[ibd];
            A.r[ibd] = 0.0;
        } else if (dk < 0.0) {
            A.z[ibd] = P.lo[ibd];
            A.r[ibd] = 0.0;
        }
    }
    LB_SYNC();
    for (int k = t; k < n; k += LB_NT)
        if (A.iwhere[k] <= 0) A.z[k] += alpha * A.r[k];
    LB_SYNC();
    return 0;
}

// ---------------------------------------------------------------------------
// More-Thuente line search (one thread).

LB_FN void ls_step(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp,
                   double fp, double dp, int& brackt, double stpmin, double stpmax) {
    const double sgnd = dp * (dx / fabs(dx));
    double stpf;
    if (fp > fx) {
        const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
        const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
        double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
        if (stp < stx) gamma = -gamma;
        const double p = (gamma - dx) + theta;
        const double q = ((gamma - dx) + gamma) + dp;
        const double r = p / q;
        const double stpc = stx + r * (stp - stx);
        const double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx);
        if (fabs(stpc - stx) < fabs(stpq - stx))
            stpf = stpc;
        else
            stpf = stpc + (stpq - stpc) / 2.0;
        brackt = 1;
    } else if (sgnd < 0.0) {
        const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
        const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
        double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
        if (stp > stx) gamma = -gamma;
        const double p = (gamma - dp) + theta;
        const double q = ((gamma - dp) + gamma) + dx;
        const double r = p / q;
        const double stpc = stp + r * (stx - stp);
        const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
        stpf = fabs(stpc - stp) > fabs(stpq - stp) ? stpc : stpq;
        brackt = 1;
    } else if (fabs(dp) < fabs(dx)) {
        const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
        const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
        double gamma = s * sqrt(fmax(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
        if (stp > stx) gamma = -gamma;
        const double p = (gamma - dp) + theta;
        const double q = (gamma + (dx - dp)) + gamma;
        const double r = p / q;
        double stpc;
        if (r < 0.0 && gamma != 0.0)
            stpc = stp + r * (stx - stp);
        else if (stp > stx)
            stpc = stpmax;
        else
            stpc = stpmin;
        const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
        if (brackt) {
            stpf = fabs(stpc - stp) < fabs(stpq - stp) ? stpc : stpq;
            if (stp > stx)
                stpf = fmin(stp + 0.66 * (sty - stp), stpf);
            else
                stpf = fmax(stp + 0.66 * (sty - stp), stpf);
        } else {
            stpf = fabs(stpc - stp) > fabs(stpq - stp) ? stpc : stpq;
            stpf = fmin(stpmax, stpf);
            stpf = fmax(stpmin, stpf);
        }
    } else {
        if (brackt) {
            const double theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp;
            const double s = fmax(fabs(theta), fmax(fabs(dy), fabs(dp)));
            double gamma = s * sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
            if (stp > sty) gamma = -gamma;
            const double p = (gamma - dp) + theta;
            const double q = ((gamma - dp) + gamma) + dy;
            const double r = p / q;
            stpf = stp + r * (sty - stp);
        } else if (stp > stx) {
            stpf = stpmax;
        } else {
            stpf = stpmin;
        }
    }
    if (fp > fx) {
        sty = stp;
        fy = fp;
        dy = dp;
    } else {
        if (sgnd < 0.0) {
            sty = stx;
            fy = fx;
            dy = dx;
        }
        stx = stp;
        fx = fp;
        dx = dp;
    }
    stp = stpf;
}

// One call of the search with f, g = f(stp), f'(stp); updates s.stp and s.ls_task.
LB_FN void ls_search(State& s, double f, double g, double stpmin, double stpmax) {
    if (s.ls_task == kLsStart) {
        if (s.stp < stpmin || s.stp > stpmax || g >= 0.0 || stpmax < stpmin) {
            s.ls_task = kLsError;
            return;
        }
        s.ls_brackt = 0;
        s.ls_stage = 1;
        s.ls_finit = f;
        s.ls_ginit = g;
        s.ls_gtest = kFtol * g;
        s.ls_width = stpmax - stpmin;
        s.ls_width1 = s.ls_width / 0.5;
        s.ls_stx = 0.0;
        s.ls_fx = f;
        s.ls_gx = g;
        s.ls_sty = 0.0;
        s.ls_fy = f;
        s.ls_gy = g;
        s.ls_stmin = 0.0;
        s.ls_stmax = s.stp + 4.0 * s.stp;
        s.ls_task = kLsFg;
        return;
    }
    const double ftest = s.ls_finit + s.stp * s.ls_gtest;
    if (s.ls_stage == 1 && f <= ftest && g >= 0.0) s.ls_stage = 2;
    int task = kLsFg;
    if (s.ls_brackt && (s.stp <= s.ls_stmin || s.stp >= s.ls_stmax)) task = kLsWarn;
    if (s.ls_brackt && s.ls_stmax - s.ls_stmin <= kXtol * s.ls_stmax) task = kLsWarn;
    if (s.stp == stpmax && f <= ftest && g <= s.ls_gtest) task = kLsWarn;
    if (s.stp == stpmin && (f > ftest || g >= s.ls_gtest)) task = kLsWarn;
    if (f <= ftest && fabs(g) <= kGtol * (-s.ls_ginit)) task = kLsConv;
    if (task == kLsWarn || task == kLsConv) {
        s.ls_task = task;
        return;
    }
    if (s.ls_stage == 1 && f <= s.ls_fx && f > ftest) {
        const double fm = f - s.stp * s.ls_gtest;
        double fxm = s.ls_fx - s.ls_stx * s.ls_gtest;
        double fym = s.ls_fy - s.ls_sty * s.ls_gtest;
        const double gm = g - s.ls_gtest;
        double gxm = s.ls_gx - s.ls_gtest;
        double gym = s.ls_gy - s.ls_gtest;
        ls_step(s.ls_stx, fxm, gxm, s.ls_sty, fym, gym, s.stp, fm, gm, s.ls_brackt, s.ls_stmin, s.ls_stmax);
        s.ls_fx = fxm + s.ls_stx * s.ls_gtest;
        s.ls_fy = fym + s.ls_sty * s.ls_gtest;
        s.ls_gx = gxm + s.ls_gtest;
        s.ls_gy = gym + s.ls_gtest;
    } else {
        ls_step(s.ls_stx, s.ls_fx, s.ls_gx, s.ls_sty, s.ls_fy, s.ls_gy, s.stp, f, g, s.ls_brackt, s.ls_stmin,
                s.ls_stmax);
    }
    if (s.ls_brackt) {
        if (fabs(s.ls_sty - s.ls_stx) >= 0.66 * s.ls_width1) s.stp = s.ls_stx + 0.5 * (s.ls_sty - s.ls_stx);
        s.ls_width1 = s.ls_width;
        s.ls_width = fabs(s.ls_sty - s.ls_stx);
    }
    if (s.ls_brackt) {
        s.ls_stmin = fmin(s.ls_stx, s.ls_sty);
        s.ls_stmax = fmax(s.ls_stx, s.ls_sty);
    } else {
        s.ls_stmin = s.stp + 1.1 * (s.stp - s.ls_stx);
        s.ls_stmax = s.stp + 4.0 * (s.stp - s.ls_stx);
    }
    s.stp = fmax(s.stp, stpmin);
    s.stp = fmin(s.stp, stpmax);
    if ((s.ls_brackt && (s.stp <= s.ls_stmin || s.stp >= s.ls_stmax)) ||
        (s.ls_brackt && s.ls_stmax - s.ls_stmin <= kXtol * s.ls_stmax))
        s.stp = s.ls_stx;
    s.ls_task = kLsFg;
}

// ---------------------------------------------------------------------------
// State machine.

LB_FN int stop(Shm& sh, int code) {
    if (lb_tid() == 0) {
        sh.s.wait = kStopped;
        sh.s.code = code;
    }
    LB_SYNC();
    return kLExit;
}

// Line search from label 556 on: evaluate the search at the current trial and
// either ask for f and g at the next trial, accept the point, or recover.
LB_FN int ls_body(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    State& s = sh.s;
    const int n = P.n, t = lb_tid();
    double gd = 0.0;
    for (int k = t; k < n; k += LB_NT) gd += A.g[k] * A.d[k];
    gd = block_sum(sh, gd);
    if (t == 0) {
        s.gd = gd;
        sh.trial = 0;
        if (s.ifun == 0) {
            s.gdold = gd;
            if (gd >= 0.0) s.info = -4;  // not a descent direction
        }
        if (s.info == 0) {
            ls_search(s, s.f, gd, 0.0, s.stpmx);
            if (s.ls_task == kLsError) s.info = -4;
        }
        if (s.info == 0 && s.ls_task != kLsConv && s.ls_task != kLsWarn) {
            ++s.ifun;
            ++s.nfgv;
            s.iback = s.ifun - 1;
            sh.trial = 1;
        }
    }
    LB_SYNC();
    if (s.info != 0 || s.iback >= P.maxls) {
        // restore the previous iterate
        for (int k = t; k < n; k += LB_NT) {
            A.x[k] = A.xold[k];
            A.g[k] = A.gold[k];
        }
        if (t == 0) {
            s.f = s.fold;
            if (s.col == 0) {
                if (s.info == 0) {
                    s.info = -9;
                    --s.nfgv;
                    --s.ifun;
                    --s.iback;
                }
                ++s.iter;
                s.wait = kStopped;
                s.code = kAbnormal;
                sh.label = kLExit;
            } else {
                if (s.info == 0) --s.nfgv;
                reset_memory(s);
                sh.label = kLIter;
            }
        }
        LB_SYNC();
        return sh.label;
    }
    if (sh.trial) {
        const double stp = s.stp;
        if (stp == 1.0) {
            for (int k = t; k < n; k += LB_NT) A.x[k] = A.z[k];
        } else {
            for (int k = t; k < n; k += LB_NT) A.x[k] = stp * A.d[k] + A.xold[k];
        }
        if (t == 0) s.wait = kWaitFgLn;
        LB_SYNC();
        return kLExit;
    }
    // a new iterate
    const double sbg = proj_grad_norm(c);
    if (t == 0) {
        ++s.iter;
        s.sbgnrm = sbg;
        ++s.nit;  // the driver's iteration count and its limits
        if (s.nit >= P.maxiter) {
            s.wait = kStopped;
            s.code = kMaxIter;
            sh.label = kLExit;
        } else if (s.nfev > P.maxfun) {
            s.wait = kStopped;
            s.code = kMaxFun;
            sh.label = kLExit;
        } else {
            sh.label = kLNewX;
        }
    }
    LB_SYNC();
    return sh.label;
}

// Labels 222-555: Cauchy point, subspace step, start of the line search.
LB_FN int iteration(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    State& s = sh.s;
    const int n = P.n, t = lb_tid();
    if (!P.cnstnd && s.col > 0) {
        for (int k = t; k < n; k += LB_NT) A.z[k] = A.x[k];
        if (t == 0) {
            s.wrk = s.updatd;
            sh.nenter = 0;
            sh.nleave = 0;
        }
        LB_SYNC();
    } else {
        if (cauchy(c)) {
            if (t == 0) reset_memory(s);
            LB_SYNC();
            return kLIter;
        }
        free_set(c);
    }
    if (s.nfree != 0 && s.col != 0) {
        int info = 0;
        if (s.wrk) info = form_k(c);
        if (!info) info = reduced_gradient(c);
        if (!info) info = subspace_min(c);
        if (info) {
            if (t == 0) reset_memory(s);
            LB_SYNC();
            return kLIter;
        }
    } else if (s.wrk) {  // the free set or the pairs changed without the Gram blocks following
        if (t == 0) s.wn1_valid = 0;
        LB_SYNC();
    }
    // line search start (lnsrlb before label 556)
    double dtd = 0.0, stpmx = kBig;
    for (int k = t; k < n; k += LB_NT) {
        const double dk = A.z[k] - A.x[k];
        A.d[k] = dk;
        dtd += dk * dk;
    }
    const bool bound_step = P.cnstnd && s.iter != 0;
    int dummy = 0;
    for (int k = t; k < n; k += LB_NT) {
        A.xold[k] = A.x[k];
        A.gold[k] = A.g[k];
        if (!bound_step) continue;
        const double a1 = A.d[k];
        const int nb = P.nbd[k];
        if (nb == 0) continue;
        if (a1 < 0.0 && nb <= 2) {
            const double a2 = P.lo[k] - A.x[k];
            if (a2 >= 0.0)
                stpmx = 0.0;
            else if (a1 * stpmx < a2)
                stpmx = a2 / a1;
        } else if (a1 > 0.0 && nb >= 2) {
            const double a2 = P.hi[k] - A.x[k];
            if (a2 <= 0.0)
                stpmx = 0.0;
            else if (a1 * stpmx > a2)
                stpmx = a2 / a1;
        }
    }
    dtd = block_sum(sh, dtd);
    block_argmin(sh, stpmx, dummy);
    if (t == 0) {
        s.dtd = dtd;
        s.dnorm = sqrt(dtd);
        s.stpmx = P.cnstnd ? (s.iter == 0 ? 1.0 : stpmx) : kBig;
        s.stp = (s.iter == 0 && !P.boxed) ? fmin(1.0 / s.dnorm, s.stpmx) : 1.0;
        s.fold = s.f;
        s.ifun = 0;
        s.iback = 0;
        s.ls_task = kLsStart;
    }
    LB_SYNC();
    return ls_body(c);
}

// Label 777: stopping tests, then the limited-memory update.
LB_FN int new_x(Ctx& c) {
    const Problem& P = c.P;
    const Arrays& A = c.A;
    Shm& sh = *c.sh;
    State& s = sh.s;
    const int n = P.n, m = P.m, t = lb_tid();
    if (s.sbgnrm <= P.pgtol) return stop(sh, kConvPgtol);
    {
        const double ddum = fmax(fabs(s.fold), fmax(fabs(s.f), 1.0));
        if (s.fold - s.f <= P.factr * kEpsMch * ddum) return stop(sh, kConvFtol);
    }
    double rr = 0.0;
    const double stp = s.stp;
    for (int k = t; k < n; k += LB_NT) {
        const double y = A.g[k] - A.gold[k];
        A.gold[k] = y;
        rr += y * y;
        if (stp != 1.0) A.d[k] = stp * A.d[k];
    }
    rr = block_sum(sh, rr);
    if (t == 0) {
        double dr, ddum;
        if (stp == 1.0) {
            dr = s.gd - s.gdold;
            ddum = -s.gdold;
        } else {
            dr = (s.gd - s.gdold) * stp;
            ddum = -s.gdold * stp;
        }
        sh.dr = dr;
        if (dr <= kEpsMch * ddum) {
            ++s.nskip;
            s.updatd = 0;
            sh.label = kLIter;
        } else {
            s.updatd = 1;
            ++s.iupdat;
            if (s.iupdat <= m) {
                s.col = s.iupdat;
                s.itail = (s.head + s.iupdat - 1) % m;
            } else {
                s.itail = (s.itail + 1) % m;
                s.head = (s.head + 1) % m;
            }
            s.theta = rr / dr;
            if (s.iupdat > m) {  // drop the oldest pair from S^T S and S^T Y
                const int col = s.col;
                for (int j = 0; j < col - 1; ++j) {
                    for (int i = 0; i <= j; ++i) sh.ss[i + j * m] = sh.ss[(i + 1) + (j + 1) * m];
                    for (int i = j; i < col - 1; ++i) sh.sy[i + j * m] = sh.sy[(i + 1) + (j + 1) * m];
                }
            }
            sh.label = kLNewX;  // marker: update in progress
        }
    }
    LB_SYNC();
    if (sh.label == kLIter) return kLIter;
    const int col = s.col, itail = s.itail;
    for (int k = t; k < n; k += LB_NT) {
        A.ws[(size_t)itail * n + k] = A.d[k];
        A.wy[(size_t)itail * n + k] = A.gold[k];
    }
    // new row of S^T Y and column of S^T S against the older pairs
    warp_dots(2 * (col - 1), n, A.iwhere,
              [&](int o, const double*& a, const double*& b, int& mode) {
                  const int j = o < col - 1 ? o : o - (col - 1);
                  a = A.d;
                  b = (o < col - 1 ? A.wy : A.ws) + (size_t)colptr(s, m, j) * n;
                  mode = 0;
              },
              sh.dots);
    if (t < LB_WARP) {
        const int l = lane_id();
        for (int j = l; j < col - 1; j += LB_WARP) {
            sh.sy[(col - 1) + j * m] = sh.dots[j];
            sh.ss[j + (col - 1) * m] = sh.dots[col - 1 + j];
        }
        if (l == 0) {
            sh.ss[(col - 1) + (col - 1) * m] = stp == 1.0 ? s.dtd : stp * stp * s.dtd;
            sh.sy[(col - 1) + (col - 1) * m] = sh.dr;
        }
        LB_SYNCWARP();
        for (int i = l; i < col; i += LB_WARP) sh.dinv[i] = 1.0 / sh.sy[i + i * m];
        LB_SYNCWARP();
        // T = theta S^T S + L D^-1 L^T (upper), then its Cholesky factor
        const double theta = s.theta;
        const int ne = col * (col + 1) / 2;
        for (int e = l; e < ne; e += LB_WARP) {
            int jj = 0;
            while ((jj + 1) * (jj + 2) / 2 <= e) ++jj;
            const int ii = e - jj * (jj + 1) / 2;
            double acc = 0.0;
            for (int k = 0; k < ii; ++k) acc += sh.sy[ii + k * m] * sh.sy[jj + k * m] * sh.dinv[k];
            sh.wt[ii + jj * m] = acc + theta * sh.ss[ii + jj * m];
        }
        LB_SYNCWARP();
        const int info = warp_chol_upper(sh.wt, m, col, sh.rd);
        if (l == 0 && info) reset_memory(s);
    }
    LB_SYNC();
    return kLIter;
}

// Consume f and g (already in s.f and A.g) and advance to the next request.
LB_FN void advance(Ctx& c) {
    Shm& sh = *c.sh;
    State& s = sh.s;
    int label;
    if (s.wait == kWaitFgStart) {
        const double sbg = proj_grad_norm(c);
        if (lb_tid() == 0) {
            s.nfgv = 1;
            s.sbgnrm = sbg;
        }
        LB_SYNC();
        label = sbg <= c.P.pgtol ? stop(sh, kConvPgtol) : kLIter;
    } else {
        label = ls_body(c);
    }
    int guard = 0;
    while (label != kLExit) {
        if (++guard > 64) {  // memory refreshes cannot repeat without a new f, g
            label = stop(sh, kAbnormal);
            break;
        }
        if (label == kLIter)
            label = iteration(c);
        else if (label == kLNewX)
            label = new_x(c);
        else
            label = kLExit;
    }
}

// ---------------------------------------------------------------------------
// Workspace layout and the per-restart bodies of the launches.

// Byte offsets in the caller's workspace. Problem-wide: header flags, bounds,
// bound codes; then the restarts' State records; then one block per restart.
struct Layout {
    long long header, lo, hi, nbd, states, per, per_bytes, total;
};

inline long long lb_align(long long x) { return (x + 255) / 256 * 256; }

inline Layout make_layout(long long R, long long n, int m) {
    Layout L;
    long long off = 0;
    auto take = [&](long long bytes) {
        const long long o = off;
        off += lb_align(bytes);
        return o;
    };
    L.header = take(64);
    L.lo = take(8 * n);
    L.hi = take(8 * n);
    L.nbd = take(n);
    L.states = take(R * (long long)sizeof(State));
    const long long doubles = 7 * n + 2 * (long long)m * n + 11 * (long long)m * m;
    L.per_bytes = lb_align(8 * doubles + 2 * n);
    L.per = off;
    off += R * L.per_bytes;
    L.total = off;
    return L;
}

// Next power of two >= n (the breakpoint sort's length).
inline int sort_len(int n) {
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    return n2;
}

// Dynamic shared memory of a step: sort keys (n2 doubles) and indices (n2 ints),
// then the Gram tile and its row flags.
LB_HD long long tile_offset(int n2) { return (12LL * n2 + 15) / 16 * 16; }
inline long long step_dyn_bytes(int n2) {
    return tile_offset(n2) + 8LL * (kTileRows + 1) * kTileCols + kTileRows;
}

struct InitArgs {
    Layout L;
    long long R;
    int n, m;
    char* ws;
    double* X;
    const double* lo;  // caller's bounds (n), +-inf where absent
    const double* hi;
};

struct StepArgs {
    Layout L;
    long long R;
    int n, m, maxls;
    long long maxiter, maxfun;
    double factr, pgtol;
    char* ws;
    double* X;             // R x n points (row r is restart r's x)
    const double* value;   // R values at X
    double sign;           // objective = sign * value (and gradient)
    const double* grad;    // R x n gradients of the value
    const int* status;     // R per-row status of the evaluation (0 = good), or null
    int ignore_status;
};

LB_FN Arrays restart_arrays(const Layout& L, char* ws, double* X, int r, int n, int m) {
    Arrays A;
    double* p = reinterpret_cast<double*>(ws + L.per + (long long)r * L.per_bytes);
    A.x = X + (long long)r * n;
    A.g = p;
    A.xold = p + n;
    A.gold = p + 2 * n;
    A.z = p + 3 * n;
    A.d = p + 4 * n;
    A.r = p + 5 * n;
    A.xp = p + 6 * n;
    A.ws = p + 7 * n;
    A.wy = A.ws + (long long)m * n;
    A.sy = A.wy + (long long)m * n;
    A.ss = A.sy + m * m;
    A.wt = A.ss + m * m;
    A.wn = A.wt + m * m;
    A.wn1 = A.wn + 4 * m * m;
    int8_t* q = reinterpret_cast<int8_t*>(A.wn1 + 4 * m * m);
    A.iwhere = q;
    A.wasfree = q + n;
    return A;
}

// Restart r: project its start onto the box and wait for f, g there. Restart 0
// also stores the bounds, their codes and the problem-wide flags.
LB_FN void init_restart(const InitArgs& a, int r, Shm& sh) {
    const int n = a.n, t = lb_tid();
    State* st = reinterpret_cast<State*>(a.ws + a.L.states) + r;
    double* wlo = reinterpret_cast<double*>(a.ws + a.L.lo);
    double* whi = reinterpret_cast<double*>(a.ws + a.L.hi);
    int8_t* wnbd = reinterpret_cast<int8_t*>(a.ws + a.L.nbd);
    Arrays A = restart_arrays(a.L, a.ws, a.X, r, n, a.m);
    double* x = A.x;
    int not_boxed = 0, constrained = 0;
    for (int k = t; k < n; k += LB_NT) {
        const double lo = a.lo[k], hi = a.hi[k];
        const bool hl = isfinite(lo), hh = isfinite(hi);
        const int nb = hl ? (hh ? 2 : 1) : (hh ? 3 : 0);
        if (r == 0) {
            wlo[k] = lo;
            whi[k] = hi;
            wnbd[k] = (int8_t)nb;
        }
        if (nb > 0) {
            if (nb <= 2 && x[k] <= lo)
                x[k] = lo;
            else if (nb >= 2 && x[k] >= hi)
                x[k] = hi;
        }
        A.iwhere[k] = (int8_t)(nb == 0 ? -1 : ((nb == 2 && hi - lo <= 0.0) ? 3 : 0));
        A.wasfree[k] = 1;
        not_boxed += nb != 2;
        constrained += nb > 0;
    }
    not_boxed = block_sum_i(sh, not_boxed);
    constrained = block_sum_i(sh, constrained);
    if (t == 0) {
        if (r == 0) {
            int* hdr = reinterpret_cast<int*>(a.ws + a.L.header);
            hdr[0] = not_boxed == 0;
            hdr[1] = constrained > 0;
        }
        State s = {};
        s.theta = 1.0;
        s.nfree = n;
        s.wait = kWaitFgStart;
        *st = s;
    }
}

// Restart r: consume f and g, advance to the next request or stop.
LB_FN void step_restart(const StepArgs& a, int r, Shm& sh, unsigned char* dyn, int n2) {
    double* key = reinterpret_cast<double*>(dyn);
    int* idx = reinterpret_cast<int*>(dyn + 8LL * n2);
    double* tile = reinterpret_cast<double*>(dyn + tile_offset(n2));
    int8_t* tmask = reinterpret_cast<int8_t*>(tile + (kTileRows + 1) * kTileCols);
    const int n = a.n, m = a.m, t = lb_tid();
    State* st = reinterpret_cast<State*>(a.ws + a.L.states) + r;
    if (t == 0) sh.s = *st;
    LB_SYNC();
    if (sh.s.wait == kStopped) return;
    if (!a.ignore_status && a.status != nullptr) {
        int bad = 0;
        for (long long i = t; i < a.R; i += LB_NT) bad += a.status[i] != 0;
        if (block_sum_i(sh, bad) > 0) {  // the caller evaluates these points again first
            if (t == 0) st->held = 1;
            return;
        }
    }
    Ctx c;
    const int* hdr = reinterpret_cast<const int*>(a.ws + a.L.header);
    c.P.n = n;
    c.P.m = m;
    c.P.maxls = a.maxls;
    c.P.boxed = hdr[0];
    c.P.cnstnd = hdr[1];
    c.P.maxiter = a.maxiter;
    c.P.maxfun = a.maxfun;
    c.P.factr = a.factr;
    c.P.pgtol = a.pgtol;
    c.P.lo = reinterpret_cast<const double*>(a.ws + a.L.lo);
    c.P.hi = reinterpret_cast<const double*>(a.ws + a.L.hi);
    c.P.nbd = reinterpret_cast<const int8_t*>(a.ws + a.L.nbd);
    c.A = restart_arrays(a.L, a.ws, a.X, r, n, m);
    c.sh = &sh;
    c.key = key;
    c.idx = idx;
    c.n2 = n2;
    c.tile = tile;
    c.tmask = tmask;
    c.elist = idx;
    c.llist = reinterpret_cast<int*>(key);
    for (int i = t; i < m * m; i += LB_NT) {
        sh.sy[i] = c.A.sy[i];
        sh.ss[i] = c.A.ss[i];
        sh.wt[i] = c.A.wt[i];
    }
    for (int i = t; i < 4 * m * m; i += LB_NT) {
        sh.wn[i] = c.A.wn[i];
        sh.wn1[i] = c.A.wn1[i];
    }
    const double fv = a.sign * a.value[r];
    int bad = isfinite(fv) ? 0 : 1;
    for (int k = t; k < n; k += LB_NT) {
        const double gk = a.sign * a.grad[(long long)r * n + k];
        c.A.g[k] = gk;
        bad += isfinite(gk) ? 0 : 1;
    }
    bad = block_sum_i(sh, bad);
    if (t == 0) {
        sh.s.f = fv;
        ++sh.s.nfev;
        sh.s.held = 0;
        if (bad) {
            sh.s.wait = kStopped;
            sh.s.code = kNonFinite;
        }
    }
    LB_SYNC();
    if (sh.s.wait != kStopped) advance(c);
    for (int i = t; i < m * m; i += LB_NT) {
        c.A.sy[i] = sh.sy[i];
        c.A.ss[i] = sh.ss[i];
        c.A.wt[i] = sh.wt[i];
    }
    for (int i = t; i < 4 * m * m; i += LB_NT) {
        c.A.wn[i] = sh.wn[i];
        c.A.wn1[i] = sh.wn1[i];
    }
    if (t == 0) *st = sh.s;
}

// Counts over the restarts: [0] waiting for f and g, [1] held back by a bad
// evaluation status, [2] stopped on a non-finite value or gradient, [3] stopped.
LB_FN void summarize(const Layout& L, const char* ws, long long R, Shm& sh, int* out) {
    const State* st = reinterpret_cast<const State*>(ws + L.states);
    int act = 0, held = 0, nonfin = 0, stopped = 0;
    for (long long i = lb_tid(); i < R; i += LB_NT) {
        const State& s = st[i];
        if (s.wait != kStopped) {
            ++act;
            held += s.held != 0;
        } else {
            ++stopped;
            nonfin += s.code == kNonFinite;
        }
    }
    act = block_sum_i(sh, act);
    held = block_sum_i(sh, held);
    nonfin = block_sum_i(sh, nonfin);
    stopped = block_sum_i(sh, stopped);
    if (lb_tid() == 0) {
        out[0] = act;
        out[1] = held;
        out[2] = nonfin;
        out[3] = stopped;
    }
}

}  // namespace bgb_lb

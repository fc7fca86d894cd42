/*
 * sw2d_oracle.c -- CPU oracle for the SW2D time-stepping core.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  The product path (libsw2d.so) never links or calls it.
 *
 * A serial FP64 restatement, written from scratch, of the update performed
 * by the reference SW2D-GPU solver loop (SW2D-GPU_linux/src/SW2D-GPU.cu,
 * cited below as "cu:<line>"):
 *
 *   cu:29-92     init_inf / initiald  active mask, face depths, wall flags
 *   cu:98-354    flux                 face discharges um (x-faces), vn (y-faces)
 *   cu:363-399   hm_hn                face depths
 *   cu:405-453   uu1_vv1              face velocities
 *   cu:459-484   uu_vv                cell velocities (output only)
 *   cu:490-523   uua_vva              transverse 4-point velocity averages
 *   cu:526-555   stream_flow          point-source / rain interpolation
 *   cu:589-601   evaporation_load     evaporation interpolation
 *   cu:603-665   continuity           depth update (called twice per step)
 *   cu:670-693   forward              state rotation
 *   cu:695-725   treat_error          dry-cell outflow fix
 *   cu:1256-1336 main loop            order of the above within one step
 *
 * Array semantics differ from the reference on purpose: faces are explicit
 * arrays with zero walls.  um is (rows+1) x cols, um[i][j] is the face between
 * cells (i-1,j) and (i,j); row 0 and row `rows` are the north/south walls.
 * vn is rows x (cols+1), vn[i][j] is the face between (i,j-1) and (i,j);
 * columns 0 and `cols` are the west/east walls.  Where the reference reads
 * its partial padding row or past its allocation (cu:829, cu:654, cu:172-174,
 * cu:298) this restatement reads the wall value 0, which is what the
 * reference reads when its buffers are zero-padded.
 *
 * Compile with -ffp-contract=off so that no multiply-add is fused: every
 * expression below keeps the reference's operation order, and the device
 * FP64 path is compiled without FMA contraction as well.
 *
 * Extensions that the reference does not have (documented, off by default):
 *   - a CFL time-step rule (the reference only has a fixed dt, cu:790);
 *   - an open south edge with free outfall q = 0.544 h sqrt(g h), the
 *     reference's own weir formula (cu:132);
 *   - per-cell Manning n (the reference has one scalar, cu:799);
 *     a face uses the mean of its two cells' n;
 *   - analytic rain (step / linear hyetograph, moving Gaussian storm);
 *   - FP64 mass budgets with Kahan summation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_RAIN_NONE 0
#define ORC_RAIN_COMPAT 1 /* mm per interval, reference formula cu:547-554 */
#define ORC_RAIN_STEP 2   /* mm/h, piecewise constant per interval          */
#define ORC_RAIN_LINEAR 3 /* mm/h, linear between knots, 0 outside          */
#define ORC_RAIN_STORM 4  /* moving Gaussian storm cell, mm/h               */

typedef struct {
    int32_t rows, cols;
    double dx, dy;
    double g;        /* 9.80, cu:809 */
    double th;       /* 1.0e-4, cu:1130 */
    double manning;  /* scalar n when no raster is given, cu:799 */
    double INT, INF, LWL, EV_WL_min; /* cu:627-634 */
    int32_t dt_mode; /* 0 = fixed dt (reference), 1 = CFL rule (extension) */
    double dt;       /* fixed half step, or the largest half step in CFL mode */
    double cfl;      /* Courant number of the CFL rule */
    int32_t south_open; /* 1 = free outfall on the south edge (extension) */
    int32_t pad0;
} orc_params;

typedef struct {
    int32_t rain_kind;
    int32_t n_rain;
    const double *rain;   /* series values */
    double rain_dt;       /* series interval [s] */
    /* storm: peak [mm/h], centre (x0,y0) [m] moving with (vx,vy) [m/s],
       sigma [m]; x grows with column j, y grows with row i (southwards) */
    double storm_peak, storm_x0, storm_y0, storm_vx, storm_vy, storm_sigma, storm_tstop;
    int32_t n_ev;
    int32_t pad0;
    const double *ev;     /* evaporation series, mm per ev_dt (cu:589-601) */
    double ev_dt;
    int32_t n_src;        /* point sources */
    int32_t n_qrec;       /* records per source series */
    const int32_t *src_cell; /* linear cell index i*cols+j of each source */
    const double *src_q;  /* [n_qrec][n_src] discharges, m^3/s */
    double dtoq;
    /* spatial rain distribution (extension; the reference rains one value
       on every cell, cu:654): per-cell factors rows*cols applied to the rain
       rate of the kind above, or NULL for uniform rain */
    const double *rain_w;
} orc_forcing;

typedef struct { double s, c; } kahan;

typedef struct {
    double rain_in;    /* m^3 added by rain on active cells */
    double source_in;  /* m^3 added by point sources (negative = sink) */
    double evap_out;   /* m^3 removed by evaporation */
    double outflow;    /* m^3 leaving through the open south edge */
    double clamp_gain; /* m^3 added by the depth clamp fmax(h,0) (cu:657) */
    double cmax;       /* wave-speed bound of the final state */
} orc_budget;

static void kadd(kahan *k, double v) {
    double y = v - k->c;
    double t = k->s + y;
    k->c = (t - k->s) - y;
    k->s = t;
}

/* ---- deterministic log / exp / power ------------------------------------
 * The friction term raises the face depth to 1.3333330 (cu:195, cu:312) and
 * the storm forcing needs exp().  Library pow/exp differ by ulps between
 * glibc and CUDA, and near the wet/dry threshold such ulps grow into
 * visible depth differences.  The oracle and the FP64 device path therefore
 * both use these routines, built only from IEEE-exact + - * / (no FMA), so
 * the two give identical bits.
 *
 * Table-driven forms (what the update calls):
 *   log: x = m 2^e with m in [1,2); the top 7 bits of m pick c = 1 + k/128;
 *        r = (m - c) * (1/c) (m - c exact), r in [0, 1/128); ln(1+r) by its
 *        series to r^8/8 (truncation < 2e-20); ln x = e ln2 + ln c + ln(1+r);
 *   exp: y = n ln2/64 + r with n = round(64 y/ln2), |r| <= ln2/128; e^r by
 *        its series to r^6/6! (truncation < 2e-20); e^y = 2^(n>>6) 2^((n&63)/64) e^r;
 *   ln2 and ln2/64 split into a 21-bit head (exact multiples) and a tail.
 * The tables 1/c, ln c and 2^(j/64) are built once from the series forms
 * below (log: atanh series on [1/sqrt2, sqrt2) to s^21/21; exp: Cody-Waite
 * by ln2 and Taylor to r^13/13!), the same way on the GPU. */
#define ORC_LN2_HI 0x1.62e42p-1
#define ORC_LN2_LO 0x1.fdf473de6af28p-22
#define ORC_INV_LN2 0x1.71547652b82fep+0

static double bits2d(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static uint64_t d2bits(double d) { uint64_t b; memcpy(&b, &d, 8); return b; }

static double log_series(double x) {
    uint64_t b = d2bits(x);
    int e = (int)((b >> 52) & 0x7ff) - 1023;
    double m = bits2d((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        e += 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double p = 1.0 / 21.0;
    p = p * s2 + 1.0 / 19.0;
    p = p * s2 + 1.0 / 17.0;
    p = p * s2 + 1.0 / 15.0;
    p = p * s2 + 1.0 / 13.0;
    p = p * s2 + 1.0 / 11.0;
    p = p * s2 + 1.0 / 9.0;
    p = p * s2 + 1.0 / 7.0;
    p = p * s2 + 1.0 / 5.0;
    p = p * s2 + 1.0 / 3.0;
    p = p * s2 + 1.0;
    double lm = 2.0 * s * p;
    double ef = (double)e;
    return ef * ORC_LN2_HI + (ef * ORC_LN2_LO + lm);
}

static double exp_series(double y) {
    double kf = floor(y * ORC_INV_LN2 + 0.5);
    double r = (y - kf * ORC_LN2_HI) - kf * ORC_LN2_LO;
    double p = 1.0 / 6227020800.0;
    p = p * r + 1.0 / 479001600.0;
    p = p * r + 1.0 / 39916800.0;
    p = p * r + 1.0 / 3628800.0;
    p = p * r + 1.0 / 362880.0;
    p = p * r + 1.0 / 40320.0;
    p = p * r + 1.0 / 5040.0;
    p = p * r + 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    int k = (int)kf;
    return p * bits2d((uint64_t)(k + 1023) << 52);
}

static double T_INV[128], T_LOGC[128], T_EXP2J[64];

__attribute__((constructor)) static void init_tables(void) {
    for (int k = 0; k < 128; k++) {
        double c = 1.0 + (double)k * 0.0078125;
        T_INV[k] = 1.0 / c;
        T_LOGC[k] = log_series(c);
    }
    for (int j = 0; j < 64; j++)
        T_EXP2J[j] = exp_series((double)j * (ORC_LN2_HI / 64.0) + (double)j * (ORC_LN2_LO / 64.0));
}

double orc_log(double x) {
    uint64_t b = d2bits(x);
    int e = (int)((b >> 52) & 0x7ff) - 1023;
    int k = (int)((b >> 45) & 127);
    double m = bits2d((b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL);
    double c = 1.0 + (double)k * 0.0078125;
    double r = (m - c) * T_INV[k];
    double p = -1.0 / 8.0;
    p = p * r + 1.0 / 7.0;
    p = p * r - 1.0 / 6.0;
    p = p * r + 1.0 / 5.0;
    p = p * r - 1.0 / 4.0;
    p = p * r + 1.0 / 3.0;
    p = p * r - 0.5;
    p = p * r + 1.0;
    double lr = p * r;
    double ef = (double)e;
    return ef * ORC_LN2_HI + (ef * ORC_LN2_LO + (T_LOGC[k] + lr));
}

double orc_exp(double y) {
    if (y < -700.0) return 0.0;
    if (y > 700.0) return HUGE_VAL;
    double nf = floor(y * (64.0 * ORC_INV_LN2) + 0.5);
    double r = (y - nf * (ORC_LN2_HI / 64.0)) - nf * (ORC_LN2_LO / 64.0);
    double p = 1.0 / 720.0;
    p = p * r + 1.0 / 120.0;
    p = p * r + 1.0 / 24.0;
    p = p * r + 1.0 / 6.0;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    int n = (int)nf;
    int j = n & 63, q = (n - j) / 64;  /* n = 64 q + j, 0 <= j < 64 */
    return (p * T_EXP2J[j]) * bits2d((uint64_t)(q + 1023) << 52);
}

/* hm^1.3333330 of the friction term (cu:195, cu:312), for hm > th > 0 */
double orc_pow43(double x) { return orc_exp(1.3333330 * orc_log(x)); }

void orc_pow43_vec(const double *x, int n, double *out) {
    for (int k = 0; k < n; k++) out[k] = orc_pow43(x[k]);
}

void orc_exp_vec(const double *x, int n, double *out) {
    for (int k = 0; k < n; k++) out[k] = orc_exp(x[k]);
}

/* ---- host forcing, restating cu:526-555 and cu:589-601 ---------------- */

/* The reference's interpolation divides by the elapsed time inside the
 * record instead of multiplying by it (cu:538, cu:552, cu:597); kept as is.
 * Table indices are clamped to the last record (the reference reads past
 * its table there). */
static double compat_series(const double *v, int n, double dtv, double t) {
    if (n <= 0) return 0.0;
    if (t <= 1.00) return v[0] * t;
    int it = (int)(t / dtv);
    int a = it < n ? it : n - 1;
    int b = it + 1 < n ? it + 1 : n - 1;
    return v[a] + (v[b] - v[a]) / (dtv * (t - dtv * (it)));
}

/* uniform rain rate [m/s] at time t, or the series part of it */
static double rain_uniform(const orc_forcing *f, double t) {
    switch (f->rain_kind) {
    case ORC_RAIN_COMPAT:
        return compat_series(f->rain, f->n_rain, f->rain_dt, t) / (f->rain_dt * 1000.0); /* cu:554 */
    case ORC_RAIN_STEP: {
        if (t < 0.0) return 0.0;
        long k = (long)floor(t / f->rain_dt);
        if (k >= f->n_rain) return 0.0;
        return f->rain[k] / 3.6e6;
    }
    case ORC_RAIN_LINEAR: {
        if (t < 0.0 || f->n_rain < 2) return 0.0;
        double s = t / f->rain_dt;
        long k = (long)floor(s);
        if (k >= f->n_rain - 1) return 0.0;
        double w = s - (double)k;
        return (f->rain[k] + w * (f->rain[k + 1] - f->rain[k])) / 3.6e6;
    }
    default:
        return 0.0;
    }
}

static double rain_cell(const orc_forcing *f, const orc_params *p, double t, int i, int j, double uni) {
    if (f->rain_kind != ORC_RAIN_STORM) return uni;
    if (t >= f->storm_tstop) return 0.0;
    double xc = f->storm_x0 + f->storm_vx * t;
    double yc = f->storm_y0 + f->storm_vy * t;
    double x = ((double)j + 0.5) * p->dx - xc;
    double y = ((double)i + 0.5) * p->dy - yc;
    double s2 = f->storm_sigma * f->storm_sigma;
    return f->storm_peak / 3.6e6 * orc_exp(-(x * x + y * y) / (2.0 * s2));
}

static double evap_rate(const orc_forcing *f, double t) {
    if (f->n_ev <= 0) return 0.0;
    return compat_series(f->ev, f->n_ev, f->ev_dt, t) / (f->ev_dt * 1000.0); /* cu:597-599 */
}

/* point sources: ql [m/s] scattered into a per-cell vector, last one wins
 * as in the reference's assignment (cu:540-545) */
static void scatter_sources(const orc_forcing *f, const orc_params *p, double t, double *ql) {
    for (int s = 0; s < f->n_src; s++) {
        double q;
        if (t <= 1.00) {
            q = f->src_q[s] * t;
        } else {
            int it = (int)(t / f->dtoq);
            int a = it < f->n_qrec ? it : f->n_qrec - 1;
            int b = it + 1 < f->n_qrec ? it + 1 : f->n_qrec - 1;
            double qa = f->src_q[(size_t)a * f->n_src + s];
            double qb = f->src_q[(size_t)b * f->n_src + s];
            q = qa + (qb - qa) / (f->dtoq * (t - f->dtoq * (it)));
        }
        q = q / (p->dx * p->dy);
        ql[f->src_cell[s]] = q;
    }
}

/* ---- derived fields (cu:363-453, cu:490-523) ----------------------------- */

typedef struct {
    int rows, cols;
    double *hm, *hn, *uu1, *vv1, *uua, *vva; /* hm/uu1/vva: (rows+1)*cols, hn/vv1/uua: rows*(cols+1) */
    double *ql, *hs;                           /* per cell */
    uint8_t *act;                              /* active mask */
    double *nf_x, *nf_y;                       /* face roughness */
} work;

#define XI(i, j) ((size_t)(i) * (size_t)cols + (size_t)(j))        /* x-faces & cells */
#define YI(i, j) ((size_t)(i) * (size_t)(cols + 1) + (size_t)(j))  /* y-faces */

static void derive(const orc_params *p, const double *h, const double *um, const double *vn, work *w) {
    const int rows = p->rows, cols = p->cols;
    const double th = p->th;
    /* hm: cu:378-387 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= rows; i++)
        for (int j = 0; j < cols; j++) {
            double hmv;
            if (i == 0) hmv = h[XI(0, j)];
            else if (i == rows) hmv = h[XI(rows - 1, j)];
            else hmv = 0.50 * (h[XI(i, j)] + h[XI(i - 1, j)]);
            w->hm[XI(i, j)] = hmv;
            w->uu1[XI(i, j)] = (hmv >= th) ? um[XI(i, j)] / hmv : 0.00; /* cu:418-423 */
        }
    /* hn: cu:374-394 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        for (int j = 0; j <= cols; j++) {
            double hnv;
            if (j == 0) hnv = h[XI(i, 0)];
            else if (j == cols) hnv = h[XI(i, cols - 1)];
            else hnv = 0.50 * (h[XI(i, j)] + h[XI(i, j - 1)]);
            w->hn[YI(i, j)] = hnv;
            w->vv1[YI(i, j)] = (hnv >= th) ? vn[YI(i, j)] / hnv : 0.0; /* cu:425-430 */
        }
    /* uua at y-faces (cu:502-513), vva at x-faces (cu:505-519) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        for (int j = 0; j <= cols; j++) {
            double v;
            if (j > 0 && j < cols)
                v = 0.250 * (w->uu1[XI(i, j)] + w->uu1[XI(i + 1, j)] + w->uu1[XI(i, j - 1)] +
                             w->uu1[XI(i + 1, j - 1)]);
            else
                v = 0.0; /* wall faces: never used */
            w->uua[YI(i, j)] = v;
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= rows; i++)
        for (int j = 0; j < cols; j++) {
            double v;
            if (i > 0 && i < rows)
                v = 0.250 * (w->vv1[YI(i, j)] + w->vv1[YI(i, j + 1)] + w->vv1[YI(i - 1, j)] +
                             w->vv1[YI(i - 1, j + 1)]);
            else
                v = 0.0;
            w->vva[XI(i, j)] = v;
        }
}

/* wave-speed bound of a state (build extension: the CFL rule).
 * max over faces between two active cells (and open south faces) whose
 * face depth is >= th of |face velocity| + sqrt(g * face depth). */
static double cmax_of(const orc_params *p, const work *w) {
    const int rows = p->rows, cols = p->cols;
    double cm = 0.0;
#pragma omp parallel for schedule(static) reduction(max : cm)
    for (int i = 0; i <= rows; i++)
        for (int j = 0; j < cols; j++) {
            int ok;
            if (i == 0) ok = 0;
            else if (i == rows) ok = p->south_open && w->act[XI(rows - 1, j)];
            else ok = w->act[XI(i, j)] && w->act[XI(i - 1, j)];
            double hmv = w->hm[XI(i, j)];
            if (ok && hmv >= p->th) {
                double c = fabs(w->uu1[XI(i, j)]) + sqrt(p->g * hmv);
                if (c > cm) cm = c;
            }
        }
#pragma omp parallel for schedule(static) reduction(max : cm)
    for (int i = 0; i < rows; i++)
        for (int j = 1; j < cols; j++) {
            if (!(w->act[XI(i, j)] && w->act[XI(i, j - 1)])) continue;
            double hnv = w->hn[YI(i, j)];
            if (hnv >= p->th) {
                double c = fabs(w->vv1[YI(i, j)]) + sqrt(p->g * hnv);
                if (c > cm) cm = c;
            }
        }
    return cm;
}

/* ---- momentum: cu:98-354 ------------------------------------------------- */

/* weir / dry-bed formulas shared by both face directions.  `a` is the cell
 * on the low-index side (north or west), `b` the high-index side. Returns 1
 * and sets *q when a dry-bed rule applies, 0 when the momentum equation must
 * be used. */
static int dry_bed(double g, double th, double ha, double za, double hb, double zb, double *q) {
    double hhb = hb + zb, hha = ha + za;
    double hbp = hb - th, hap = ha - th;
    if (hhb < za) { /* cu:130-137 */
        *q = (ha > th) ? 0.5440 * ha * sqrt(g * ha) : 0;
        return 1;
    }
    if (hha < zb) { /* cu:138-145 */
        *q = (hb > th) ? -0.544 * hb * sqrt(g * hb) : 0;
        return 1;
    }
    if (hbp * hap < 0) { /* cu:149-158 */
        if ((hb > 0) || (ha > 0)) {
            double hhan = hbp - hap;
            double sgnm = hhan / fabs(hhan);
            double hh3 = fmax((hb + zb), (ha + za)) - fmax(zb, za);
            *q = -sgnm * 0.350 * hh3 * sqrt(2.00 * g * hh3);
        } else {
            *q = 0;
        }
        return 1;
    }
    return 0;
}

static void momentum(const orc_params *p, const double *h, const double *z, const double *um_o,
                     const double *vn_o, const work *w, double dt2, double *um, double *vn) {
    const int rows = p->rows, cols = p->cols;
    const double g = p->g, th = p->th, dx = p->dx, dy = p->dy;
    /* x-faces (cu:116-225) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= rows; i++)
        for (int j = 0; j < cols; j++) {
            double out = 0;
            if (i > 0 && i < rows) {
                size_t e = XI(i, j), wc = XI(i - 1, j);
                if (w->act[e] && w->act[wc] && ((h[wc] > th) || (h[e] > th))) {
                    double q;
                    if (dry_bed(g, th, h[wc], z[wc], h[e], z[e], &q)) {
                        out = q;
                    } else {
                        double hmv = w->hm[e];
                        /* gravity, cu:166 */
                        double u13 = g * hmv * (dt2 / dx) * (h[e] + z[e] - h[wc] - z[wc]);
                        /* convection along i, cu:172-176 */
                        double uu_s = w->uu1[XI(i + 1, j)], uu_c = w->uu1[e], uu_n = w->uu1[XI(i - 1, j)];
                        double mo_s = um_o[XI(i + 1, j)], mo_c = um_o[e], mo_n = um_o[XI(i - 1, j)];
                        double u11uur = 0.50 * (uu_s + uu_c);
                        double u11uul = 0.50 * (uu_c + uu_n);
                        double umr = u11uur * (mo_s + mo_c) * 0.50 + fabs(u11uur) * (mo_c - mo_s) * 0.50;
                        double uml = u11uul * (mo_c + mo_n) * 0.50 + fabs(u11uul) * (mo_n - mo_c) * 0.50;
                        double u11 = (dt2 / dx) * (umr - uml);
                        /* convection along j, cu:178-190 (zero on column 0) */
                        double u12;
                        if (j == 0) {
                            u12 = 0;
                        } else {
                            double vv_ec = w->vv1[YI(i, j + 1)], vv_en = w->vv1[YI(i - 1, j + 1)];
                            double vv_wc = w->vv1[YI(i, j)], vv_wn = w->vv1[YI(i - 1, j)];
                            double mo_e = (j + 1 < cols) ? um_o[XI(i, j + 1)] : 0.0;
                            double mo_w = um_o[XI(i, j - 1)];
                            double u12vvu = 0.50 * (vv_ec + vv_en);
                            double u12vvd = 0.50 * (vv_wc + vv_wn);
                            double umu = u12vvu * (mo_e + mo_c) * 0.50 + fabs(u12vvu) * (mo_c - mo_e) * 0.50;
                            double umd = u12vvd * (mo_w + mo_c) * 0.50 + fabs(u12vvd) * (mo_w - mo_c) * 0.50;
                            u12 = (dt2 / dy) * (umu - umd);
                        }
                        /* friction, cu:194-199 */
                        double rn = w->nf_x ? w->nf_x[e] : p->manning;
                        double ram;
                        if (hmv <= th || rn == 0.0) {
                            ram = 0.00;
                        } else {
                            double sqx = sqrt(w->uu1[e] * w->uu1[e] + w->vva[e] * w->vva[e]);
                            double expx = orc_pow43(hmv);
                            ram = g * rn * rn * sqx / expx;
                        }
                        /* cu:203 */
                        out = ((1.00 - dt2 * ram * 0.50) * mo_c + (-u11 - u12 - u13)) / (1.00 + dt2 * ram * 0.50);
                    }
                }
            } else if (i == rows && p->south_open) {
                /* free outfall through the south edge (extension) */
                size_t c = XI(rows - 1, j);
                double hc = h[c];
                out = (w->act[c] && hc > th) ? 0.5440 * hc * sqrt(g * hc) : 0.0;
            }
            um[XI(i, j)] = out;
        }
    /* y-faces (cu:232-342) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        for (int j = 0; j <= cols; j++) {
            double out = 0;
            if (j > 0 && j < cols) {
                size_t nc = XI(i, j), sc = XI(i, j - 1);
                if (w->act[nc] && w->act[sc] && ((h[sc] > th) || (h[nc] > th))) {
                    double q;
                    if (dry_bed(g, th, h[sc], z[sc], h[nc], z[nc], &q)) {
                        out = q;
                    } else {
                        double hnv = w->hn[YI(i, j)];
                        double v13 = g * hnv * (dt2 / dy) * (h[nc] + z[nc] - h[sc] - z[sc]); /* cu:283 */
                        double mo_c = vn_o[YI(i, j)];
                        double v11;
                        if (i == 0) { /* cu:289-301 */
                            v11 = 0;
                        } else {
                            double v11uur = 0.50 * (w->uu1[XI(i + 1, j)] + w->uu1[XI(i + 1, j - 1)]);
                            double v11uul = 0.50 * (w->uu1[XI(i, j)] + w->uu1[XI(i, j - 1)]);
                            double mo_s = (i + 1 < rows) ? vn_o[YI(i + 1, j)] : 0.0;
                            double mo_n = vn_o[YI(i - 1, j)];
                            double vnr = v11uur * (mo_s + mo_c) * 0.50 + fabs(v11uur) * (mo_c - mo_s) * 0.50;
                            double vnl = v11uul * (mo_c + mo_n) * 0.50 + fabs(v11uul) * (mo_n - mo_c) * 0.50;
                            v11 = (dt2 / dx) * (vnr - vnl);
                        }
                        /* cu:303-307 */
                        double vv_e = w->vv1[YI(i, j + 1)], vv_c = w->vv1[YI(i, j)], vv_w = w->vv1[YI(i, j - 1)];
                        double mo_e = vn_o[YI(i, j + 1)], mo_w = vn_o[YI(i, j - 1)];
                        double v12vvu = 0.50 * (vv_e + vv_c);
                        double v12vvd = 0.50 * (vv_c + vv_w);
                        double vnu = v12vvu * (mo_e + mo_c) * 0.50 + fabs(v12vvu) * (mo_c - mo_e) * 0.50;
                        double vnd = v12vvd * (mo_w + mo_c) * 0.50 + fabs(v12vvd) * (mo_w - mo_c) * 0.50;
                        double v12 = (dt2 / dy) * (vnu - vnd);
                        /* friction, cu:311-316 */
                        double rn = w->nf_y ? w->nf_y[YI(i, j)] : p->manning;
                        double ram;
                        if (hnv <= th || rn == 0.0) {
                            ram = 0.00;
                        } else {
                            double sqy = sqrt(w->uua[YI(i, j)] * w->uua[YI(i, j)] + vv_c * vv_c);
                            double expy = orc_pow43(hnv);
                            ram = g * rn * rn * sqy / expy;
                        }
                        out = ((1.00 - dt2 * ram * 0.50) * mo_c + (-v11 - v12 - v13)) / (1.00 + dt2 * ram * 0.50); /* cu:320 */
                    }
                }
            }
            vn[YI(i, j)] = out;
        }
}

/* ---- continuity: cu:603-665 ---------------------------------------------- */

static void continuity(const orc_params *p, const orc_forcing *f, const double *ho, const double *um,
                       const double *vn, const work *w, double dt2, double t, double *h, int final,
                       kahan *rain_k, kahan *src_k, kahan *ev_k, kahan *clamp_k) {
    const int rows = p->rows, cols = p->cols;
    const double dx = p->dx, dy = p->dy;
    const double rr_u = rain_uniform(f, t);
    const double ev_u = evap_rate(f, t);
    const double area = dx * dy;
    double rain_s = 0.0, src_s = 0.0, ev_s = 0.0, cl_s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : rain_s, src_s, ev_s, cl_s)
    for (int i = 0; i < rows; i++) {
        /* per-row partials keep the sums deterministic for a given thread count */
        for (int j = 0; j < cols; j++) {
            size_t c = XI(i, j);
            double pct, evapo;
            if (ho[c] > p->EV_WL_min) { /* cu:627-634 */
                pct = 1.00 - p->LWL;
                evapo = ev_u;
            } else {
                pct = 1.00 - (p->INT + p->INF);
                evapo = 0.000;
            }
            double rr = rain_cell(f, p, t, i, j, rr_u);
            if (f->rain_w) rr = rr * f->rain_w[(size_t)i * cols + j];
            double ql = w->ql[c];
            /* cu:654 */
            double hv = ho[c] - dt2 * ((um[XI(i + 1, j)] - um[c]) / dx + (vn[YI(i, j + 1)] - vn[YI(i, j)]) / dy - ql - rr * pct + evapo);
            double hc = fmax(hv, 0.00); /* cu:657 */
            if (!w->act[c]) hc = 0.00;   /* cu:658-660 */
            h[c] = hc;
            if (final && w->act[c]) {
                rain_s += dt2 * rr * pct * area;
                src_s += dt2 * ql * area;
                ev_s += dt2 * evapo * area;
                if (hv < 0.0) cl_s += -hv * area;
            }
        }
    }
    if (final) {
        kadd(rain_k, rain_s);
        kadd(src_k, src_s);
        kadd(ev_k, ev_s);
        kadd(clamp_k, cl_s);
    }
}

/* ---- treat_error: cu:695-725, written per face ---------------------------- */

static void treat_error(const orc_params *p, const double *hs, const work *w, double *um, double *vn) {
    const int rows = p->rows, cols = p->cols;
    const double th = p->th;
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= rows; i++)
        for (int j = 0; j < cols; j++) {
            double q = um[XI(i, j)];
            /* cell above drains through its south face (cu:707-709) */
            if (q > 0 && i > 0 && w->act[XI(i - 1, j)] && hs[XI(i - 1, j)] < th) q = 0;
            /* cell below drains through its north face (cu:711) */
            else if (q < 0.0 && i < rows && w->act[XI(i, j)] && hs[XI(i, j)] < th) q = 0.00;
            um[XI(i, j)] = q;
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; i++)
        for (int j = 0; j <= cols; j++) {
            double q = vn[YI(i, j)];
            if (q > 0 && j > 0 && w->act[XI(i, j - 1)] && hs[XI(i, j - 1)] < th) q = 0; /* cu:713-715 */
            else if (q < 0 && j < cols && w->act[XI(i, j)] && hs[XI(i, j)] < th) q = 0; /* cu:717 */
            vn[YI(i, j)] = q;
        }
}

/* ---- public oracle API ------------------------------------------------------ */

typedef struct {
    orc_params p;
    work w;
    double *z, *h, *um, *vn, *um_o, *vn_o, *ho;
    double t;
    int64_t steps;
    kahan rain, src, ev, out, clamp;
    double cmax;
} orc_state;

static void *xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

orc_state *orc_create(const orc_params *p, const double *z, const double *nraster, double nodata) {
    orc_state *S = (orc_state *)xcalloc(1, sizeof(orc_state));
    S->p = *p;
    const int rows = p->rows, cols = p->cols;
    size_t nc = (size_t)rows * cols, nx = (size_t)(rows + 1) * cols, ny = (size_t)rows * (cols + 1);
    S->z = (double *)xcalloc(nc, sizeof(double));
    S->h = (double *)xcalloc(nc, sizeof(double));
    S->ho = (double *)xcalloc(nc, sizeof(double));
    S->um = (double *)xcalloc(nx, sizeof(double));
    S->um_o = (double *)xcalloc(nx, sizeof(double));
    S->vn = (double *)xcalloc(ny, sizeof(double));
    S->vn_o = (double *)xcalloc(ny, sizeof(double));
    work *w = &S->w;
    w->rows = rows;
    w->cols = cols;
    w->hm = (double *)xcalloc(nx, sizeof(double));
    w->uu1 = (double *)xcalloc(nx, sizeof(double));
    w->vva = (double *)xcalloc(nx, sizeof(double));
    w->hn = (double *)xcalloc(ny, sizeof(double));
    w->vv1 = (double *)xcalloc(ny, sizeof(double));
    w->uua = (double *)xcalloc(ny, sizeof(double));
    w->ql = (double *)xcalloc(nc, sizeof(double));
    w->hs = (double *)xcalloc(nc, sizeof(double));
    w->act = (uint8_t *)xcalloc(nc, 1);
    memcpy(S->z, z, nc * sizeof(double));
    for (size_t c = 0; c < nc; c++) w->act[c] = (z[c] != nodata) ? 1 : 0; /* cu:39-44 */
    if (nraster) {
        w->nf_x = (double *)xcalloc(nx, sizeof(double));
        w->nf_y = (double *)xcalloc(ny, sizeof(double));
        for (int i = 1; i < rows; i++)
            for (int j = 0; j < cols; j++)
                w->nf_x[XI(i, j)] = 0.5 * (nraster[XI(i, j)] + nraster[XI(i - 1, j)]);
        for (int i = 0; i < rows; i++)
            for (int j = 1; j < cols; j++)
                w->nf_y[YI(i, j)] = 0.5 * (nraster[XI(i, j)] + nraster[XI(i, j - 1)]);
    }
    return S;
}

void orc_destroy(orc_state *S) {
    if (!S) return;
    free(S->z); free(S->h); free(S->ho); free(S->um); free(S->um_o); free(S->vn); free(S->vn_o);
    work *w = &S->w;
    free(w->hm); free(w->uu1); free(w->vva); free(w->hn); free(w->vv1); free(w->uua);
    free(w->ql); free(w->hs); free(w->act); free(w->nf_x); free(w->nf_y);
    free(S);
}

/* Sets the state.  Inactive cells get h = 0 (the reference zeroes them in
 * the first continuity call, cu:658-660, and never reads them before). */
void orc_set_state(orc_state *S, const double *h, const double *um, const double *vn, double t) {
    const int rows = S->p.rows, cols = S->p.cols;
    size_t nc = (size_t)rows * cols, nx = (size_t)(rows + 1) * cols, ny = (size_t)rows * (cols + 1);
    for (size_t c = 0; c < nc; c++) S->h[c] = S->w.act[c] ? h[c] : 0.0;
    if (um) memcpy(S->um, um, nx * sizeof(double)); else memset(S->um, 0, nx * sizeof(double));
    if (vn) memcpy(S->vn, vn, ny * sizeof(double)); else memset(S->vn, 0, ny * sizeof(double));
    /* walls: faces on the domain edge or next to an inactive cell carry no
       flow (cu:116-118, cu:232-234); the open south edge is the exception */
    const uint8_t *act = S->w.act;
    for (int i = 0; i <= rows; i++)
        for (int j = 0; j < cols; j++) {
            int open;
            if (i == 0) open = 0;
            else if (i == rows) open = S->p.south_open && act[XI(rows - 1, j)];
            else open = act[XI(i, j)] && act[XI(i - 1, j)];
            if (!open) S->um[XI(i, j)] = 0.0;
        }
    for (int i = 0; i < rows; i++)
        for (int j = 0; j <= cols; j++) {
            int open = j > 0 && j < cols && act[XI(i, j)] && act[XI(i, j - 1)];
            if (!open) S->vn[YI(i, j)] = 0.0;
        }
    S->t = t;
    S->steps = 0;
    memset(&S->rain, 0, sizeof(kahan)); memset(&S->src, 0, sizeof(kahan));
    memset(&S->ev, 0, sizeof(kahan)); memset(&S->out, 0, sizeof(kahan));
    memset(&S->clamp, 0, sizeof(kahan));
    derive(&S->p, S->h, S->um, S->vn, &S->w);
    S->cmax = cmax_of(&S->p, &S->w);
}

/* the half step of the next iteration; returns 0 when the run is over */
static int next_dt(const orc_state *S, double t_end, double *dt_out) {
    const orc_params *p = &S->p;
    if (p->dt_mode == 0) {
        if (!(S->t + p->dt <= t_end)) return 0; /* cu:1256 */
        *dt_out = p->dt;
        return 1;
    }
    if (!(t_end - S->t > 1.0e-9)) return 0;
    double dt2 = 2.0 * p->dt;
    if (S->cmax > 0.0) {
        double dmin = p->dx < p->dy ? p->dx : p->dy;
        double cand = p->cfl * dmin / S->cmax;
        if (cand < dt2) dt2 = cand;
    }
    if (S->t + dt2 > t_end) dt2 = t_end - S->t;
    *dt_out = 0.5 * dt2;
    return 1;
}

/* One iteration of the reference loop (cu:1256-1336). */
static void orc_step(orc_state *S, const orc_forcing *f, double dt) {
    const orc_params *p = &S->p;
    const int rows = p->rows, cols = p->cols;
    size_t nc = (size_t)rows * cols, nx = (size_t)(rows + 1) * cols, ny = (size_t)rows * (cols + 1);
    work *w = &S->w;
    const double dt2 = 2.00 * dt; /* cu:808 */
    kahan dummy = {0, 0};
    /* the previous state becomes ho/umo/vno (cu:670-693) */
    memcpy(S->ho, S->h, nc * sizeof(double));
    memcpy(S->um_o, S->um, nx * sizeof(double));
    memcpy(S->vn_o, S->vn, ny * sizeof(double));
    /* flux (cu:1268) from h, umo, vno and the derived fields of this state */
    momentum(p, S->ho, S->z, S->um_o, S->vn_o, w, dt2, S->um, S->vn);
    /* provisional continuity with forcing at t (cu:1278-1287) */
    double t = S->t;
    memset(w->ql, 0, nc * sizeof(double));
    scatter_sources(f, p, t, w->ql);
    continuity(p, f, S->ho, S->um, S->vn, w, dt2, t, w->hs, 0, &dummy, &dummy, &dummy, &dummy);
    /* dry-cell outflow fix (cu:1294) */
    treat_error(p, w->hs, w, S->um, S->vn);
    t = t + dt; /* cu:1297 */
    /* final continuity with forcing at t+dt (cu:1302-1313) */
    memset(w->ql, 0, nc * sizeof(double));
    scatter_sources(f, p, t, w->ql);
    continuity(p, f, S->ho, S->um, S->vn, w, dt2, t, S->h, 1, &S->rain, &S->src, &S->ev, &S->clamp);
    if (p->south_open) {
        double o = 0.0;
        for (int j = 0; j < cols; j++) o += S->um[XI(rows, j)];
        kadd(&S->out, dt2 * o * p->dy);
    }
    t = t + dt; /* cu:1335 */
    S->t = t;
    S->steps += 1;
    /* derived fields of the new state (cu:1319-1326) */
    derive(p, S->h, S->um, S->vn, w);
    S->cmax = cmax_of(p, w);
}

/* Advances until max_steps iterations are done or the end time is reached.
 * Returns the number of iterations performed. */
int64_t orc_advance(orc_state *S, const orc_forcing *f, int64_t max_steps, double t_end) {
    int64_t n = 0;
    double dt;
    while (n < max_steps && next_dt(S, t_end, &dt)) {
        orc_step(S, f, dt);
        n++;
    }
    return n;
}

void orc_get(const orc_state *S, double *h, double *um, double *vn, double *t, int64_t *steps) {
    const int rows = S->p.rows, cols = S->p.cols;
    if (h) memcpy(h, S->h, (size_t)rows * cols * sizeof(double));
    if (um) memcpy(um, S->um, (size_t)(rows + 1) * cols * sizeof(double));
    if (vn) memcpy(vn, S->vn, (size_t)rows * (cols + 1) * sizeof(double));
    if (t) *t = S->t;
    if (steps) *steps = S->steps;
}

/* cell velocities of the current state (cu:459-484): uu along rows (i),
 * vv along columns (j) */
void orc_cell_velocity(const orc_state *S, double *uu, double *vv) {
    const int rows = S->p.rows, cols = S->p.cols;
    const work *w = &S->w;
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            size_t c = XI(i, j);
            if (S->h[c] >= S->p.th) {
                uu[c] = (w->uu1[XI(i + 1, j)] + w->uu1[c]) / 2.00;
                vv[c] = (w->vv1[YI(i, j + 1)] + w->vv1[YI(i, j)]) / 2.00;
            } else {
                uu[c] = 0.00;
                vv[c] = 0.00;
            }
        }
}

/* volume of water on active cells, Kahan-summed in row-major order */
double orc_volume(const orc_state *S) {
    kahan k = {0, 0};
    size_t nc = (size_t)S->p.rows * S->p.cols;
    for (size_t c = 0; c < nc; c++)
        if (S->w.act[c]) kadd(&k, S->h[c]);
    return k.s * S->p.dx * S->p.dy;
}

void orc_budget_get(const orc_state *S, orc_budget *b) {
    b->rain_in = S->rain.s;
    b->source_in = S->src.s;
    b->evap_out = S->ev.s;
    b->outflow = S->out.s;
    b->clamp_gain = S->clamp.s;
    b->cmax = S->cmax;
}

/* the half step the next iteration would use (0 when the run is over) */
double orc_next_dt(const orc_state *S, double t_end) {
    double dt = 0.0;
    if (!next_dt(S, t_end, &dt)) return 0.0;
    return dt;
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* oracle.c -- CPU restatement of SixTrackLib's tracking hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Plain C99, compiled with
 * -O2 -fno-fast-math -ffp-contract=off so that every +,-,*,/ is rounded
 * separately, exactly as the reference CPU build does.
 *
 * Every function cites the reference file:line whose arithmetic it restates;
 * the operation order inside each expression follows the reference so that
 * results are bit-identical to it (checked against oracle/_ref).
 *
 * Built with -DORC_FAST_POLICY=1 (oracle/liboracle_fast.so) the plain-ring
 * maps -- drift, multipole, rotation, elliptic aperture -- instead take the
 * CUDA engine's fast arithmetic policy: explicit fused multiply-adds, the
 * multipole's first Horner step without the products with a zero top-order
 * skew coefficient, and the Goertzel recurrence for multipoles of order >= 3
 * with real coefficients; =2 keeps the Horner kick for every multipole.
 * Those libraries measure on the CPU how far the fast policy departs from
 * the reference (tests/test_fast_policy_cpu.py); every other map is the
 * reference's in them as well.
 */
#include "oracle.h"

#include <math.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Host threads of the particle loops (all cores by default); returns the
 * number the loops will use. */
int orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ---------------------------------------------------------------- consts */
/* sixtracklib/common/constants.h:10-35, internal/physics_constants.h:28-70 */
#define O_PI 3.1415926535897932384626433832795028841971693993751
#define O_C_LIGHT 299792458.0
#define O_EPSILON_0 8.854187817620e-12
#define O_SQRT_PI 1.7724538509055160272981674833411451827975494561224
#define O_QELEM 1.60217662e-19
#define O_CHARGE0_SI 1.602176634e-19
#define O_DEG2RAD_LD 0.0174532925199432957692369076848861271344287188854172546L
#define O_QGAUSS_Q_EPS 1e-6L

/* object type ids: sixtracklib/common/internal/objects_type_id.h:16-55 */
enum {
    T_DRIFT = 2, T_DRIFT_EXACT = 3, T_MULTIPOLE = 4, T_CAVITY = 5,
    T_XYSHIFT = 6, T_SROTATION = 7, T_BB4D = 8, T_BB6D = 9, T_MONITOR = 10,
    T_LIMIT_RECT = 11, T_LIMIT_ELLIPSE = 12, T_SC_COASTING = 13,
    T_SC_QGAUSS = 14, T_LIMIT_RECT_ELLIPSE = 16, T_DIPEDGE = 24,
    T_RF_MULTIPOLE = 256, T_SC_INTERPOL = 257, T_LINE_DENSITY = 258,
    T_TRICUB_DATA = 260, T_TRICUB = 261
};

#define ST_OK 0
#define ST_FAIL (-1)

static int g_ap_mode = 2;
static double g_ap_min_len = 0.0;
static double g_ap_xlim = 1.0;
static double g_ap_ylim = 1.0;

void orc_set_aperture_mode(int mode, double min_length, double x_limit,
                           double y_limit)
{
    g_ap_mode = mode;
    g_ap_min_len = min_length;
    g_ap_xlim = x_limit;
    g_ap_ylim = y_limit;
}

static int g_flag_bb4d = 2, g_flag_bb6d = 2, g_flag_sc = 2, g_flag_tricub = 0;

void orc_set_track_flags(int bb4d, int bb6d, int sc, int tricub)
{
    g_flag_bb4d = bb4d;
    g_flag_bb6d = bb6d;
    g_flag_sc = sc;
    g_flag_tricub = tricub;
}

/* ------------------------------------------------------- particle record */
typedef struct {
    double q0, mass0, beta0, gamma0, p0c, s, x, y, px, py, zeta, psigma,
        delta, rpp, rvv, chi, charge_ratio;
    int64_t pid, at_element, at_turn, state;
} prec;

static void p_load(prec *p, const void *cols, int64_t n, int64_t i)
{
    const double *d = (const double *)cols;
    const int64_t *k = (const int64_t *)cols;
    p->q0 = d[0 * n + i];
    p->mass0 = d[1 * n + i];
    p->beta0 = d[2 * n + i];
    p->gamma0 = d[3 * n + i];
    p->p0c = d[4 * n + i];
    p->s = d[5 * n + i];
    p->x = d[6 * n + i];
    p->y = d[7 * n + i];
    p->px = d[8 * n + i];
    p->py = d[9 * n + i];
    p->zeta = d[10 * n + i];
    p->psigma = d[11 * n + i];
    p->delta = d[12 * n + i];
    p->rpp = d[13 * n + i];
    p->rvv = d[14 * n + i];
    p->chi = d[15 * n + i];
    p->charge_ratio = d[16 * n + i];
    p->pid = k[17 * n + i];
    p->at_element = k[18 * n + i];
    p->at_turn = k[19 * n + i];
    p->state = k[20 * n + i];
}

static void p_store(const prec *p, void *cols, int64_t n, int64_t i)
{
    double *d = (double *)cols;
    int64_t *k = (int64_t *)cols;
    d[0 * n + i] = p->q0;
    d[1 * n + i] = p->mass0;
    d[2 * n + i] = p->beta0;
    d[3 * n + i] = p->gamma0;
    d[4 * n + i] = p->p0c;
    d[5 * n + i] = p->s;
    d[6 * n + i] = p->x;
    d[7 * n + i] = p->y;
    d[8 * n + i] = p->px;
    d[9 * n + i] = p->py;
    d[10 * n + i] = p->zeta;
    d[11 * n + i] = p->psigma;
    d[12 * n + i] = p->delta;
    d[13 * n + i] = p->rpp;
    d[14 * n + i] = p->rvv;
    d[15 * n + i] = p->chi;
    d[16 * n + i] = p->charge_ratio;
    k[17 * n + i] = p->pid;
    k[18 * n + i] = p->at_element;
    k[19 * n + i] = p->at_turn;
    k[20 * n + i] = p->state;
}

/* ------------------------------------------------------ CObjects reading */
/* Layout: sixtracklib/common/buffer/managed_buffer_minimal.h:396-466 (header
 * [0]=stored base address, [4]=objects section address), sections are
 * [max_size, num_entities, entries...], an object entry is {begin_addr,
 * type_id, size} (buffer/buffer_object.h:24-30).  Stored addresses are
 * translated relative to the stored base, which makes remapping implicit. */
typedef struct {
    const uint8_t *img;
    uint64_t base;
    const uint64_t *objs;
    int64_t nobj;
} lattice_t;

static void lat_open(lattice_t *L, const uint8_t *img)
{
    const uint64_t *h = (const uint64_t *)img;
    L->img = img;
    L->base = h[0];
    const uint64_t *sec = (const uint64_t *)(img + (h[4] - h[0]));
    L->nobj = (int64_t)sec[1];
    L->objs = sec + 2;
}

int64_t orc_num_objects(const uint8_t *lattice)
{
    lattice_t L;
    lat_open(&L, lattice);
    return L.nobj;
}

static const void *lat_at(const lattice_t *L, uint64_t addr)
{
    return (const void *)(L->img + (addr - L->base));
}

static uint64_t obj_type(const lattice_t *L, int64_t i)
{
    return L->objs[3 * i + 1];
}

static const uint64_t *obj_words(const lattice_t *L, int64_t i)
{
    return (const uint64_t *)lat_at(L, L->objs[3 * i]);
}

static double w2d(uint64_t w)
{
    double d;
    memcpy(&d, &w, 8);
    return d;
}

static const double *obj_reals(const lattice_t *L, int64_t i)
{
    return (const double *)obj_words(L, i);
}

/* ------------------------------------------------------------- energy */
/* NS(Particles_add_to_energy_value): particles.h:5255-5297 */
static void p_add_energy(prec *p, double de)
{
    double const beta0 = p->beta0;
    double const delta_beta0 = p->delta * beta0;
    double const energy0 = sqrt(p->p0c * p->p0c + p->mass0 * p->mass0);
    double const ptau_beta0 =
        de / energy0 +
        sqrt(delta_beta0 * delta_beta0 + 2.0 * delta_beta0 * beta0 + 1.0) -
        1.0;
    double const ptau = ptau_beta0 / beta0;
    double const psigma = ptau / beta0;
    double const delta = sqrt(ptau * ptau + 2.0 * psigma + 1.0) - 1.0;
    double const opd = delta + 1.0;
    double const rvv = opd / (1.0 + ptau_beta0);
    p->delta = delta;
    p->psigma = psigma;
    p->zeta *= rvv / p->rvv;
    p->rvv = rvv;
    p->rpp = 1.0 / opd;
}

/* NS(Particles_update_delta_value): particles.h:5459-5496 */
static void p_set_delta(prec *p, double nd)
{
    double const beta0 = p->beta0;
    double const delta_beta0 = nd * beta0;
    double const ptau_beta0 =
        sqrt(delta_beta0 * delta_beta0 + 2.0 * delta_beta0 * beta0 + 1.0) -
        1.0;
    double const opd = 1.0 + nd;
    double const rvv = opd / (1.0 + ptau_beta0);
    double const rpp = 1.0 / opd;
    double const psigma = ptau_beta0 / (beta0 * beta0);
    p->delta = nd;
    p->rvv = rvv;
    p->rpp = rpp;
    p->psigma = psigma;
}

/* ------------------------------------------------------------ the maps */
/* be_drift/track.h:45-67 */
static int m_drift(prec *p, double L)
{
    double const rpp = p->rpp;
    double const xp = p->px * rpp;
    double const yp = p->py * rpp;
#if ORC_FAST_POLICY
    double const u = fma(fma(yp, yp, xp * xp), 0.5, 1.0);
    p->x = fma(xp, L, p->x);
    p->y = fma(yp, L, p->y);
    p->s += L;
    p->zeta = fma(L, p->rvv - u, p->zeta);
#else
    double const dzeta = p->rvv - (1.0 + (xp * xp + yp * yp) / 2.0);
    p->x += xp * L;
    p->y += yp * L;
    p->s += L;
    p->zeta += L * dzeta;
#endif
    return ST_OK;
}

/* be_drift/track.h:71-97 */
static int m_drift_exact(prec *p, double L)
{
    double const px = p->px, py = p->py;
    double const opd = p->delta + 1.0;
    double const lpzi = L / sqrt(opd * opd - (px * px + py * py));
    double const dzeta = p->rvv * L - opd * lpzi;
    p->x += px * lpzi;
    p->y += py * lpzi;
    p->s += L;
    p->zeta += dzeta;
    return ST_OK;
}

/* be_limit/track.h:54-88 */
static int m_limit_global(prec *p)
{
    double const x = p->x, y = p->y;
    double const sx = (double)((0.0 < x) - (double)(x < 0.0));
    double const sy = (double)((0.0 < y) - (double)(y < 0.0));
    p->state &= (int64_t)(((sx * x) < g_ap_xlim) & ((sy * y) < g_ap_ylim));
    return ST_OK;
}

/* be_multipole/track.h:38-112; struct be_multipole.h:27-34 */
static int m_multipole(const lattice_t *L, prec *p, const uint64_t *w)
{
    int64_t const order = (int64_t)w[0];
    double const length = w2d(w[1]);
    double const hxl = w2d(w[2]);
    double const hyl = w2d(w[3]);
    const double *bal = (const double *)lat_at(L, w[4]);
    int64_t ix = 2 * order;
    int64_t iy = ix + 1;
    double dpx = bal[ix];
    double dpy = bal[iy];
    double const x = p->x, y = p->y, chi = p->chi;
    int const curved = (hxl > 0.0) || (hyl > 0.0) || (hxl < 0.0) || (hyl < 0.0);
#if ORC_FAST_POLICY
    {
        const uint64_t *bw = (const uint64_t *)bal;
        int64_t k = order - 1;
        int real = 0;
        if (ORC_FAST_POLICY == 1 && order >= 3) {
            uint64_t im = 0;
            for (int64_t j = 0; j <= order; ++j) im |= bw[2 * j + 1];
            real = (im << 1) == 0;
        }
        if (real) {
            double const r = x + x, s = fma(x, x, y * y);
            double c1 = dpx, c0 = fma(r, c1, bal[2 * k]);
            for (int64_t j = order - 2; j >= 1; --j) {
                double const cj = fma(r, c0, fma(-s, c1, bal[2 * j]));
                c1 = c0;
                c0 = cj;
            }
            dpx = fma(x, c0, fma(-s, c1, bal[0]));
            dpy = y * c0;
            k = -1;
        } else if (k >= 0 && (bw[2 * order + 1] << 1) == 0) {
            double const nx = fma(dpx, x, bal[2 * k]);
            dpy = fma(dpx, y, bal[2 * k + 1]);
            dpx = nx;
            --k;
        }
        for (; k >= 0; --k) {
            double const tx = fma(-dpy, y, bal[2 * k]);
            double const ty = fma(dpy, x, bal[2 * k + 1]);
            double const nx = fma(dpx, x, tx);
            dpy = fma(dpx, y, ty);
            dpx = nx;
        }
        if (!curved) {
            p->px = fma(-chi, dpx, p->px);
            p->py = fma(chi, dpy, p->py);
            return ST_OK;
        }
        ix = 0;
    }
#endif
    while (ix > 0) {
        double const zre = dpx * x - dpy * y;
        double const zim = dpx * y + dpy * x;
        ix -= 2;
        iy -= 2;
        dpx = bal[ix] + zre;
        dpy = bal[iy] + zim;
    }
    dpx = -chi * dpx;
    dpy = chi * dpy;
    if (curved) {
        double const delta = p->delta;
        double const hxlx = x * hxl;
        double const hyly = y * hyl;
        p->zeta += chi * (hyly - hxlx);
        dpx += hxl + hxl * delta;
        dpy -= hyl + hyl * delta;
        if (length > 0.0) {
            double const b1l = chi * bal[0];
            double const a1l = chi * bal[1];
            dpx -= b1l * hxlx / length;
            dpy += a1l * hyly / length;
        }
    }
    p->px += dpx;
    p->py += dpy;
    return ST_OK;
}

/* be_cavity/track.h:39-67 */
static int m_cavity(prec *p, const double *c)
{
    double const DEG2RAD = O_PI / 180.0;
    double const K_FACTOR = (2.0 * O_PI) / O_C_LIGHT;
    double const q = p->q0 * p->charge_ratio;
    double const tau = p->zeta / (p->beta0 * p->rvv);
    double const phase = DEG2RAD * c[2] - K_FACTOR * c[1] * tau;
    double const energy = q * c[0] * sin(phase);
    p_add_energy(p, energy);
    return ST_OK;
}

/* be_xyshift/track.h:38-55 */
static int m_xyshift(prec *p, const double *c)
{
    double const mdx = -(c[0]);
    double const mdy = -(c[1]);
    p->x += mdx;
    p->y += mdy;
    return ST_OK;
}

/* be_srotation/track.h:38-69 */
static int m_srotation(prec *p, const double *c)
{
    double const cz = c[0], sz = c[1];
    double const x = p->x, y = p->y, px = p->px, py = p->py;
#if ORC_FAST_POLICY
    double const xh = fma(cz, x, sz * y);
    double const yh = fma(-sz, x, cz * y);
    double const pxh = fma(cz, px, sz * py);
    double const pyh = fma(-sz, px, cz * py);
#else
    double const xh = cz * x + sz * y;
    double const yh = -sz * x + cz * y;
    double const pxh = cz * px + sz * py;
    double const pyh = -sz * px + cz * py;
#endif
    p->x = xh;
    p->y = yh;
    p->px = pxh;
    p->py = pyh;
    return ST_OK;
}

/* be_limit/track.h:90-111 */
static int m_limit_rect(prec *p, const double *c)
{
    double const x = p->x, y = p->y;
    int64_t const ns =
        (int64_t)((x >= c[0]) && (x <= c[1]) && (y >= c[2]) && (y <= c[3]));
    p->state &= ns;
    return ST_OK;
}

/* be_limit/track.h:113-137 */
static int m_limit_ellipse(prec *p, const double *c)
{
#if ORC_FAST_POLICY
    double const t = fma(p->y * p->y, c[0], (p->x * p->x) * c[1]);
#else
    double t = p->x;
    double ys = p->y;
    t *= t;
    t *= c[1];
    ys *= ys;
    ys *= c[0];
    t += ys;
#endif
    p->state &= (int64_t)(t <= c[2]);
    return ST_OK;
}

/* be_limit/track.h:139-162 */
static int m_limit_rect_ellipse(prec *p, const double *c)
{
    double const x = p->x, y = p->y;
    double t = x * x * c[3];
    t += y * y * c[2];
    int64_t const ns = (int64_t)((x <= c[0]) && (x >= -c[0]) &&
                                 (y <= c[1]) && (y >= -c[1]) && (t <= c[4]));
    p->state &= ns;
    return ST_OK;
}

/* be_dipedge/track.h:37-51 */
static int m_dipedge(prec *p, const double *c)
{
    p->px += c[0] * p->x;
    p->py += c[1] * p->y;
    return ST_OK;
}

/* be_rfmultipole/track.h:39-118; struct be_rfmultipole.h */
static int m_rf_multipole(const lattice_t *L, prec *p, const uint64_t *w)
{
    int64_t const order = (int64_t)w[0];
    double const voltage = w2d(w[1]);
    double const frequency = w2d(w[2]);
    double const lag = w2d(w[3]);
    const double *bal = (const double *)lat_at(L, w[4]);
    const double *phase = (const double *)lat_at(L, w[5]);
    double const DEG2RAD = O_PI / 180.0;
    double const DEG2RAD_C = (double)O_DEG2RAD_LD;
    double const k = frequency * (2.0 * O_PI) / O_C_LIGHT;
    double const x = p->x, y = p->y;
    double const beta0 = p->beta0;
    double const zeta = p->zeta;
    double const q = p->q0 * p->charge_ratio * 1.0;
    double const rvv = p->rvv;
    double const ktau = k * zeta / (beta0 * rvv);
    double dpx = 0.0, dpy = 0.0, dptr = 0.0, zre = 1.0, zim = 0.0;
    for (int64_t kk = 0; kk <= order; kk++) {
        double const pn = DEG2RAD_C * phase[2 * kk] - ktau;
        double const ps = DEG2RAD * phase[2 * kk + 1] - ktau;
        double const bn = bal[2 * kk];
        double const bs = bal[2 * kk + 1];
        double const cn = cos(pn);
        double const cs = cos(ps);
        double const sn = sin(pn);
        double const ss = sin(ps);
        dpx += cn * (bn * zre) - cs * (bs * zim);
        dpy += cs * (bs * zre) + cn * (bn * zim);
        double const zret = zre * x - zim * y;
        zim = zim * x + zre * y;
        zre = zret;
        dptr += sn * (bn * zre) - ss * (bs * zim);
    }
    double const cav_energy = q * (voltage * sin(lag * DEG2RAD_C - ktau));
    double const p0c = p->p0c;
    double const rfm_energy = -q * ((k * p0c) * dptr);
    double const chi = p->chi;
    double const pxk = -chi * dpx;
    double const pyk = chi * dpy;
    double const ek = cav_energy + rfm_energy;
    p->px += pxk;
    p->py += pyk;
    p_add_energy(p, ek);
    return ST_OK;
}

/* -------------------------------------------------- Faddeeva / fields */
/* Complex error function w(z), CERN algorithm of K. Koelbig (program C335,
 * 1970) as used by be_beamfields/faddeeva_cern.h:45-120.  The backward
 * continued-fraction recursion and the Taylor-type sum are run in the same
 * operation order; the two loops are fused so no arrays are needed (the sum
 * consumes R[n-1] right after the recursion produces it). */
void orc_cerrf(double in_re, double in_im, double *w_re, double *w_im)
{
    double const a_const = 1.12837916709551;
    double const xlim = 5.33, ylim = 4.29;
    double const x = fabs(in_re);
    double const y = fabs(in_im);
    double wx, wy;
    if (y < ylim && x < xlim) {
        double const q = (1.0 - y / ylim) * sqrt(1.0 - (x / xlim) * (x / xlim));
        double const h = 1.0 / (3.2 * q);
        int const nc = 7 + (int)(23.0 * q);
        double xl = pow(h, (double)(1 - nc));
        double const xh = y + 0.5 / h;
        double const yh = x;
        int const nu = 10 + (int)(21.0 * q);
        double rx = 0.0, ry = 0.0; /* R[n] while iterating downwards */
        double sx = 0.0, sy = 0.0;
        for (int n = nu; n > 0; n--) {
            double const tx = xh + n * rx;
            double const ty = yh - n * ry;
            double const tn = tx * tx + ty * ty;
            rx = 0.5 * tx / tn; /* R[n-1] */
            ry = 0.5 * ty / tn;
            if (n <= nc) {
                double const saux = sx + xl;
                sx = rx * saux - ry * sy;
                sy = rx * sy + ry * saux;
                xl = h * xl;
            }
        }
        wx = a_const * sx;
        wy = a_const * sy;
    } else {
        double const xh = y;
        double const yh = x;
        double rx = 0.0, ry = 0.0;
        for (int n = 9; n > 0; n--) {
            double const tx = xh + n * rx;
            double const ty = yh - n * ry;
            double const tn = tx * tx + ty * ty;
            rx = 0.5 * tx / tn;
            ry = 0.5 * ty / tn;
        }
        wx = a_const * rx;
        wy = a_const * ry;
    }
    if (y == 0.0) {
        wx = exp(-x * x);
    }
    if (in_im < 0.0) {
        wx = 2.0 * exp(y * y - x * x) * cos(2.0 * x * y) - wx;
        wy = -2.0 * exp(y * y - x * x) * sin(2.0 * x * y) - wy;
        if (in_re > 0.0) {
            wy = -wy;
        }
    } else if (in_re < 0.0) {
        wy = -wy;
    }
    *w_re = wx;
    *w_im = wy;
}

/* Vectorised form for the dual-number oracle (one call per array). */
void orc_cerrf_n(const double *re, const double *im, double *w_re, double *w_im, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) orc_cerrf(re[i], im[i], &w_re[i], &w_im[i]);
}

/* gauss_fields.h:56-66 (Delta_x = Delta_y = 0 at every call site) */
static void field_round(double sigma, double x, double y, double *ex,
                        double *ey)
{
    double const dx = x - 0.0, dy = y - 0.0;
    double const r2 = dx * dx + dy * dy;
    double t;
    if (r2 < 1e-20) {
        t = sqrt(r2) / (2. * O_PI * O_EPSILON_0 * sigma);
    } else {
        t = (1 - exp(-0.5 * r2 / (sigma * sigma))) /
            (2. * O_PI * O_EPSILON_0 * r2);
    }
    *ex = t * dx;
    *ey = t * dy;
}

/* gauss_fields.h:68-131 (Bassetti-Erskine) */
static void field_ellip(double sigmax, double sigmay, double x, double y,
                        double *ex_out, double *ey_out)
{
    double const abx = fabs(x - 0.0);
    double const aby = fabs(y - 0.0);
    double S, fact, ex, ey, wz_re, wz_im, we_re, we_im, e;
    if (sigmax > sigmay) {
        S = sqrt(2. * (sigmax * sigmax - sigmay * sigmay));
        fact = 1. / (2. * O_EPSILON_0 * O_SQRT_PI * S);
        double const eta_re = sigmay / sigmax * abx;
        double const eta_im = sigmax / sigmay * aby;
        orc_cerrf(abx / S, aby / S, &wz_re, &wz_im);
        orc_cerrf(eta_re / S, eta_im / S, &we_re, &we_im);
        e = exp(-abx * abx / (2 * sigmax * sigmax) -
                aby * aby / (2 * sigmay * sigmay));
        ex = fact * (wz_im - we_im * e);
        ey = fact * (wz_re - we_re * e);
    } else if (sigmax < sigmay) {
        S = sqrt(2. * (sigmay * sigmay - sigmax * sigmax));
        fact = 1. / (2. * O_EPSILON_0 * O_SQRT_PI * S);
        double const eta_re = sigmax / sigmay * aby;
        double const eta_im = sigmay / sigmax * abx;
        orc_cerrf(aby / S, abx / S, &wz_re, &wz_im);
        orc_cerrf(eta_re / S, eta_im / S, &we_re, &we_im);
        e = exp(-aby * aby / (2 * sigmay * sigmay) -
                abx * abx / (2 * sigmax * sigmax));
        ey = fact * (wz_im - we_im * e);
        ex = fact * (wz_re - we_re * e);
    } else {
        ex = ey = 1. / 0.;
    }
    if ((x - 0.0) < 0) ex = -ex;
    if ((y - 0.0) < 0) ey = -ey;
    *ex_out = ex;
    *ey_out = ey;
}

/* gauss_fields.h:133-208 */
void orc_fields_gauss(double x, double y, double sigma_x, double sigma_y,
                      double min_sigma_diff, int skip_gs, double *ex_p,
                      double *ey_p, double *gx_p, double *gy_p)
{
    double ex, ey, gx, gy;
    if (fabs(sigma_x - sigma_y) < min_sigma_diff) {
        double const sigma = 0.5 * (sigma_x + sigma_y);
        field_round(sigma, x, y, &ex, &ey);
        if (skip_gs) {
            gx = 0.;
            gy = 0.;
        } else {
            gx = 1 / (2. * (x * x + y * y)) *
                 (y * ey - x * ex +
                  1. / (2 * O_PI * O_EPSILON_0 * sigma * sigma) * x * x *
                      exp(-(x * x + y * y) / (2. * sigma * sigma)));
            gy = 1. / (2 * (x * x + y * y)) *
                 (x * ex - y * ey +
                  1. / (2 * O_PI * O_EPSILON_0 * sigma * sigma) * y * y *
                      exp(-(x * x + y * y) / (2. * sigma * sigma)));
        }
    } else {
        field_ellip(sigma_x, sigma_y, x, y, &ex, &ey);
        double const s11 = sigma_x * sigma_x;
        double const s33 = sigma_y * sigma_y;
        if (skip_gs) {
            gx = 0.;
            gy = 0.;
        } else {
            gx = -1. / (2 * (s11 - s33)) *
                 (x * ex + y * ey +
                  1. / (2 * O_PI * O_EPSILON_0) *
                      (sigma_y / sigma_x *
                           exp(-x * x / (2 * s11) - y * y / (2 * s33)) -
                       1.));
            gy = 1. / (2 * (s11 - s33)) *
                 (x * ex + y * ey +
                  1. / (2 * O_PI * O_EPSILON_0) *
                      (sigma_x / sigma_y *
                           exp(-x * x / (2 * s11) - y * y / (2 * s33)) -
                       1.));
        }
    }
    *ex_p = ex;
    *ey_p = ey;
    if (!skip_gs) {
        *gx_p = gx;
        *gy_p = gy;
    }
}

/* be_beamfields/track.h:89-149; data layout be_beamfields.h:36-56 */
static int m_bb4d(const lattice_t *L, prec *p, const uint64_t *w)
{
    const double *d = (const double *)lat_at(L, w[1]);
    /* d: q_part N_part sigma_x sigma_y beta_s min_sigma_diff Delta_x Delta_y
     *    Dpx_sub Dpy_sub enabled */
    if (d[10] > 0.) {
        double px = p->px, py = p->py;
        double const qratio = 1.;
        double const charge = qratio * p->q0 * O_QELEM;
        double const x = p->x - d[6];
        double const y = p->y - d[7];
        double const chi = p->chi;
        double const beta = p->beta0 / p->rvv;
        double const p0c = p->p0c * O_QELEM;
        double ex, ey, gx, gy;
        orc_fields_gauss(x, y, d[2], d[3], d[5], 1, &ex, &ey, &gx, &gy);
        double const fact_kick = chi * d[1] * d[0] * charge *
                                 (1. + beta * d[4]) / (p0c * (beta + d[4]));
        px += (fact_kick * ex - d[8]);
        py += (fact_kick * ey - d[9]);
        p->px = px;
        p->py = py;
    }
    return ST_OK;
}

/* be_beamfields/be_beamfields.h:2101-2160 */
static void bb6d_boost(const double *b, double *x_s, double *px_s, double *y_s,
                       double *py_s, double *sg_s, double *dl_s)
{
    double const sphi = b[0], cphi = b[1], tphi = b[2], salpha = b[3],
                 calpha = b[4];
    double const x = *x_s, px = *px_s, y = *y_s, py = *py_s, sigma = *sg_s,
                 delta = *dl_s;
    double const h =
        delta + 1. - sqrt((1. + delta) * (1. + delta) - px * px - py * py);
    double const px_st = px / cphi - h * calpha * tphi / cphi;
    double const py_st = py / cphi - h * salpha * tphi / cphi;
    double const delta_st =
        delta - px * calpha * tphi - py * salpha * tphi + h * tphi * tphi;
    double const pz_st = sqrt((1. + delta_st) * (1. + delta_st) -
                              px_st * px_st - py_st * py_st);
    double const hx_st = px_st / pz_st;
    double const hy_st = py_st / pz_st;
    double const hsigma_st = 1. - (delta_st + 1) / pz_st;
    double const L11 = 1. + hx_st * calpha * sphi;
    double const L12 = hx_st * salpha * sphi;
    double const L13 = calpha * tphi;
    double const L21 = hy_st * calpha * sphi;
    double const L22 = 1. + hy_st * salpha * sphi;
    double const L23 = salpha * tphi;
    double const L31 = hsigma_st * calpha * sphi;
    double const L32 = hsigma_st * salpha * sphi;
    double const L33 = 1. / cphi;
    *x_s = L11 * x + L12 * y + L13 * sigma;
    *px_s = px_st;
    *y_s = L21 * x + L22 * y + L23 * sigma;
    *py_s = py_st;
    *sg_s = L31 * x + L32 * y + L33 * sigma;
    *dl_s = delta_st;
}

/* be_beamfields/be_beamfields.h:2162-2230 */
static void bb6d_inv_boost(const double *b, double *x, double *px, double *y,
                           double *py, double *sigma, double *delta)
{
    double const sphi = b[0], cphi = b[1], tphi = b[2], salpha = b[3],
                 calpha = b[4];
    double const x_st = *x, px_st = *px, y_st = *y, py_st = *py,
                 sigma_st = *sigma, delta_st = *delta;
    double const pz_st = sqrt((1. + delta_st) * (1. + delta_st) -
                              px_st * px_st - py_st * py_st);
    double const hx_st = px_st / pz_st;
    double const hy_st = py_st / pz_st;
    double const hsigma_st = 1. - (delta_st + 1) / pz_st;
    double const Det_L =
        1. / cphi + (hx_st * calpha + hy_st * salpha - hsigma_st * sphi) * tphi;
    double const Li11 =
        (1. / cphi + salpha * tphi * (hy_st - hsigma_st * salpha * sphi)) /
        Det_L;
    double const Li12 =
        (salpha * tphi * (hsigma_st * calpha * sphi - hx_st)) / Det_L;
    double const Li13 = -tphi *
                        (calpha - hx_st * salpha * salpha * sphi +
                         hy_st * calpha * salpha * sphi) /
                        Det_L;
    double const Li21 =
        (calpha * tphi * (-hy_st + hsigma_st * salpha * sphi)) / Det_L;
    double const Li22 =
        (1. / cphi + calpha * tphi * (hx_st - hsigma_st * calpha * sphi)) /
        Det_L;
    double const Li23 = -tphi *
                        (salpha - hy_st * calpha * calpha * sphi +
                         hx_st * calpha * salpha * sphi) /
                        Det_L;
    double const Li31 = -hsigma_st * calpha * sphi / Det_L;
    double const Li32 = -hsigma_st * salpha * sphi / Det_L;
    double const Li33 =
        (1. + hx_st * calpha * sphi + hy_st * salpha * sphi) / Det_L;
    double const x_i = Li11 * x_st + Li12 * y_st + Li13 * sigma_st;
    double const y_i = Li21 * x_st + Li22 * y_st + Li23 * sigma_st;
    double const sigma_i = Li31 * x_st + Li32 * y_st + Li33 * sigma_st;
    double const h = (delta_st + 1. - pz_st) * cphi * cphi;
    double const px_i = px_st * cphi + h * calpha * tphi;
    double const py_i = py_st * cphi + h * salpha * tphi;
    double const delta_i =
        delta_st + px_i * calpha * tphi + py_i * salpha * tphi - h * tphi * tphi;
    *x = x_i;
    *px = px_i;
    *y = y_i;
    *py = py_i;
    *sigma = sigma_i;
    *delta = delta_i;
}

static double o_sign(double a) { return (double)((a >= 0) - (a < 0)); }

/* be_beamfields/be_beamfields.h:2232-2385 */
static void bb6d_sigma(const double *sg, double S, double thr, int handle,
                       double *s11h, double *s33h, double *ct, double *st,
                       double *ds11h, double *ds33h, double *dct, double *dst)
{
    double const S11_0 = sg[0], S12_0 = sg[1], S13_0 = sg[2], S14_0 = sg[3],
                 S22_0 = sg[4], S23_0 = sg[5], S24_0 = sg[6], S33_0 = sg[7],
                 S34_0 = sg[8], S44_0 = sg[9];
    double const S11 = S11_0 + 2. * S12_0 * S + S22_0 * S * S;
    double const S33 = S33_0 + 2. * S34_0 * S + S44_0 * S * S;
    double const S13 = S13_0 + (S14_0 + S23_0) * S + S24_0 * S * S;
    double const S12 = S12_0 + S22_0 * S;
    double const S14 = S14_0 + S24_0 * S;
    double const S22 = S22_0 + 0. * S;
    double const S23 = S23_0 + S24_0 * S;
    double const S24 = S24_0 + 0. * S;
    double const S34 = S34_0 + S44_0 * S;
    double const S44 = S44_0 + 0. * S;
    double const R = S11 - S33;
    double const W = S11 + S33;
    double const T = R * R + 4 * S13 * S13;
    double const dS_R = 2. * (S12_0 - S34_0) + 2 * S * (S22_0 - S44_0);
    double const dS_W = 2. * (S12_0 + S34_0) + 2 * S * (S22_0 + S44_0);
    double const dS_S13 = S14_0 + S23_0 + 2 * S24_0 * S;
    double const dS_T = 2 * R * dS_R + 8. * S13 * dS_S13;
    double Sig_11_hat, Sig_33_hat, costheta, sintheta, dS_Sig_11_hat,
        dS_Sig_33_hat, dS_costheta, dS_sintheta, cos2theta, dS_cos2theta;
    double const signR = o_sign(R);
    if (T < thr && handle) {
        double const a = S12 - S34;
        double const b = S22 - S44;
        double const c = S14 + S23;
        double const d = S24;
        double sqrt_a2_c2 = sqrt(a * a + c * c);
        if (sqrt_a2_c2 * sqrt_a2_c2 * sqrt_a2_c2 < thr) {
            if (fabs(d) > thr) {
                cos2theta = fabs(b) / sqrt(b * b + 4 * d * d);
            } else {
                cos2theta = 1.;
            }
            costheta = sqrt(0.5 * (1. + cos2theta));
            sintheta = o_sign(b) * o_sign(d) * sqrt(0.5 * (1. - cos2theta));
            dS_costheta = 0.;
            dS_sintheta = 0.;
            Sig_11_hat = 0.5 * W;
            Sig_33_hat = 0.5 * W;
            dS_Sig_11_hat = 0.5 * dS_W;
            dS_Sig_33_hat = 0.5 * dS_W;
        } else {
            sqrt_a2_c2 = sqrt(a * a + c * c);
            cos2theta = fabs(2. * a) / (2 * sqrt_a2_c2);
            costheta = sqrt(0.5 * (1. + cos2theta));
            sintheta = o_sign(a) * o_sign(c) * sqrt(0.5 * (1. - cos2theta));
            dS_cos2theta =
                o_sign(a) * (0.5 * b / sqrt_a2_c2 -
                             a * (a * b + 2. * c * d) /
                                 (2. * sqrt_a2_c2 * sqrt_a2_c2 * sqrt_a2_c2));
            dS_costheta = 1. / (4. * costheta) * dS_cos2theta;
            if (fabs(sintheta) > thr) {
                dS_sintheta = -1. / (4. * sintheta) * dS_cos2theta;
            } else {
                dS_sintheta = d / (2. * a);
            }
            Sig_11_hat = 0.5 * W;
            Sig_33_hat = 0.5 * W;
            dS_Sig_11_hat = 0.5 * dS_W + o_sign(a) * sqrt_a2_c2;
            dS_Sig_33_hat = 0.5 * dS_W - o_sign(a) * sqrt_a2_c2;
        }
    } else {
        double const sqrtT = sqrt(T);
        cos2theta = signR * R / sqrtT;
        costheta = sqrt(0.5 * (1. + cos2theta));
        sintheta = signR * o_sign(S13) * sqrt(0.5 * (1. - cos2theta));
        Sig_11_hat = 0.5 * (W + signR * sqrtT);
        Sig_33_hat = 0.5 * (W - signR * sqrtT);
        dS_cos2theta =
            signR * (dS_R / sqrtT - R / (2 * sqrtT * sqrtT * sqrtT) * dS_T);
        dS_costheta = 1. / (4. * costheta) * dS_cos2theta;
        if (fabs(sintheta) < thr && handle) {
            dS_sintheta = (S14 + S23) / R;
        } else {
            dS_sintheta = -1. / (4. * sintheta) * dS_cos2theta;
        }
        dS_Sig_11_hat = 0.5 * (dS_W + signR * 0.5 / sqrtT * dS_T);
        dS_Sig_33_hat = 0.5 * (dS_W - signR * 0.5 / sqrtT * dS_T);
    }
    (void)S12;
    (void)S14;
    (void)S22;
    (void)S23;
    (void)S24;
    (void)S34;
    (void)S44;
    *s11h = Sig_11_hat;
    *s33h = Sig_33_hat;
    *ct = costheta;
    *st = sintheta;
    *ds11h = dS_Sig_11_hat;
    *ds33h = dS_Sig_33_hat;
    *dct = dS_costheta;
    *dst = dS_sintheta;
}

/* Relative-offset pointer of the BB6D payload (be_beamfields.h:23-27):
 * the word at field index f holds an offset o, data starts at f + o + 1. */
static const double *bb_rel(const uint64_t *d, int f)
{
    return (const double *)(d + f + d[f] + 1);
}

/* be_beamfields/track.h:342-507; payload be_beamfields.h:222-250 */
static int m_bb6d(const lattice_t *L, prec *p, const uint64_t *w)
{
    const uint64_t *dw = (const uint64_t *)lat_at(L, w[1]);
    const double *d = (const double *)dw;
    if (d[33] > 0.) {
        const double *n_part = bb_rel(dw, 34);
        const double *x_sl = bb_rel(dw, 35);
        const double *y_sl = bb_rel(dw, 36);
        const double *s_sl = bb_rel(dw, 37);
        int const n_slices = (int)((int64_t)dw[18]);
        double x = p->x, px = p->px, y = p->y, py = p->py, zeta = p->zeta,
               delta = p->delta;
        double const q0 = O_QELEM * p->q0;
        double const p0c = p->p0c;
        double const P0 = p0c / O_C_LIGHT * O_QELEM;
        double x_s = x - d[21] - d[19];
        double px_s = px - d[22];
        double y_s = y - d[23] - d[20];
        double py_s = py - d[24];
        double sg_s = zeta - d[25];
        double dl_s = delta - d[26];
        bb6d_boost(d + 1, &x_s, &px_s, &y_s, &py_s, &sg_s, &dl_s);
        for (int i = 0; i < n_slices; i++) {
            double const sig_sl = s_sl[i];
            double const x_sl_i = x_sl[i];
            double const y_sl_i = y_sl[i];
            double const Ksl = n_part[i] * d[0] * q0 / (P0 * O_C_LIGHT);
            double const S = 0.5 * (sg_s - sig_sl);
            double s11h, s33h, ct, st, ds11h, ds33h, dct, dst;
            bb6d_sigma(d + 6, S, d[17], 1, &s11h, &s33h, &ct, &st, &ds11h,
                       &ds33h, &dct, &dst);
            double const xb = x_s + px_s * S - x_sl_i;
            double const yb = y_s + py_s * S - y_sl_i;
            double const xbh = xb * ct + yb * st;
            double const ybh = -xb * st + yb * ct;
            double const dxbh = xb * dct + yb * dst;
            double const dybh = -xb * dst + yb * dct;
            double ex, ey, gx = 0.0, gy = 0.0;
            orc_fields_gauss(xbh, ybh, sqrt(s11h), sqrt(s33h), d[16], 0, &ex,
                             &ey, &gx, &gy);
            double const Fxh = Ksl * ex;
            double const Fyh = Ksl * ey;
            double const Gxh = Ksl * gx;
            double const Gyh = Ksl * gy;
            double const Fx = Fxh * ct - Fyh * st;
            double const Fy = Fxh * st + Fyh * ct;
            double const Fz =
                0.5 * (Fxh * dxbh + Fyh * dybh + Gxh * ds11h + Gyh * ds33h);
            dl_s = dl_s + Fz +
                   0.5 * (Fx * (px_s + 0.5 * Fx) + Fy * (py_s + 0.5 * Fy));
            x_s = x_s - S * Fx;
            px_s = px_s + Fx;
            y_s = y_s - S * Fy;
            py_s = py_s + Fy;
        }
        bb6d_inv_boost(d + 1, &x_s, &px_s, &y_s, &py_s, &sg_s, &dl_s);
        x = x_s + d[21] + d[19] - d[27];
        px = px_s + d[22] - d[28];
        y = y_s + d[23] + d[20] - d[29];
        py = py_s + d[24] - d[30];
        zeta = sg_s + d[25] - d[31];
        delta = dl_s + d[26] - d[32];
        p->x = x;
        p->px = px;
        p->y = y;
        p->py = py;
        p->zeta = zeta;
        p_set_delta(p, delta);
    }
    return ST_OK;
}

/* be_beamfields/track.h:154-198; struct be_beamfields.h:418-429 */
static int m_sc_coasting(prec *p, const double *c)
{
    /* c: number_of_particles circumference sigma_x sigma_y length x_co y_co
     *    min_sigma_diff enabled */
    double ex, ey, gx, gy;
    double const charge = O_CHARGE0_SI * p->q0;
    double const beta0 = p->beta0;
    double const pc0 = p->p0c * O_CHARGE0_SI;
    double fk = c[0] * c[4] * p->chi * p->charge_ratio * charge * charge *
                (1.0 - beta0 * beta0);
    fk /= c[1] * pc0 * beta0 * p->rvv;
    orc_fields_gauss(p->x - c[5], p->y - c[6], c[2], c[3], c[7], 1, &ex, &ey,
                     &gx, &gy);
    p->px += fk * ex;
    p->py += fk * ey;
    return ST_OK;
}

/* internal/math_qgauss.h:114-175 */
static double q_gauss(double x, double q, double sqrt_beta, double cq)
{
    double const arg = -(sqrt_beta * sqrt_beta * x * x);
    double const omq = 1.0 - q;
    double const abs_omq = (omq >= 0.0) ? omq : -omq;
    double e;
    if (abs_omq >= (double)O_QGAUSS_Q_EPS) {
        double u = 1.0 + omq * arg;
        if (u < 0.0) u = 0.0;
        e = pow(u, 1.0 / omq);
    } else {
        e = exp(arg);
    }
    return (sqrt_beta / cq) * e;
}

/* be_beamfields/track.h:203-268; struct be_beamfields.h:638-651 */
static int m_sc_qgauss(prec *p, const double *c)
{
    /* c: number_of_particles bunchlength_rms sigma_x sigma_y length x_co y_co
     *    min_sigma_diff q_param cq enabled */
    double ex, ey, gx, gy;
    double const charge = O_CHARGE0_SI * p->q0;
    double const beta0 = p->beta0;
    double const beta = beta0 * p->rvv;
    double const pc0 = p->p0c * O_CHARGE0_SI;
    double const z = p->zeta / p->rvv;
    double const blen = c[1];
    double fk = p->chi * p->charge_ratio * c[4] * charge * charge *
                (1.0 - beta0 * beta);
    fk *= c[0];
    fk *= q_gauss(z, c[8], 1.0 / (sqrt(2.0) * blen), c[9]);
    fk /= pc0 * beta;
    orc_fields_gauss(p->x - c[5], p->y - c[6], c[2], c[3], c[7], 1, &ex, &ey,
                     &gx, &gy);
    p->px += fk * ex;
    p->py += fk * ey;
    return ST_OK;
}

/* NS(LineDensityProfileData_interpolate_value), be_beamfields.h:3385-3408,
 * with NS(Math_interpol_y_equ) (internal/math_interpol.h:901-920): linear
 * (:649-665, y[i] + (z - (z0 + dz i)) yp[i]) and cubic (:789-816) evaluation.
 * d: the LineDensityProfileData object {method, capacity, values_addr,
 * derivatives_addr, z0, dz, num_values} (be_beamfields.h:887-897). */
static double ldp_word(const lattice_t *L, const uint64_t *d, int which, int64_t i)
{
    /* the readable window: from the first array's start to the end of the
     * second; inside the image or at a host address (the reference's CPU
     * semantics); reads outside it give 0 */
    uint64_t const va = d[2], da = d[3], cap = d[1];
    uint64_t const lo = va < da ? va : da;
    uint64_t const hi = (va > da ? va : da) + cap * 8u;
    uint64_t const a = d[2 + which] + (uint64_t)i * 8u;
    uint64_t const size = ((const uint64_t *)L->img)[1];
    double v = 0.0;
    if (i < 0 || a < lo || a + 8u > hi) return 0.0;
    if (lo >= L->base && hi <= L->base + size)
        memcpy(&v, lat_at(L, a), 8);
    else
        memcpy(&v, (const void *)(uintptr_t)a, 8);
    return v;
}

static double ldp_interpolate(const lattice_t *L, const uint64_t *d, double z)
{
    uint64_t const method = d[0];
    double z0, dz;
    memcpy(&z0, &d[4], 8);
    memcpy(&dz, &d[5], 8);
    int64_t const nv = (int64_t)d[6];
    double result = 0.0;
    if ((z <= z0 + dz * nv) && (z >= z0)) {
        int64_t const idx = (int64_t)((z - z0) / dz);
        if (method == 0) {
            result = ldp_word(L, d, 0, idx) + (z - (z0 + dz * idx)) * ldp_word(L, d, 1, idx);
        } else if (method == 1) {
            double const t2 = (z0 + dz * (idx + 1) - z) / dz;
            double const t1 = (z - (z0 + dz * idx)) / dz;
            double y = ldp_word(L, d, 0, idx + 1) * t1 + ldp_word(L, d, 0, idx) * t2;
            y -= ldp_word(L, d, 1, idx) * dz * dz * (t2 - t2 * t2 * t2) / 6.0;
            y -= ldp_word(L, d, 1, idx + 1) * dz * dz * (t1 - t1 * t1 * t1) / 6.0;
            result = y;
        }
    }
    return result;
}

/* be_beamfields/track.h:273-337; struct be_beamfields.h:1281-1293:
 * {number_of_particles, sigma_x, sigma_y, length, x_co, y_co,
 *  interpol_data_addr, line_density_prof_fallback, min_sigma_diff, enabled} */
static int m_sc_interpol(const lattice_t *L, prec *p, const uint64_t *w)
{
    const double *c = (const double *)w;
    double ex, ey, gx, gy;
    double const charge = O_CHARGE0_SI * p->q0;
    double const beta0 = p->beta0;
    double const beta = beta0 * p->rvv;
    double const pc0 = p->p0c * O_CHARGE0_SI;
    double fk = p->chi * p->charge_ratio * c[3] * c[0] * charge * charge *
                (1.0 - beta0 * beta);
    uint64_t const addr = w[6];
    uint64_t const size = ((const uint64_t *)L->img)[1];
    const uint64_t *d = NULL;
    if (addr != 0 && addr >= L->base && addr + 56u <= L->base + size)
        d = (const uint64_t *)lat_at(L, addr);
    else if (addr != 0)
        d = (const uint64_t *)(uintptr_t)addr; /* host address, as the reference */
    if (d != NULL && d[0] != 255u && (int64_t)d[6] > 0) {
        fk *= ldp_interpolate(L, d, p->zeta);
    } else {
        fk *= c[7];
    }
    fk /= (pc0 * beta);
    orc_fields_gauss(p->x - c[4], p->y - c[5], c[1], c[2], c[8], 1, &ex, &ey, &gx, &gy);
    p->px += fk * ex;
    p->py += fk * ey;
    return ST_OK;
}

/* ------------------------------------------------------------ TriCub */
/* NS(tricub_construct_coefs) (be_tricub/coefficients.h): the coefficients
 * c[i + 4 j + 16 k] of x^i y^j z^k are the inverse tricubic Hermite
 * constraint matrix times the corner values b[8 l + corner] (l: f, f_x, f_y,
 * f_z, f_xy, f_xz, f_yz, f_xyz; corner bit 0 / 1 / 2: upper node in x / y /
 * z).  That matrix is the Kronecker product of the 1-D cubic Hermite inverse
 * H (columns f(0), f(1), f'(0), f'(1)) in x, y and z; the reference's
 * generated code sums, per coefficient, entry * value over the nonzero
 * entries in ascending value order, the first one assigned, which is what
 * this loop does. */
static const int o_hermite[4][4] = {
    {1, 0, 0, 0}, {0, 0, 1, 0}, {-3, 3, -2, -1}, {2, -2, 1, 1}};
static const int o_tc_order[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                     {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

void orc_tricub_coefs(const double *b, double *coefs)
{
    for (int r = 0; r < 64; ++r) {
        int const i = r & 3, j = (r >> 2) & 3, k = r >> 4;
        int first = 1;
        double acc = 0.0;
        for (int v = 0; v < 64; ++v) {
            int const l = v >> 3, c = v & 7;
            int const a = o_hermite[i][2 * o_tc_order[l][0] + (c & 1)] *
                          o_hermite[j][2 * o_tc_order[l][1] + ((c >> 1) & 1)] *
                          o_hermite[k][2 * o_tc_order[l][2] + (c >> 2)];
            if (a == 0) continue;
            double const t = (double)a * b[v];
            acc = first ? t : acc + t;
            first = 0;
        }
        coefs[r] = acc;
    }
}

/* be_tricub/track.h:51-262; NS(TriCub) {x_shift, y_shift, tau_shift,
 * dipolar_kick_px, dipolar_kick_py, dipolar_kick_ptau, length, data_addr}
 * and NS(TriCubData) {x0, dx, nx, y0, dy, ny, z0, dz, nz, mirror_x,
 * mirror_y, mirror_z, table_addr} (be_tricub.h:33-52, 309-319).  data_addr
 * is a plain address: inside this image or a host address.  The reference
 * reads outside its table for a particle outside the grid (a debug
 * assertion only); here the particle is lost and the map fails, as on the
 * GPU.  data_addr 0 (the reference dereferences null) fails likewise. */
static int m_tricub(const lattice_t *L, prec *p, const uint64_t *w)
{
    const double *e = (const double *)w;
    uint64_t const addr = w[7];
    uint64_t const size = ((const uint64_t *)L->img)[1];
    const uint64_t *d;
    const double *table;
    if (addr == 0) return ST_FAIL;
    if (addr >= L->base && addr + 13u * 8u <= L->base + size) {
        d = (const uint64_t *)lat_at(L, addr);
        table = (const double *)lat_at(L, d[12]);
    } else {
        d = (const uint64_t *)(uintptr_t)addr;
        table = (const double *)(uintptr_t)d[12];
    }
    double const dx = w2d(d[1]), dy = w2d(d[4]), dz = w2d(d[7]);
    int64_t const nx = (int64_t)d[2], ny = (int64_t)d[5], nz = (int64_t)d[8];
    double const inv_dx = 1. / dx, inv_dy = 1. / dy, inv_dz = 1. / dz;
    double const z = p->zeta / (p->beta0 * p->rvv);
    double const fx = ((p->x - e[0]) - w2d(d[0])) * inv_dx;
    double const fy = ((p->y - e[1]) - w2d(d[3])) * inv_dy;
    double const fz = ((z - e[2]) - w2d(d[6])) * inv_dz;
    double const sign_x = ((int64_t)d[9] == 1 && fx < 0.0) ? -1. : 1.;
    double const sign_y = ((int64_t)d[10] == 1 && fy < 0.0) ? -1. : 1.;
    double const sign_z = ((int64_t)d[11] == 1 && fz < 0.0) ? -1. : 1.;
    double const sfx = sign_x * fx, sfy = sign_y * fy, sfz = sign_z * fz;
    double const ixf = floor(sfx), iyf = floor(sfy), izf = floor(sfz);
    if (!(ixf >= 0.0 && ixf <= (double)(nx - 2) && iyf >= 0.0 && iyf <= (double)(ny - 2) &&
          izf >= 0.0 && izf <= (double)(nz - 2))) {
        p->state = 0;
        return ST_FAIL;
    }
    int64_t const ix = (int64_t)ixf, iy = (int64_t)iyf, iz = (int64_t)izf;
    double const xn = sfx - ixf, yn = sfy - iyf, zn = sfz - izf;
    double b[64], c[64];
    for (int l = 0; l < 8; ++l)
        for (int corner = 0; corner < 8; ++corner) {
            int64_t const node = (ix + (corner & 1)) +
                                 nx * ((iy + ((corner >> 1) & 1)) + ny * (iz + (corner >> 2)));
            b[8 * l + corner] = table[l + 8 * node];
        }
    orc_tricub_coefs(b, c);
    double xp[4], yp[4], zp[4];
    xp[0] = yp[0] = zp[0] = 1.;
    xp[1] = xn;
    yp[1] = yn;
    zp[1] = zn;
    xp[2] = xn * xn;
    yp[2] = yn * yn;
    zp[2] = zn * zn;
    xp[3] = xp[2] * xn;
    yp[3] = yp[2] * yn;
    zp[3] = zp[2] * zn;
    double kpx = 0., kpy = 0., kpt = 0.;
    for (int i = 1; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 4; ++k)
                kpx += i * (((c[i + 4 * j + 16 * k] * xp[i - 1]) * yp[j]) * zp[k]);
    kpx *= (e[6] * inv_dx);
    kpx *= -sign_x;
    kpx -= e[3];
    for (int i = 0; i < 4; ++i)
        for (int j = 1; j < 4; ++j)
            for (int k = 0; k < 4; ++k)
                kpy += j * (((c[i + 4 * j + 16 * k] * xp[i]) * yp[j - 1]) * zp[k]);
    kpy *= (e[6] * inv_dy);
    kpy *= -sign_y;
    kpy -= e[4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            for (int k = 1; k < 4; ++k)
                kpt += k * (((c[i + 4 * j + 16 * k] * xp[i]) * yp[j]) * zp[k - 1]);
    kpt *= (e[6] * inv_dz);
    kpt *= -sign_z;
    kpt -= e[5];
    double const q = p->q0 * p->charge_ratio;
    double const energy_kick = q * (p->p0c * kpt);
    p->px += kpx;
    p->py += kpy;
    p_add_energy(p, energy_kick);
    return ST_OK;
}

/* ---------------------------------------------------------- monitors */
typedef struct {
    const orc_monitor_outputs *mon;
} track_ctx;

/* be_monitor/track.h:48-110 */
static int64_t monitor_store_index(const int64_t *m, int64_t turn,
                                   int64_t pid)
{
    /* m: num_stores start skip out_address max_pid min_pid is_rolling
     *    is_turn_ordered */
    int64_t out = -1;
    int64_t const start = m[1], nstores = m[0], skip = m[2];
    int64_t const since = turn - start;
    if ((since >= 0) && ((since % skip) == 0)) {
        int64_t idx = since / skip;
        if ((idx >= nstores) && (m[6] != 0)) idx = idx % nstores;
        if (idx < nstores) {
            int64_t const off = pid - m[5];
            int64_t const np = m[4] - m[5] + 1;
            if (m[7] != 0) {
                out = np * idx + off;
            } else {
                out = off * np + idx;
            }
        }
    }
    return out;
}

static int m_monitor(const lattice_t *L, prec *p, int64_t obj,
                     const track_ctx *ctx)
{
    const int64_t *m = (const int64_t *)obj_words(L, obj);
    int rc = 0;
    if (m[3] != 0) {
        /* output slot: ordinal among monitors with an output address */
        int64_t k = 0;
        for (int64_t j = 0; j < obj; j++) {
            if (obj_type(L, j) == T_MONITOR &&
                ((const int64_t *)obj_words(L, j))[3] != 0)
                k++;
        }
        int64_t const oi = monitor_store_index(m, p->at_turn, p->pid);
        if (oi >= 0) {
            if (ctx->mon && k < ctx->mon->num && oi < ctx->mon->caps[k]) {
                p_store(p, ctx->mon->cols[k], ctx->mon->caps[k], oi);
                rc = 0;
            } else {
                rc = -1;
            }
            if (rc != 0) p->state = 0;
        }
    }
    return rc;
}

/* ------------------------------------------------------- dispatcher */
/* track/track.h:209-585 with the default feature flags (BB4D/BB6D/SC
 * enabled, TriCub disabled, global aperture after every drift). */
static int dispatch(const lattice_t *L, prec *p, int64_t obj,
                    const track_ctx *ctx)
{
    uint64_t const t = obj_type(L, obj);
    int ret = ST_OK;
    switch (t) {
    case T_DRIFT:
    case T_DRIFT_EXACT: {
        double const len = obj_reals(L, obj)[0];
        ret = (t == T_DRIFT) ? m_drift(p, len) : m_drift_exact(p, len);
        if (g_ap_mode == 2 || (g_ap_mode == 1 && len >= g_ap_min_len)) {
            ret |= m_limit_global(p);
        }
        break;
    }
    case T_MULTIPOLE:
        ret = m_multipole(L, p, obj_words(L, obj));
        break;
    case T_RF_MULTIPOLE:
        ret = m_rf_multipole(L, p, obj_words(L, obj));
        break;
    case T_CAVITY:
        ret = m_cavity(p, obj_reals(L, obj));
        break;
    case T_XYSHIFT:
        ret = m_xyshift(p, obj_reals(L, obj));
        break;
    case T_SROTATION:
        ret = m_srotation(p, obj_reals(L, obj));
        break;
    case T_MONITOR:
        ret = m_monitor(L, p, obj, ctx);
        break;
    case T_LIMIT_RECT:
        ret = m_limit_rect(p, obj_reals(L, obj));
        break;
    case T_LIMIT_ELLIPSE:
        ret = m_limit_ellipse(p, obj_reals(L, obj));
        break;
    case T_LIMIT_RECT_ELLIPSE:
        ret = m_limit_rect_ellipse(p, obj_reals(L, obj));
        break;
    case T_DIPEDGE:
        ret = m_dipedge(p, obj_reals(L, obj));
        break;
    /* feature flags, track.h:421-575: a disabled map fails (the loop marks
     * the particle lost), a skipped one succeeds */
    case T_TRICUB:
        ret = g_flag_tricub == 2 ? m_tricub(L, p, obj_words(L, obj))
                                 : (g_flag_tricub == 1 ? ST_OK : ST_FAIL);
        break;
    case T_TRICUB_DATA:
        ret = g_flag_tricub != 0 ? ST_OK : ST_FAIL;
        break;
    case T_BB4D:
        ret = g_flag_bb4d == 2 ? m_bb4d(L, p, obj_words(L, obj))
                               : (g_flag_bb4d == 1 ? ST_OK : ST_FAIL);
        break;
    case T_BB6D:
        ret = g_flag_bb6d == 2 ? m_bb6d(L, p, obj_words(L, obj))
                               : (g_flag_bb6d == 1 ? ST_OK : ST_FAIL);
        break;
    case T_SC_COASTING:
        ret = g_flag_sc == 2 ? m_sc_coasting(p, obj_reals(L, obj))
                             : (g_flag_sc == 1 ? ST_OK : ST_FAIL);
        break;
    case T_SC_QGAUSS:
        ret = g_flag_sc == 2 ? m_sc_qgauss(p, obj_reals(L, obj))
                             : (g_flag_sc == 1 ? ST_OK : ST_FAIL);
        break;
    /* with space charge skipped or disabled the interpolated profile has no
     * case label (the preprocessor branch that starts in the q-Gaussian
     * case, track.h:537-575, encloses it): the default branch below */
    case T_SC_INTERPOL:
        if (g_flag_sc != 2) goto unknown;
        ret = m_sc_interpol(L, p, obj_words(L, obj));
        break;
    default:
    unknown:
        p->state = 0;
        ret = ST_FAIL;
    }
    return ret;
}

/* ------------------------------------------------------- tracking loops */
/* track/track.h:610-670 */
static int32_t until_one(const lattice_t *L, prec *p, int64_t until_turn,
                         const track_ctx *ctx)
{
    int32_t ok = (L->nobj > 0) ? ST_OK : ST_FAIL;
    int64_t const start = p->at_element;
    int cont = (ok == ST_OK) && (until_turn > p->at_turn) && (p->state == 1);
    while (cont) {
        int64_t e = 0;
        while (cont && e != L->nobj) {
            ok = dispatch(L, p, e++, ctx);
            cont = (ok == ST_OK) && (p->state == 1);
            if (cont) p->at_element++;
        }
        if (cont) {
            p->at_element = start;
            p->at_turn++;
            p->s = 0.0;
            cont = (p->at_turn < until_turn);
        } else {
            p->state = 0;
        }
    }
    return ok;
}

int32_t orc_track_until(const uint8_t *lattice, void *cols, int64_t n,
                        int64_t idx_begin, int64_t idx_end, int64_t until_turn,
                        const orc_monitor_outputs *mon)
{
    lattice_t L;
    track_ctx ctx = {mon};
    int32_t status = ST_OK;
    lat_open(&L, lattice);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) reduction(| : status)
#endif
    for (int64_t i = idx_begin; i < idx_end; i++) {
        prec p;
        p_load(&p, cols, n, i);
        status |= until_one(&L, &p, until_turn, &ctx);
        p_store(&p, cols, n, i);
    }
    return status;
}

/* track/track.h:779-822 */
int32_t orc_track_line(const uint8_t *lattice, void *cols, int64_t n,
                       int64_t idx_begin, int64_t idx_end, uint64_t line_begin,
                       uint64_t line_end, int finish_turn,
                       const orc_monitor_outputs *mon)
{
    lattice_t L;
    track_ctx ctx = {mon};
    int32_t status = ST_OK;
    lat_open(&L, lattice);
    for (int64_t i = idx_begin; i < idx_end; i++) {
        prec p;
        int ok = ST_OK;
        p_load(&p, cols, n, i);
        int64_t e = (int64_t)line_begin;
        int cont = (line_begin != line_end) && (p.state == 1);
        while (cont) {
            ok = dispatch(&L, &p, e, &ctx);
            cont = (ok == ST_OK) && (p.state == 1);
            if (cont) {
                p.at_element++;
                ++e;
                cont = (e != (int64_t)line_end);
            }
        }
        if (finish_turn && ok == ST_OK && p.state == 1) {
            p.at_element = 0;
            p.at_turn++;
            p.s = 0.0;
        }
        status |= ok;
        p_store(&p, cols, n, i);
    }
    return status;
}

/* output/elem_by_elem_config.h:667-763 */
int64_t orc_ebe_store_index(const orc_ebe_config *c, int64_t pid,
                            int64_t at_element, int64_t at_turn)
{
    int64_t out = -1;
    if ((c->min_particle_id <= pid) && (c->max_particle_id >= pid) &&
        (c->min_element_id <= at_element) && (c->max_element_id >= at_element) &&
        (c->min_turn <= at_turn) &&
        ((c->max_turn >= at_turn) || (c->is_rolling != 0))) {
        int64_t const poff = pid - c->min_particle_id;
        int64_t const eoff = at_element - c->min_element_id;
        int64_t const toff = at_turn - c->min_turn;
        int64_t const np = c->num_particles_to_store;
        int64_t const ne = c->num_elements_to_store;
        int64_t const nt = c->num_turns_to_store;
        int64_t cap = 0;
        if (c->order == 0) {
            out = toff * np * ne + eoff * np + poff;
            cap = np * ne * nt;
        } else {
            out = -1;
        }
        if ((out >= cap) && (cap > 0) && (c->is_rolling != 0)) {
            out = out % cap;
        }
    }
    return out;
}

/* track/track.h:672-777 */
int32_t orc_track_elem_by_elem(const uint8_t *lattice, void *cols, int64_t n,
                               int64_t idx_begin, int64_t idx_end,
                               const orc_ebe_config *cfg, void *out_cols,
                               int64_t out_n, int64_t until_turn,
                               const orc_monitor_outputs *mon)
{
    lattice_t L;
    track_ctx ctx = {mon};
    int32_t status = ST_OK;
    lat_open(&L, lattice);
    for (int64_t i = idx_begin; i < idx_end; i++) {
        prec p;
        int32_t ok = ST_OK;
        p_load(&p, cols, n, i);
        if (out_cols != NULL) {
            int64_t const pid = p.pid;
            int64_t const start = p.at_element;
            int64_t ae = start;
            int64_t at = p.at_turn;
            int cont = (L.nobj != 0) && (until_turn > at) && (at >= 0) &&
                       (start >= 0) && (pid >= 0);
            while (cont) {
                int64_t e = 0;
                while (cont && e != L.nobj) {
                    int64_t const oi = orc_ebe_store_index(cfg, pid, ae, at);
                    if (oi >= 0 && oi < out_n) {
                        p_store(&p, out_cols, out_n, oi);
                    }
                    ok = dispatch(&L, &p, e, &ctx);
                    cont = (ok == ST_OK) && (p.state == 1);
                    if (cont) {
                        ++e;
                        if (e != L.nobj) {
                            ++ae;
                            p.at_element++;
                        } else {
                            p.at_element = start;
                            p.s = 0.0;
                            p.at_turn++;
                            ++at;
                            ae = start;
                            cont = (at < until_turn);
                        }
                    }
                }
            }
        } else {
            ok = until_one(&L, &p, until_turn, &ctx);
        }
        status |= ok;
        p_store(&p, cols, n, i);
    }
    return status;
}

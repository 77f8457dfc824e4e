/*
 * marschner.c -- FP64 hair scattering lobes.  TEST INFRASTRUCTURE ONLY.
 *
 * The FP64 reference for shading error: the single-scattering lobes R, TT, TRT of a
 * dielectric cylinder (Marschner et al. 2003, "Light Scattering from Human
 * Hair Fibers"; d'Eon et al. 2011, "An Energy-Conserving Hair Reflectance
 * Model"; Chiang et al. 2016, "A Practical and Controllable Hair and Fur Model
 * for Production Path Tracing") with the azimuthal scattering integrated
 * exactly over the offset h, and the local back-scattering term of the dual
 * scattering approximation (Zinke et al. 2008) built from the same exact
 * lobes.  It follows shade.wesl's conventions so that the Karis-fit lobes of
 * shade.wesl:94-128 and the learned surrogate are measured against it on the same terms:
 *   S_p = M_p(theta_i + theta_o - alpha_p; beta_p) * N_p(phi; theta_d)
 * with shade.wesl's Gaussian longitudinal lobes (alpha = tilt, -tilt/2,
 * -3 tilt/2; beta = b_m, b_m/2, 2 b_m) and
 *   N_p(phi) = 1/2 Int_{-1}^{1} A_p(h) D(phi - Phi_p(h); beta_n) dh,
 *   Phi_p(h) = 2 p gamma_t - 2 gamma_i + p pi,  gamma_i = asin h,
 *   gamma_t = asin(h / eta'),  eta' = sqrt(eta^2 - sin^2 theta_d) / cos theta_d,
 *   A_0 = F,  A_1 = (1-F)^2 T,  A_2 = (1-F)^2 F T^2,
 *   F = dielectric Fresnel at cos(theta_d) cos(gamma_i),
 *   T = exp(-sigma_a 2 cos gamma_t / cos theta_t),  sin theta_t = sin theta_d / eta,
 * D a wrapped Gaussian of standard deviation beta_n.  The h integral is
 * taken over gamma_i = asin h (dh = cos gamma_i dgamma_i), which removes the
 * square-root behaviour of the integrand at h = +-1, with 64-point
 * Gauss-Legendre; it agrees with a 20001-point Simpson rule to ~3e-11
 * relative.  The azimuthal integrals of the dual-scattering terms use the
 * wrapped Gaussian's CDF, so they are exact in phi.
 *
 * Inputs of one evaluation (the surrogate's 10 inputs):
 *   sin theta_i, sin theta_o, cos phi, sin phi, sigma_a (rgb), beta_m,
 *   beta_n, eta; tilt is a parameter.
 * Output (12): R (rgb), TT (rgb), TRT (rgb), back-scattering B (rgb), where
 *   B = 2 A_back g(sigma_b; theta_i + theta_o - delta_b) / pi
 * with A_back, delta_b, sigma_b from Zinke Eqs. 13-17 as shade.wesl:175-189
 * evaluates them, at theta_d = theta_o (the specular cone, shade.wesl:444).
 */
#include <math.h>
#include <string.h>

#define M_PI 3.14159265358979323846

#define GL_N 64
static double g_gl_x[GL_N], g_gl_w[GL_N];
static int g_gl_ready = 0;

/* Gauss-Legendre nodes by Newton iteration on P_n, mapped to gamma_i. */
static void gl_init(void) {
    if (g_gl_ready) return;
    const int n = GL_N;
    for (int i = 0; i < n; ++i) {
        double x = cos(M_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = x;
            for (int k = 2; k <= n; ++k) {
                double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            double dp = n * (x * p1 - p0) / (x * x - 1.0);
            double dx = p1 / dp;
            x -= dx;
            if (fabs(dx) < 1e-16) break;
        }
        double p0 = 1.0, p1 = x;
        for (int k = 2; k <= n; ++k) {
            double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        double dp = n * (x * p1 - p0) / (x * x - 1.0);
        /* nodes and weights on gamma_i in [-pi/2, pi/2], Jacobian cos(gamma_i) folded in */
        g_gl_x[i] = 0.5 * M_PI * x;
        g_gl_w[i] = 0.5 * M_PI * 2.0 / ((1.0 - x * x) * dp * dp) * cos(g_gl_x[i]);
    }
    g_gl_ready = 1;
}

/* Unpolarised dielectric Fresnel reflectance at incidence cosine c. */
static double fresnel_exact(double c, double eta) {
    c = fmin(fmax(c, 0.0), 1.0);
    double s2 = 1.0 - c * c;
    double st2 = s2 / (eta * eta);
    if (st2 >= 1.0) return 1.0;
    double ct = sqrt(1.0 - st2);
    double rs = (c - eta * ct) / (c + eta * ct);
    double rp = (eta * c - ct) / (eta * c + ct);
    return 0.5 * (rs * rs + rp * rp);
}

static double gauss_pdf(double x, double s) { return exp(-0.5 * x * x / (s * s)) / (sqrt(2.0 * M_PI) * s); }

/* Wrapped Gaussian density on the circle. */
static double wrapped_pdf(double x, double s) {
    x = remainder(x, 2.0 * M_PI);
    double d = 0.0;
    for (int k = -3; k <= 3; ++k) d += gauss_pdf(x + 2.0 * M_PI * k, s);
    return d;
}

/* Integral of the wrapped Gaussian (centre c) over [a, b], b - a <= 2 pi. */
static double wrapped_mass(double a, double b, double c, double s) {
    double m = 0.0;
    double r = 1.0 / (s * sqrt(2.0));
    for (int k = -4; k <= 4; ++k) {
        double cc = c + 2.0 * M_PI * k;
        m += 0.5 * (erf((b - cc) * r) - erf((a - cc) * r));
    }
    return m;
}

/* shade.wesl:51-54 in FP64 */
static double gauss3_1(double b, double x) {
    double bb = fmax(b, 1e-3);
    return exp(-0.5 * x * x / (bb * bb)) / (sqrt(2.0 * M_PI) * bb);
}

typedef struct {
    double a[3][3];  /* A_p(h) per colour at one node: [lobe][rgb] */
    double phi[3];   /* Phi_p(h) */
} lobe_node;

/* Attenuation and exit azimuth of every lobe at the GL nodes. */
static void lobe_nodes(double cos_td, double sin_td, const double sigma_a[3], double eta, lobe_node* out) {
    double eta_p = sqrt(eta * eta - sin_td * sin_td) / cos_td;
    double sin_tt = sin_td / eta;
    double cos_tt = sqrt(1.0 - sin_tt * sin_tt);
    for (int i = 0; i < GL_N; ++i) {
        double gi = g_gl_x[i];
        double h = sin(gi);
        double gt = asin(h / eta_p);
        double f = fresnel_exact(cos_td * cos(gi), eta);
        double path = 2.0 * cos(gt) / cos_tt;
        for (int c = 0; c < 3; ++c) {
            double t = exp(-sigma_a[c] * path);
            out[i].a[0][c] = f;
            out[i].a[1][c] = (1.0 - f) * (1.0 - f) * t;
            out[i].a[2][c] = (1.0 - f) * (1.0 - f) * f * t * t;
        }
        for (int p = 0; p < 3; ++p) out[i].phi[p] = 2.0 * p * gt - 2.0 * gi + p * M_PI;
    }
}

void oracle_marschner_lobes(const double in[10], double tilt, double out[12]) {
    gl_init();
    static __thread lobe_node nodes[GL_N];
    double sin_i = fmin(fmax(in[0], -1.0), 1.0), sin_o = fmin(fmax(in[1], -1.0), 1.0);
    double phi = atan2(in[3], in[2]);
    double sigma_a[3] = {in[4], in[5], in[6]};
    double beta_m = in[7], beta_n = in[8], eta = in[9];
    double th_i = asin(sin_i), th_o = asin(sin_o);
    double th_h = th_i + th_o;
    double alpha[3] = {tilt, -0.5 * tilt, -1.5 * tilt};
    double beta[3] = {beta_m, 0.5 * beta_m, 2.0 * beta_m};

    /* single scattering at theta_d = (theta_o - theta_i) / 2 */
    double td = 0.5 * (th_o - th_i);
    double cos_td = fmax(cos(td), 1e-3), sin_td = sin(td);
    lobe_nodes(cos_td, sin_td, sigma_a, eta, nodes);
    for (int p = 0; p < 3; ++p) {
        double m = gauss3_1(beta[p], th_h - alpha[p]);
        for (int c = 0; c < 3; ++c) {
            double n = 0.0;
            for (int i = 0; i < GL_N; ++i) n += g_gl_w[i] * nodes[i].a[p][c] * wrapped_pdf(phi - nodes[i].phi[p], beta_n);
            out[3 * p + c] = m * 0.5 * n;
        }
    }

    /* dual scattering at the specular cone, theta_d = theta_o (shade.wesl:444) */
    double cos_to = fmax(sqrt(fmax(1.0 - sin_o * sin_o, 1e-6)), 1e-3);
    lobe_nodes(cos_to, sqrt(fmax(0.0, 1.0 - cos_to * cos_to)), sigma_a, eta, nodes);
    double fwd[3][3], back[3][3];
    for (int p = 0; p < 3; ++p) {
        for (int c = 0; c < 3; ++c) {
            double f = 0.0, b = 0.0;
            for (int i = 0; i < GL_N; ++i) {
                double w = g_gl_w[i] * nodes[i].a[p][c];
                /* both mirrored halves: back |phi| < pi/2, forward pi/2 < |phi| < pi */
                b += w * wrapped_mass(-0.5 * M_PI, 0.5 * M_PI, nodes[i].phi[p], beta_n);
                f += w * wrapped_mass(0.5 * M_PI, 1.5 * M_PI, nodes[i].phi[p], beta_n);
            }
            fwd[p][c] = 0.5 * f;
            back[p][c] = 0.5 * b;
        }
    }
    for (int c = 0; c < 3; ++c) {
        double a_f = fmin(fwd[0][c] + fwd[1][c] + fwd[2][c], 0.95);
        double a_b = back[0][c] + back[1][c] + back[2][c];
        double b2[3] = {beta[0] * beta[0], beta[1] * beta[1], beta[2] * beta[2]};
        double tf = fmax(a_f, 1e-5), tb = fmax(a_b, 1e-5);
        double beta_f2 = (fwd[0][c] * b2[0] + fwd[1][c] * b2[1] + fwd[2][c] * b2[2]) / tf;
        double alpha_b = (back[0][c] * alpha[0] + back[1][c] * alpha[1] + back[2][c] * alpha[2]) / tb;
        double beta_b2 = (back[0][c] * b2[0] + back[1][c] * b2[1] + back[2][c] * b2[2]) / tb;
        double af2 = a_f * a_f, rest = 1.0 - af2, ab2 = a_b * a_b, ab3 = ab2 * a_b;
        double a_back = a_b * af2 / rest + ab3 * af2 / (rest * rest * rest);
        double delta_b = alpha_b * (1.0 - 2.0 * ab2 / (rest * rest)) +
                         alpha_b * (2.0 * rest * rest + 4.0 * af2 * ab2) / (rest * rest * rest);
        double beta_f = sqrt(beta_f2), beta_b = sqrt(beta_b2);
        double sigma_b = (1.0 + 0.7 * af2) *
                         (a_b * sqrt(2.0 * beta_f2 + beta_b2) + ab3 * sqrt(2.0 * beta_f2 + 3.0 * beta_b2)) /
                         fmax(a_b + ab3 * (2.0 * beta_f + 3.0 * beta_b), 1e-5);
        out[9 + c] = 2.0 * a_back * gauss3_1(sigma_b, th_h - delta_b) / M_PI;
    }
}

/* The same 12 outputs from shade.wesl's Karis fits (azimuthal :94-116, lobe
 * shape :124-128, dual_scatter :153-190) in FP64, for the error comparison.
 * beta_n has no counterpart in the fits. */
static double fresnel_schlick(double c, double eta) {
    double r0 = (1.0 - eta) / (1.0 + eta), f0 = r0 * r0;
    return f0 + (1.0 - f0) * pow(1.0 - fmin(fmax(c, 0.0), 1.0), 5.0);
}

static void karis_azimuthal(double ctd, double cphi, const double sa[3], double eta, double out[3][3]) {
    double chp = sqrt(fmin(fmax(0.5 + 0.5 * cphi, 0.0), 1.0));
    double n_r = 0.25 * chp * fresnel_schlick(ctd * chp, eta);
    double e = 1.19 / ctd + 0.36 * ctd;
    double a = 1.0 / e;
    double h = chp * (1.0 + a * (0.6 - 0.8 * cphi));
    double f_tt = fresnel_schlick(ctd * sqrt(fmin(fmax(1.0 - h * h, 0.0), 1.0)), eta);
    double f_trt = fresnel_schlick(ctd * 0.5, eta);
    for (int c = 0; c < 3; ++c) {
        double t_tt = exp(-sa[c] * 2.0 * sqrt(fmin(fmax(1.0 - h * h * a * a, 0.0), 1.0)) / ctd);
        double t_trt = exp(-sa[c] * 3.2 / ctd);
        out[0][c] = n_r;
        out[1][c] = exp(-3.65 * cphi - 3.98) * (1.0 - f_tt) * (1.0 - f_tt) * t_tt;
        out[2][c] = exp(17.0 * cphi - 16.78) * (1.0 - f_trt) * (1.0 - f_trt) * f_trt * t_trt;
    }
}

void oracle_karis_lobes(const double in[10], double tilt, double out[12]) {
    double sin_i = fmin(fmax(in[0], -1.0), 1.0), sin_o = fmin(fmax(in[1], -1.0), 1.0);
    double cphi = fmin(fmax(in[2], -1.0), 1.0);
    double sa[3] = {in[4], in[5], in[6]};
    double beta_m = in[7], eta = in[9];
    double th_i = asin(sin_i), th_o = asin(sin_o), th_h = th_i + th_o;
    double alpha[3] = {tilt, -0.5 * tilt, -1.5 * tilt};
    double beta[3] = {beta_m, 0.5 * beta_m, 2.0 * beta_m};
    double ctd = fmax(cos(0.5 * fabs(th_i - th_o)), 1e-3);
    double n[3][3];
    karis_azimuthal(ctd, cphi, sa, eta, n);
    for (int p = 0; p < 3; ++p) {
        double m = gauss3_1(beta[p], th_h - alpha[p]);
        for (int c = 0; c < 3; ++c) out[3 * p + c] = m * n[p][c];
    }
    double cto = sqrt(fmax(1.0 - sin_o * sin_o, 1e-6));
    double fwd[3][3] = {{0}}, back[3][3] = {{0}};
    for (int i = 0; i < 8; ++i) {
        double u = (i + 0.5) / 8.0;
        double b[3][3], f[3][3];
        karis_azimuthal(cto, cos(u * 0.5 * M_PI), sa, eta, b);
        karis_azimuthal(cto, cos((1.0 + u) * 0.5 * M_PI), sa, eta, f);
        for (int p = 0; p < 3; ++p)
            for (int c = 0; c < 3; ++c) {
                back[p][c] += b[p][c] * (M_PI / 8.0);
                fwd[p][c] += f[p][c] * (M_PI / 8.0);
            }
    }
    for (int c = 0; c < 3; ++c) {
        double a_f = fmin(fwd[0][c] + fwd[1][c] + fwd[2][c], 0.95);
        double a_b = back[0][c] + back[1][c] + back[2][c];
        double b2[3] = {beta[0] * beta[0], beta[1] * beta[1], beta[2] * beta[2]};
        double tf = fmax(a_f, 1e-5), tb = fmax(a_b, 1e-5);
        double beta_f2 = (fwd[0][c] * b2[0] + fwd[1][c] * b2[1] + fwd[2][c] * b2[2]) / tf;
        double alpha_b = (back[0][c] * alpha[0] + back[1][c] * alpha[1] + back[2][c] * alpha[2]) / tb;
        double beta_b2 = (back[0][c] * b2[0] + back[1][c] * b2[1] + back[2][c] * b2[2]) / tb;
        double af2 = a_f * a_f, rest = 1.0 - af2, ab2 = a_b * a_b, ab3 = ab2 * a_b;
        double a_back = a_b * af2 / rest + ab3 * af2 / (rest * rest * rest);
        double delta_b = alpha_b * (1.0 - 2.0 * ab2 / (rest * rest)) +
                         alpha_b * (2.0 * rest * rest + 4.0 * af2 * ab2) / (rest * rest * rest);
        double beta_f = sqrt(beta_f2), beta_b = sqrt(beta_b2);
        double sigma_b = (1.0 + 0.7 * af2) *
                         (a_b * sqrt(2.0 * beta_f2 + beta_b2) + ab3 * sqrt(2.0 * beta_f2 + 3.0 * beta_b2)) /
                         fmax(a_b + ab3 * (2.0 * beta_f + 3.0 * beta_b), 1e-5);
        out[9 + c] = 2.0 * a_back * gauss3_1(sigma_b, th_h - delta_b) / M_PI;
    }
}

/* Batch evaluation for the tests: in[n*10] -> out[n*12]; model 0 FP64
 * Marschner, 1 Karis fits. */
void oracle_lobes_batch(int model, const double* in, unsigned n, double tilt, double* out) {
    gl_init();
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < (long)n; ++i) {
        if (model == 0) oracle_marschner_lobes(in + 10 * i, tilt, out + 12 * i);
        else oracle_karis_lobes(in + 10 * i, tilt, out + 12 * i);
    }
}

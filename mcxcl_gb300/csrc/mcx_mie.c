/*
 * mcx_mie.c -- Mie scattering of a homogeneous sphere for the polarised
 * transport: the Mueller-matrix elements S11, S12, S33, S34 at 181 polar
 * angles, the scattering efficiency and the anisotropy, as the reference's
 * mcx_prep_polarized needs them (src/mcx_utils.c:1483-1519, which calls its
 * Mie routine in src/mcx_mie.cpp:91).
 *
 * The series follows Bohren & Huffman, "Absorption and Scattering of Light by
 * Small Particles" (Wiley, 1983): the coefficients a_n, b_n from the
 * logarithmic derivative D_n(mx) of the interior field (downward recurrence,
 * eq. 4.89) and the Riccati-Bessel functions psi_n, xi_n of the size
 * parameter x (upward recurrence), truncated after x + 4 x^(1/3) + 2 terms
 * (Wiscombe's criterion); the amplitude functions
 *   S1 = sum (2n+1)/(n(n+1)) (a_n pi_n + b_n tau_n),
 *   S2 = sum (2n+1)/(n(n+1)) (a_n tau_n + b_n pi_n)
 * with the angular functions pi_n, tau_n from their recurrences (4.47);
 *   Q_sca = 2/x^2 sum (2n+1)(|a_n|^2 + |b_n|^2),
 *   g Q_sca = 4/x^2 [sum n(n+2)/(n+1) Re(a_n a*_{n+1} + b_n b*_{n+1})
 *                  + sum (2n+1)/(n(n+1)) Re(a_n b*_n)]       (4.62);
 * and S11 = (|S2|^2 + |S1|^2)/2, S12 = (|S2|^2 - |S1|^2)/2,
 * S33 = Re(S1* S2), S34 = Im(S1* S2) (4.77).  The reference's amplitude
 * functions are the complex conjugates of these (the opposite sign of the
 * time factor), which flips the sign of S34 only: S34 is stored as
 * Im(S1 S2*) to match.  The relative refractive index is real, as the
 * reference's input (particle over background index).
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>

#include "../../include/mcx_gb300.h"

#define MIE_NANGLES 181

int mcx_mie(double x, double mrel, float* smatrix, double* qsca, double* g) {
    if (!(x > 0.0) || !(mrel > 0.0) || !smatrix || !qsca || !g) {
        return -1;
    }
    const long nstop = (long)(x + 4.0 * cbrt(x) + 2.0);
    const double mx = mrel * x;
    const long nmx = (long)((nstop > fabs(mx) ? nstop : fabs(mx)) + 16);
    double* D = (double*)calloc((size_t)nmx + 1, sizeof(double));
    double complex* S1 = (double complex*)calloc(MIE_NANGLES, sizeof(double complex));
    double complex* S2 = (double complex*)calloc(MIE_NANGLES, sizeof(double complex));
    double* mu = (double*)malloc(sizeof(double) * MIE_NANGLES);
    double* pi0 = (double*)calloc(MIE_NANGLES, sizeof(double));
    double* pi1 = (double*)malloc(sizeof(double) * MIE_NANGLES);
    if (!D || !S1 || !S2 || !mu || !pi0 || !pi1) {
        free(D), free(S1), free(S2), free(mu), free(pi0), free(pi1);
        return -2;
    }
    for (int j = 0; j < MIE_NANGLES; j++) {
        /* the reference's angles: a float pi, the cosine in double (mcx_utils.c:1486-1488) */
        mu[j] = cos((double)(3.1415926535897932f * j / (MIE_NANGLES - 1)));
        pi1[j] = 1.0;
    }
    /* D_{n-1} = n/(mx) - 1/(D_n + n/(mx)), started at zero well above nstop */
    for (long n = nmx; n >= 2; n--) {
        const double r = (double)n / mx;
        D[n - 1] = r - 1.0 / (D[n] + r);
    }
    double psi0 = cos(x), psi1 = sin(x);
    double chi0 = -sin(x), chi1 = cos(x);
    double complex xi1 = psi1 - I * chi1;
    double complex an_prev = 0.0, bn_prev = 0.0;
    double sq = 0.0, sg = 0.0;
    for (long n = 1; n <= nstop; n++) {
        const double dn = (double)n;
        const double fn = (2.0 * dn + 1.0) / (dn * (dn + 1.0));
        const double psi = (2.0 * dn - 1.0) * psi1 / x - psi0;
        const double chi = (2.0 * dn - 1.0) * chi1 / x - chi0;
        const double complex xi = psi - I * chi;
        const double da = D[n] / mrel + dn / x;
        const double db = mrel * D[n] + dn / x;
        const double complex an = (da * psi - psi1) / (da * xi - xi1);
        const double complex bn = (db * psi - psi1) / (db * xi - xi1);
        sq += (2.0 * dn + 1.0) * (creal(an) * creal(an) + cimag(an) * cimag(an) +
                                   creal(bn) * creal(bn) + cimag(bn) * cimag(bn));
        if (n > 1) {
            const double dm = dn - 1.0;
            sg += dm * (dm + 2.0) / (dm + 1.0) * creal(an_prev * conj(an) + bn_prev * conj(bn));
        }
        sg += fn * creal(an * conj(bn));
        for (int j = 0; j < MIE_NANGLES; j++) {
            const double tau = dn * mu[j] * pi1[j] - (dn + 1.0) * pi0[j];
            S1[j] += fn * (an * pi1[j] + bn * tau);
            S2[j] += fn * (an * tau + bn * pi1[j]);
            const double pnext = ((2.0 * dn + 1.0) * mu[j] * pi1[j] - (dn + 1.0) * pi0[j]) / dn;
            pi0[j] = pi1[j];
            pi1[j] = pnext;
        }
        an_prev = an;
        bn_prev = bn;
        psi0 = psi1;
        psi1 = psi;
        chi0 = chi1;
        chi1 = chi;
        xi1 = psi1 - I * chi1;
    }
    *qsca = 2.0 / (x * x) * sq;
    *g = 4.0 / (x * x) * sg / *qsca;
    for (int j = 0; j < MIE_NANGLES; j++) {
        const double a1 = creal(S1[j]) * creal(S1[j]) + cimag(S1[j]) * cimag(S1[j]);
        const double a2 = creal(S2[j]) * creal(S2[j]) + cimag(S2[j]) * cimag(S2[j]);
        const double complex c = S1[j] * conj(S2[j]);
        smatrix[4 * j] = (float)(0.5 * a2 + 0.5 * a1);
        smatrix[4 * j + 1] = (float)(0.5 * a2 - 0.5 * a1);
        smatrix[4 * j + 2] = (float)creal(c);
        smatrix[4 * j + 3] = (float)cimag(c);
    }
    free(D), free(S1), free(S2), free(mu), free(pi0), free(pi1);
    return 0;
}

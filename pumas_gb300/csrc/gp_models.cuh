/*
 * gp_models.cuh -- the non-default DCS models of PUMAS
 * (struct pumas_physics_settings, pumas.h:742-771), as code that compiles
 * both as C (host) and as CUDA (the engine):
 *
 *   bremsstrahlung  KKP (Kelner, Kokoulin & Petrukhin), ABB (Andreev,
 *                   Bezrukov & Bugaev);
 *   pair production KKP;
 *   photonuclear    BM (Butkevich & Mikheyev, with its doubly differential
 *                   cross section for the polar angle sampler), BBKS
 *                   (Bezrukov & Bugaev with the Kokoulin photon-nucleon
 *                   cross section and the Bugaev-Montaruli-Shlepin-Sokalski
 *                   hard component).
 *
 * Each function cites the reference lines it follows; their arithmetic is
 * kept in the reference's order so that the host build reproduces the
 * reference bit for bit (the golden cases of the tests check it). The device
 * build calls the CUDA math library, within an ulp of the host's.
 * Element data that the callers hold (the radiation logarithm) and the
 * Gauss-Legendre nodes are passed as arguments.
 */
#ifndef GP_MODELS_CUH
#define GP_MODELS_CUH

#include <math.h>

#ifdef __CUDACC__
/* Out of line on the device: the default models' kernels keep their
 * registers. */
#define GPM_HD static __host__ __device__ __noinline__
#ifdef __CUDA_ARCH__
#define GPM_TABLE static __device__ const
#else
#define GPM_TABLE static const
#endif
#else
#define GPM_HD static inline
#define GPM_TABLE static const
#endif

/* The reference's constants (pumas.c:125-170, 13827-13830). */
#define GPM_ALPHA_EM 7.2973525693E-03
#define GPM_HBAR_C 1.973269804E-16
#define GPM_ELECTRON_MASS 0.510998910E-03
#define GPM_PROTON_MASS 0.938272
#define GPM_NEUTRON_MASS 0.939565
#define GPM_PION_MASS 0.13957018
#define GPM_MUON_MASS 0.10565839
#define GPM_TAU_MASS 1.77682
#define GPM_PI 3.14159265358979323846
#define GPM_SQRTE 1.648721270700128
#define GPM_ME_MEV 0.5109989461
#define GPM_RE_CM 2.8179403227E-13
#define GPM_MMU_MEV 105.6583745

/* dcs_bremsstrahlung_KKP (pumas.c:13759-13810). */
GPM_HD double gpm_bremsstrahlung_KKP(
    double Z, double A, double mu, double K, double q, double rad_log)
{
        if ((Z <= 0) || (A <= 0) || (mu <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        const double Z13 = pow(Z, 1. / 3.);
        const double sqrte = 1.648721271;
        if (q >= K + mu * (1. - 0.75 * sqrte * Z13)) return 0.;
        const double me = GPM_ELECTRON_MASS;
        const double phie_factor = mu / (me * me * sqrte);
        const double rem = 5.63588E-13 * me / mu;
        const double BZ_n = rad_log / Z13;
        const double BZ_e = (Z == 1.) ? 446. : 1429. / (Z13 * Z13);
        const double D_n = 1.54 * pow(A, 0.27);
        const double E = K + mu;
        const double dcs_factor = 7.297182E-07 * rem * rem * Z / E;
        const double delta_factor = 0.5 * mu * mu / E;
        const double qe_max = E / (1. + 0.5 * mu * mu / (me * E));
        const double nu = q / E;
        const double delta = delta_factor * nu / (1. - nu);
        const double muD_factor = mu + delta * (D_n * sqrte - 2.);
        /* Nuclear, inelastic nuclear and electron screening terms. */
        double Phi_n = log(BZ_n * muD_factor /
            (D_n * (me + delta * sqrte * BZ_n)));
        if (Phi_n < 0.) Phi_n = 0.;
        double Phi_x = 0.;
        if (Z >= 2) {
                Phi_x = log(mu * D_n / muD_factor);
                if (Phi_x < 0.) Phi_x = 0.;
        }
        double Phi_e = 0.;
        if (q < qe_max) {
                Phi_e = log(BZ_e * mu /
                    ((1. + delta * phie_factor) * (me + delta * sqrte * BZ_e)));
                if (Phi_e < 0.) Phi_e = 0.;
        }
        const double dcs = dcs_factor * (Z * Phi_n + Phi_x + Phi_e) *
            (4. / 3. * (1. / nu - 1.) + nu);
        return (dcs < 0.) ? 0. : dcs;
}

/* dcs_bremsstrahlung_ABB (pumas.c:13824-13905), in MeV internally, with the
 * constants of pumas.c:13827-13830. */
GPM_HD double gpm_bremsstrahlung_ABB(
    double Z, double A, double m, double K, double q)
{
        if ((Z <= 0) || (A <= 0) || (m <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        const double Z13 = pow(Z, 1. / 3.);
        if (q >= K + m * (1. - 0.75 * GPM_SQRTE * Z13)) return 0.;
        const double energy = (K + m) * 1E+03;
        const double v = q * 1E+03 / energy;
        m *= 1E+03;
        /* Screening constants and the nuclear form factor terms (eq. 2.18,
         * 2.19, 2.30). */
        const double Z3 = 1. / Z13;
        const double a1 = 184.15 * Z3 / (GPM_SQRTE * GPM_ME_MEV);
        const double a2 = 1194 * Z3 * Z3 / (GPM_SQRTE * GPM_ME_MEV);
        const double qc = 1.9 * GPM_MMU_MEV * Z3;
        double aux = 2 * m / qc;
        const double zeta = sqrt(1 + aux * aux);
        const double delta = m * m * v / (2 * energy * (1 - v));
        const double x1 = a1 * delta;
        const double x2 = a2 * delta;
        double aux1, aux2, d1, d2;
        if (Z == 1) {
                d1 = 0;
                d2 = 0;
        } else {
                aux1 = log(m / qc);
                aux2 = 0.5 * zeta * log((zeta + 1) / (zeta - 1));
                d1 = aux1 + aux2;
                d2 = aux1 + 0.5 * ((3 - zeta * zeta) * aux2 + aux * aux);
        }
        /* Atomic screening functions (eq. 2.20, 2.21). */
        aux = m * a1;
        aux1 = log(aux * aux / (1 + x1 * x1));
        aux = m * a2;
        aux2 = log(aux * aux / (1 + x2 * x2));
        double psi1 = 0.5 * ((1 + aux1) + (1 + aux2) / Z);
        double psi2 = 0.5 * ((2. / 3 + aux1) + (2. / 3 + aux2) / Z);
        aux1 = x1 * atan(1 / x1);
        aux2 = x2 * atan(1 / x2);
        psi1 -= aux1 + aux2 / Z;
        aux = x1 * x1;
        psi2 += 2 * aux * (1 - aux1 + 0.75 * log(aux / (1 + aux)));
        aux = x2 * x2;
        psi2 += 2 * aux * (1 - aux2 + 0.75 * log(aux / (1 + aux))) / Z;
        psi1 -= d1;
        psi2 -= d2;
        const double result =
            (2 - 2 * v + v * v) * psi1 - (2. / 3) * (1 - v) * psi2;
        if (result < 0) return 0;
        aux = 2 * (GPM_ME_MEV / m) * GPM_RE_CM * Z;
        return aux * aux * (GPM_ALPHA_EM / q) * result * 1E-04;
}

/* dcs_pair_production_KKP (pumas.c:14255-14373): integral over
 * t = ln(1 - rho) with the 12 point Gauss-Legendre nodes, electron and muon
 * terms, and the atomic electrons' form factor. */
GPM_HD double gpm_pair_production_KKP(double Z, double A_,
    double mass, double K, double q, double rad_log, const double * xGQ,
    const double * wGQ)
{
        if ((Z <= 0) || (A_ <= 0) || (mass <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        {
                /* dcs_pair_production_range (pumas.c:14230-14240). */
                const double qmax = K + mass * (1. - 0.75 * 1.6487212707 *
                                                   pow(Z, 1. / 3.));
                if ((q < 4. * GPM_ELECTRON_MASS) || (q > qmax)) return 0.;
        }
        const double nu = q / (K + mass);
        const double r = mass / GPM_ELECTRON_MASS;
        const double beta = 0.5 * nu * nu / (1. - nu);
        const double xi_factor = 0.5 * r * r * beta;
        const double A = rad_log;
        const double Z13 = pow(Z, 1. / 3.);
        const double AZ13 = A / Z13;
        const double sqrte = 1.6487212707;
        const double cL = 2. * sqrte * GPM_ELECTRON_MASS * AZ13;
        const double cLe = 2.25 * Z13 * Z13 / (r * r);
        const double gamma = 1. + K / mass;
        const double x0 = 4. * GPM_ELECTRON_MASS / q;
        const double x1 = 6. / (gamma * (gamma - q / mass));
        const double argmin =
            (x0 + 2. * (1. - x0) * x1) / (1. + (1. - x1) * sqrt(1. - x0));
        if ((argmin >= 1.) || (argmin <= 0.)) return 0.;
        const double tmin = log(argmin);
        double I = 0.;
        int i;
        for (i = 0; i < 12; i++) {
                const double eps = exp(xGQ[i] * tmin);
                const double rho = 1. - eps;
                const double rho2 = rho * rho;
                const double rho21 = eps * (2. - eps);
                const double xi = xi_factor * rho21;
                const double xi_i = 1. / xi;
                double Be;
                if (xi >= 1E+03)
                        Be = 0.5 * xi_i *
                            ((3 - rho2) + 2. * beta * (1. + rho2));
                else
                        Be = ((2. + rho2) * (1. + beta) + xi * (3. + rho2)) *
                                log(1. + xi_i) +
                            (rho21 - beta) / (1. + xi) - 3. - rho2;
                const double Ye = (5. - rho2 + 4. * beta * (1. + rho2)) /
                    (2. * (1. + 3. * beta) * log(3. + xi_i) - rho2 -
                        2. * beta * (2. - rho2));
                const double xe = (1. + xi) * (1. + Ye);
                const double cLi = cL / rho21;
                const double Le = log(AZ13 * sqrt(xe) * q / (q + cLi * xe)) -
                    0.5 * log(1. + cLe * xe);
                double Phi_e = Be * Le;
                if (Phi_e < 0.) Phi_e = 0.;
                double Bmu;
                if (xi <= 1E-03)
                        Bmu = 0.5 * xi * (5. - rho2 + beta * (3. + rho2));
                else
                        Bmu = ((1. + rho2) * (1. + 1.5 * beta) -
                                  xi_i * (1. + 2. * beta) * rho21) *
                                log(1. + xi) +
                            xi * (rho21 - beta) / (1. + xi) +
                            (1. + 2. * beta) * rho21;
                const double Ymu = (4. + rho2 + 3. * beta * (1. + rho2)) /
                    ((1. + rho2) * (1.5 + 2. * beta) * log(3. + xi) + 1. -
                        1.5 * rho2);
                const double xmu = (1. + xi) * (1. + Ymu);
                const double Lmu =
                    log(r * AZ13 * q / (1.5 * Z13 * (q + cLi * xmu)));
                double Phi_mu = Bmu * Lmu;
                if (Phi_mu < 0.) Phi_mu = 0.;
                I -= (Phi_e + Phi_mu / (r * r)) * (1. - rho) * wGQ[i] *
                    tmin;
        }
        double zeta = 0.;
        if (gamma > 35.) {
                double gamma1, gamma2;
                if (Z == 1.) {
                        gamma1 = 4.4E-05;
                        gamma2 = 4.8E-05;
                } else {
                        gamma1 = 1.95E-05;
                        gamma2 = 5.30E-05;
                }
                zeta = 0.073 * log(gamma / (1. + gamma1 * gamma * Z13 * Z13)) -
                    0.26;
                if (zeta <= 0.)
                        zeta = 0.;
                else
                        zeta /= 0.058 * log(gamma /
                                                (1. + gamma2 * gamma * Z13)) -
                            0.14;
        }
        const double E = K + mass;
        const double dcs =
            1.794664E-34 * Z * (Z + zeta) * (E - q) * I / (q * E);
        return (dcs < 0.) ? 0. : dcs;
}

/* Wood-Saxon factor of Butkevich & Mikheyev (dcs_wood_saxon,
 * pumas.c:14732-14748). */
GPM_HD double gpm_wood_saxon(double Z, double A)
{
        if (Z == 1) return 0.;
        double r0 = pow(A, 1. / 3.);
        r0 = 1.12 * r0 - 0.86 / r0;
        const double a = 0.54;
        const double zeta3 = 1.202056903159594;
        const double V = a * (r0 * r0 * log(2.) + a * r0 * GPM_PI * GPM_PI / 6. +
                                 a * a * 1.5 * zeta3);
        return 1. - 4. * GPM_PI * 0.17 * V / A;
}

/* Shadowing factor of Butkevich & Mikheyev
 * (dcs_photonuclear_shadowing_BM, pumas.c:14768-14827). */
GPM_HD double gpm_photonuclear_shadowing_BM(
    double Z, double A, double x, double q)
{
        if (Z == 1.) return 1;
        if (x > 0.3) {
                const double Mb = 0.437;
                const double la = 0.5;
                const double x2 = 0.278;
                const double au = 1. / (1. - x);
                const double ac = 1. / (1. - x2);
                const double MPI = 0.13957018;
                const double M =
                    ((A - Z) * GPM_NEUTRON_MASS + Z * GPM_PROTON_MASS) / A;
                const double Aosc = (1. - la * x) *
                    (au - ac - MPI / M * (au * au - ac * ac));
                return 1. - Mb * gpm_wood_saxon(Z, A) * Aosc;
        } else {
                const double M1 = 0.129;
                const double M2 = 0.456;
                const double M3 = 0.553;
                const double ws = gpm_wood_saxon(Z, A);
                const double m1 = M1 * ws;
                const double m2 = M2 * ws;
                const double m3 = M3 * ws;
                const double sgn = 112.2 *
                    (0.609 * pow(q, 0.0988) + 1.037 * pow(q, -0.5944));
                const double tmp = 0.00282 * pow(A, 1. / 3.) * sgn;
                double G = (3. / tmp) *
                    (0.5 + ((1. + tmp) * exp(-tmp) - 1.) / (tmp * tmp));
                G = 0.75 * G + 0.25;
                const double x0 = pow(G / (1. + m2), 1. / m1);
                if (x >= x0)
                        return pow(x, m1) * (1 + m2) * (1 - m3 * x);
                else
                        return G;
        }
}

/* Nuclear structure function F2 of Butkevich & Mikheyev
 * (dcs_photonuclear_f2a_BM, pumas.c:14837-14907): singlet (sea quarks and
 * gluons) and valence terms of the proton and of the neutron. */
GPM_HD double gpm_photonuclear_f2a_BM(
    double Z, double A, double shadowing, double x, double Q2)
{
        Q2 *= 1E+06;
        const double a = 0.2513E+06;
        const double b = 0.6186E+06;
        const double c = 3.0292E+06;
        const double d = 1.4817E+06;
        const double intercept_pomeron = 0.0988;
        const double intercept_reggeon = 0.4056;
        const double tau = 1.8152;
        const double A_s = 0.12;
        const double B_up = 1.2437;
        const double B_down = 0.1853;
        const double n = 1.5 * (1. + Q2 / (Q2 + c));
        const double dl = intercept_pomeron * (1. + 2. * Q2 / (Q2 + d));
        double aux = A_s * pow(x, -dl) * pow(Q2 / (Q2 + a), 1. + dl);
        const double F_proton_singlet = aux * pow(1. - x, n + 4.);
        const double F_neutron_singlet = aux * pow(1. - x, n + tau);
        aux = pow(x, 1. - intercept_reggeon) * pow(1. - x, n) *
            pow(Q2 / (Q2 + b), intercept_reggeon);
        const double Up_valence = B_up * aux;
        const double Down_valence = B_down * aux * (1. - x);
        const double F_proton_non_singlet = Up_valence + Down_valence;
        const double F_neutron_non_singlet =
            Up_valence / 4. + Down_valence * 4.;
        const double structure_function_proton =
            F_proton_singlet + F_proton_non_singlet;
        const double structure_function_neutron =
            F_neutron_singlet + F_neutron_non_singlet;
        return shadowing * (Z * structure_function_proton +
                               (A - Z) * structure_function_neutron);
}

/* dcs_photonuclear_d2_BM (pumas.c:14963-14981). */
GPM_HD double gpm_photonuclear_d2_BM(
    double Z, double A, double ml, double K, double q, double Q2)
{
        const double cf = 4 * GPM_PI * GPM_ALPHA_EM * GPM_ALPHA_EM * GPM_HBAR_C * GPM_HBAR_C;
        const double M = 0.5 * (GPM_PROTON_MASS + GPM_NEUTRON_MASS);
        const double E = K + ml;
        const double y = q / E;
        const double x = 0.5 * Q2 / (M * q);
        const double shadowing = gpm_photonuclear_shadowing_BM(Z, A, x, q);
        const double F2A = gpm_photonuclear_f2a_BM(Z, A, shadowing, x, Q2);
        const double R = 0.25;
        const double dds = (1 - y +
                               0.5 * (1 - 2 * ml * ml / Q2) *
                                   (y * y + Q2 / (E * E)) / (1 + R)) /
                (Q2 * Q2) -
            0.25 / (E * E * Q2);
        return cf * F2A * dds / q;
}

/* Photon-nucleon cross section of Kokoulin, in micro barn
 * (dcs_photonuclear_phn_Kokoulin, pumas.c:15193-15203). */
GPM_HD double gpm_photonuclear_phn_kokoulin(double q)
{
        if (q <= 17.) {
                return 96.1 + 82. / sqrt(q);
        } else if (q <= 200.) {
                const double aux = log(0.0213 * q);
                return 114.3 + 1.647 * aux * aux;
        } else {
                return 49.2 + 11.1 * log(q) + 151.8 / sqrt(q);
        }
}

/* Hard component parameters of the BBKS model (Bugaev, Montaruli, Shlepin &
 * Sokalski), 7 energy decades by 8 polynomial coefficients in log10(v), for
 * muons and for taus (pumas.c:15268-15313). */
GPM_TABLE double gpm_bbks_hard_muon[7][8] = {
        { 7.174409E-04, -0.2436045, -0.2942209, -0.1658391, -0.05227727,
          -9.328318E-03, -8.751909E-04, -3.343145E-05 },
        { 1.7132E-03, -0.5756682, -0.68615, -0.3825223, -0.1196482,
          -0.02124577, -1.987841E-03, -7.584046E-05 },
        { 4.082304E-03, -1.553973, -2.004218, -1.207777, -0.4033373,
          -0.07555636, -7.399682E-03, -2.943396E-04 },
        { 8.628455E-03, -3.251305, -3.999623, -2.33175, -0.7614046,
          -0.1402496, -0.01354059, -5.3155E-04 },
        { 0.01244159, -5.976818, -6.855045, -3.88775, -1.270677,
          -0.2370768, -0.02325118, -9.265136E-04 },
        { 0.02204591, -9.495636, -10.05705, -5.636636, -1.883845,
          -0.3614146, -0.03629659, -1.473118E-03 },
        { 0.03228755, -13.92918, -14.37232, -8.418409, -2.948277,
          -0.5819409, -0.059275, -2.419946E-03 } };
GPM_TABLE double gpm_bbks_hard_tau[7][8] = {
        { -1.269205E-04, -0.01563032, 0.04693954, 0.05338546, 0.02240132,
          4.658909E-03, 4.822364E-04, 1.9837E-05 },
        { -2.843877E-04, -0.03589573, 0.1162945, 0.130975, 0.05496,
          0.01146659, 1.193018E-03, 4.940182E-05 },
        { -5.761546E-04, -0.07768545, 0.3064255, 0.3410341, 0.144945,
          0.03090286, 3.302773E-03, 1.409573E-04 },
        { -1.195445E-03, -0.157375, 0.7041273, 0.7529364, 0.3119032,
          0.06514455, 6.843364E-03, 2.877909E-04 },
        { -1.317386E-03, -0.2720009, 1.440518, 1.425927, 0.5576727,
          0.1109868, 0.011191, 4.544877E-04 },
        { -9.689228E-15, -0.4186136, 2.533355, 2.284968, 0.8360727,
          0.1589677, 0.015614, 6.280818E-04 },
        { -6.4595E-15, -0.8045046, 3.217832, 2.5487, 0.8085682, 0.1344223,
          0.01173827, 4.281932E-04 } };

/* dcs_photonuclear_BBKS (pumas.c:15223-15357): real photon soft component
 * with the Bugaev-Shlepin shadowing, plus the tabulated hard component. */
GPM_HD double gpm_photonuclear_BBKS(
    double Z, double A, double m, double K, double q)
{
        if ((Z <= 0) || (A <= 0) || (m <= 0) || (K <= 0)) return 0.;
        const double M = 0.5 * (GPM_NEUTRON_MASS + GPM_PROTON_MASS);
        const double mpi = GPM_PION_MASS;
        if ((q <= mpi + 0.5 * mpi * mpi / M) ||
            (q >= K + m - 0.5 * (M + m * m / M)))
                return 0.;
        const double m1 = 0.54;
        const double m2 = 1.80;
        const double sgn = gpm_photonuclear_phn_kokoulin(q);
        const double v = q / (K + m);
        double G = 1.;
        if (Z != 1) {
                const double tmp = 0.00282 * pow(A, 1. / 3) * sgn;
                G = (3. / tmp) *
                    (0.5 + ((1. + tmp) * exp(-tmp) - 1.) / (tmp * tmp));
        }
        G *= 3.;
        double aux = v * m;
        const double t = aux * aux / (1. - v);
        double aum = m;
        aum *= aum;
        aux = 2. * aum / t;
        const double kappa = 1. - 2. / v + 2. / (v * v);
        aux = G * ((kappa + 4. * aum / m1) * log(1. + m1 / t) -
                      (kappa * m1) / (m1 + t) - aux) +
            ((kappa + 2. * aum / m2) * log(1. + m2 / t) - aux) +
            aux * (G * (m1 - 4. * t) / (m1 + t) + (m2 / t) * log(1. + t / m2));
        aux *= GPM_ALPHA_EM / (8. * GPM_PI) * A * v * sgn;

        const double(*table)[8] =
            (fabs(m - GPM_MUON_MASS) < fabs(m - GPM_TAU_MASS)) ?
            gpm_bbks_hard_muon : gpm_bbks_hard_tau;
        const double E = K + m;
        if ((E > 1E+02) && (v > 1E-07)) {
                const double lE = log10(E) - 3.;
                const double lv = log10(v);
                int iE = (int)lE;
                double f[2] = { 0., 0. };
                int i;
                for (i = 0; i < 2; i++, iE++) {
                        const int j = (iE > 6) ? 6 : iE;
                        const double x = (lv > -6.) ? lv : -6.;
                        const double * const c = &table[j][0];
                        f[i] = c[0] + x * (c[1] + x * (c[2] + x * (c[3] +
                            x * (c[4] + x * (c[5] + x * (c[6] + x * c[7]))))));
                        if (lv < -6.) f[i] *= 7 + lv;
                        if (lE < 0) f[i] *= 1. + lE;
                }
                const double h = lE - (int)lE;
                double fi;
                if ((f[0] > 0.) && (f[1] > 0.))
                        fi = exp(log(f[0]) * (1. - h) + log(f[1]) * h);
                else
                        fi = f[0] * (1. - h) + f[1] * h;
                aux += A * fi / v;
        }
        return aux * 1E-34 / (K + m);
}

/* dcs_photonuclear_BM (pumas.c:15099-15104): dcs_photonuclear_integrated
 * in mode 0 (pumas.c:15002-15060) of the BM doubly differential cross
 * section, over the 9 Gauss-Legendre nodes xGQ, wGQ of [0, 1] mapped to
 * log Q2 (math_gauss_quad_initialise, pumas.c:12575-12602). */
GPM_HD double gpm_photonuclear_BM(double Z, double A, double ml, double K,
    double q, const double * xGQ, const double * wGQ)
{
        if ((Z <= 0) || (A <= 0) || (ml <= 0) || (K <= 0)) return 0.;
        const double M = 0.5 * (GPM_NEUTRON_MASS + GPM_PROTON_MASS);
        const double mpi = GPM_PION_MASS;
        if ((q <= mpi + 0.5 * mpi * mpi / M) ||
            (q >= K + ml - 0.5 * (M + ml * ml / M)))
                return 0.;
        const double E = K + ml;
        const double ml2 = ml * ml;
        const double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
        const double Q2max = 2.0 * M * (q - mpi) - mpi * mpi;
        if ((Q2max < Q2min) | (Q2min < 0)) return 0.;
        const double xmin = log(Q2min);
        const double xmax = log(Q2max);
        const double dx = xmax - xmin;
        double ds = 0.;
        int i;
        for (i = 0; i < 9; i++) {
                const double Q2 = exp(xmin + dx * xGQ[i]);
                const double w = wGQ[i] * (dx * Q2);
                const double tmp =
                    gpm_photonuclear_d2_BM(Z, A, ml, K, q, Q2);
                if (tmp <= 0.) continue;
                ds += tmp * w;
        }
        return (ds < 0.) ? 0. : ds;
}

#endif

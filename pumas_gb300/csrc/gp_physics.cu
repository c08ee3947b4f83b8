/*
 * gp_physics.cu -- physics tables: dump parsing and device upload.
 *
 * Replaces pumas_physics_load (pumas.c:2049-2165) for the GPU: the blob of a
 * `pumas_physics_dump` stream (or a live `struct pumas_physics`) is parsed
 * with the private layout of pumas.c:660-806 on LP64 hosts (10 ints and the
 * particle enum, 4 doubles, 53 data pointers, 3 DCS pointers, data segment at
 * byte 528), copied to one device allocation, and completed with per element
 * constants (gp_internal.h).
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gpumas.h"
#include "gp_internal.h"

#define ALPHA_EM 7.2973525693E-03
#define HBAR_C 1.973269804E-16
#define BOHR_RADIUS 0.529177210903E-10
#define PROTON_MASS 0.938272
#define NEUTRON_MASS 0.939565

/* Nuclear r.m.s. charge radii in fm (data_nuclear_radius,
 * pumas.c:7143-7175): entry 0 is deuterium-like hydrogen, entry Z is
 * element Z, the last entry the standard rock pseudo element. */
static const double nuclear_radius_fm[120] = {
        2.098, 0.858, 1.680, 2.400, 2.518, 2.405,
        2.470, 2.548, 2.734, 2.900, 2.993, 2.940,
        3.043, 3.035, 3.098, 3.187, 3.245, 3.360,
        3.413, 3.408, 3.477, 3.443, 3.595, 3.600,
        3.644, 3.681, 3.748, 3.843, 3.776, 3.943,
        3.942, 4.032, 4.065, 4.078, 4.123, 4.135,
        4.188, 4.209, 4.237, 4.249, 4.306, 4.318,
        4.363, 4.388, 4.432, 4.435, 4.479, 4.520,
        4.612, 4.646, 4.640, 4.630, 4.714, 4.706,
        4.756, 4.774, 4.823, 4.848, 4.878, 4.897,
        4.927, 4.948, 5.054, 5.093, 5.133, 5.177,
        5.197, 5.210, 5.264, 5.301, 5.390, 5.371,
        5.429, 5.479, 5.423, 5.400, 5.409, 5.411,
        5.387, 5.318, 5.404, 5.471, 5.498, 5.520,
        5.520, 5.529, 5.629, 5.637, 5.661, 5.669,
        5.710, 5.701, 5.784, 5.825, 5.824, 5.817,
        5.843, 5.843, 5.868, 5.875, 5.906, 5.912,
        5.918, 5.937, 5.967, 5.973, 5.979, 5.985,
        5.980, 6.033, 6.051, 6.056, 6.074, 6.079,
        6.097, 6.097, 6.119, 6.125, 6.125, 2.958,
};

/* Atomic screening of Salvat et al. (1987), one row per Z = 1..103:
 * amplitudes A1, A2 and exponents b1, b2, b3 (pumas.c:7229-7342). */
static const double salvat_screening[103][5] = {
        { 1.00000E+00, 0.00000E+00, 1.11728E+00, 1.00000E+00, 1.00000E+00 },  /* Z = 1 */
        { -2.25920E-01, 1.22592E+00, 5.52725E+00, 2.39924E+00, 1.00000E+00 },  /* Z = 2 */
        { 6.04537E-01, 3.95463E-01, 2.81741E+00, 6.62463E-01, 1.00000E+00 },  /* Z = 3 */
        { 3.27766E-01, 6.72234E-01, 4.54302E+00, 9.85154E-01, 1.00000E+00 },  /* Z = 4 */
        { 2.32684E-01, 7.67316E-01, 5.99006E+00, 1.21347E+00, 1.00000E+00 },  /* Z = 5 */
        { 1.53676E-01, 8.46324E-01, 8.04043E+00, 1.49129E+00, 1.00000E+00 },  /* Z = 6 */
        { 9.95750E-02, 9.00425E-01, 1.08122E+01, 1.76868E+00, 1.00000E+00 },  /* Z = 7 */
        { 6.25130E-02, 9.37487E-01, 1.48233E+01, 2.04035E+00, 1.00000E+00 },  /* Z = 8 */
        { 3.68040E-02, 9.63196E-01, 2.14001E+01, 2.30601E+00, 1.00000E+00 },  /* Z = 9 */
        { 1.88410E-02, 9.81159E-01, 3.49994E+01, 2.56621E+00, 1.00000E+00 },  /* Z = 10 */
        { 7.44440E-01, 2.55560E-01, 4.12050E+00, 8.71798E-01, 1.00000E+00 },  /* Z = 11 */
        { 6.42349E-01, 3.57651E-01, 4.72663E+00, 1.00247E+00, 1.00000E+00 },  /* Z = 12 */
        { 6.00152E-01, 3.99848E-01, 5.14051E+00, 1.01529E+00, 1.00000E+00 },  /* Z = 13 */
        { 5.15971E-01, 4.84029E-01, 5.84918E+00, 1.17314E+00, 1.00000E+00 },  /* Z = 14 */
        { 4.38675E-01, 5.61325E-01, 6.67070E+00, 1.34102E+00, 1.00000E+00 },  /* Z = 15 */
        { 5.45871E-01, -5.33329E-01, 6.37029E+00, 2.55169E+00, 1.67534E+00 },  /* Z = 16 */
        { 7.24889E-01, -7.54809E-01, 6.21183E+00, 3.38827E+00, 1.85964E+00 },  /* Z = 17 */
        { 2.19124E+00, -2.2852E+00, 5.54701E+00, 4.56873E+00, 2.04455E+00 },  /* Z = 18 */
        { 4.85607E-02, 7.75935E-01, 3.02597E+01, 3.12426E+00, 7.32637E-01 },  /* Z = 19 */
        { 5.80017E-01, 4.19983E-01, 6.32184E+00, 1.00935E+00, 1.00000E+00 },  /* Z = 20 */
        { 5.54340E-01, 4.45660E-01, 6.63280E+00, 1.10227E+00, 1.00000E+00 },  /* Z = 21 */
        { 1.11950E-02, 6.83176E-01, 9.97569E+01, 4.12865E+00, 1.00896E+00 },  /* Z = 22 */
        { 3.18350E-02, 6.75303E-01, 4.25330E+01, 3.94043E+00, 1.05333E+00 },  /* Z = 23 */
        { 1.07503E-01, 7.16172E-01, 1.89587E+01, 3.06375E+00, 1.00137E+00 },  /* Z = 24 */
        { 4.97556E-02, 6.86632E-01, 3.18642E+01, 3.78110E+00, 1.12787E+00 },  /* Z = 25 */
        { 5.11841E-02, 6.99533E-01, 3.18251E+01, 3.77161E+00, 1.16064E+00 },  /* Z = 26 */
        { 5.00039E-02, 7.14201E-01, 3.29153E+01, 3.79085E+00, 1.19152E+00 },  /* Z = 27 */
        { 4.73509E-02, 7.29404E-01, 3.47580E+01, 3.82989E+00, 1.22089E+00 },  /* Z = 28 */
        { 7.70967E-02, 7.95083E-01, 2.53264E+01, 3.39276E+00, 1.14261E+00 },  /* Z = 29 */
        { 4.00041E-02, 7.59034E-01, 4.03429E+01, 3.94645E+00, 1.27594E+00 },  /* Z = 30 */
        { 1.08344E-01, 7.48941E-01, 2.01922E+01, 3.47325E+00, 1.00643E+00 },  /* Z = 31 */
        { 6.09767E-02, 7.15671E-01, 2.91996E+01, 4.12525E+00, 1.18447E+00 },  /* Z = 32 */
        { 2.11561E-02, 6.70932E-01, 6.24873E+01, 4.95015E+00, 1.35819E+00 },  /* Z = 33 */
        { 4.83575E-01, 5.16425E-01, 8.78242E+00, 1.69671E+00, 1.00000E+00 },  /* Z = 34 */
        { 4.50364E-01, 5.49636E-01, 9.33480E+00, 1.79002E+00, 1.00000E+00 },  /* Z = 35 */
        { 4.19036E-01, 5.80964E-01, 9.91420E+00, 1.88354E+00, 1.00000E+00 },  /* Z = 36 */
        { 1.73438E-01, 7.25336E-01, 1.71659E+01, 3.11025E+00, 7.17673E-01 },  /* Z = 37 */
        { 3.35694E-02, 7.81581E-01, 5.52077E+01, 4.28418E+00, 8.57842E-01 },  /* Z = 38 */
        { 6.88939E-02, 7.20203E-01, 3.13659E+01, 4.24121E+00, 9.47152E-01 },  /* Z = 39 */
        { 1.17552E-01, 6.58088E-01, 2.20537E+01, 4.03254E+00, 1.01806E+00 },  /* Z = 40 */
        { 2.55689E-01, 5.82051E-01, 1.42403E+01, 2.97020E+00, 1.01699E+00 },  /* Z = 41 */
        { 2.69313E-01, 5.75262E-01, 1.40442E+01, 2.86107E+00, 1.05906E+00 },  /* Z = 42 */
        { 2.20138E-01, 5.61797E-01, 1.59176E+01, 3.36719E+00, 1.15477E+00 },  /* Z = 43 */
        { 2.75057E-01, 5.94338E-01, 1.43137E+01, 2.73701E+00, 1.10923E+00 },  /* Z = 44 */
        { 2.71053E-01, 6.11921E-01, 1.46537E+01, 2.71828E+00, 1.12336E+00 },  /* Z = 45 */
        { 2.78363E-01, 6.06653E-01, 1.46455E+01, 2.61549E+00, 1.43183E+00 },  /* Z = 46 */
        { 2.56210E-01, 6.50520E-01, 1.55878E+01, 2.74124E+00, 1.14079E+00 },  /* Z = 47 */
        { 2.27100E-01, 6.15496E-01, 1.69141E+01, 3.08408E+00, 1.26189E+00 },  /* Z = 48 */
        { 2.49215E-01, 6.43990E-01, 1.61552E+01, 2.88189E+00, 9.94156E-01 },  /* Z = 49 */
        { 2.15313E-01, 6.11497E-01, 1.77931E+01, 3.29372E+00, 1.14781E+00 },  /* Z = 50 */
        { 1.80560E-01, 5.76688E-01, 1.98751E+01, 3.80921E+00, 1.28288E+00 },  /* Z = 51 */
        { 1.30772E-01, 5.50366E-01, 2.41540E+01, 4.61191E+00, 1.41954E+00 },  /* Z = 52 */
        { 5.88293E-02, 5.48174E-01, 3.99955E+01, 5.91318E+00, 1.54707E+00 },  /* Z = 53 */
        { 4.45145E-01, 5.54855E-01, 1.18053E+01, 1.79673E+00, 1.00000E+00 },  /* Z = 54 */
        { 2.70796E-01, 6.52415E-01, 1.65915E+01, 2.69645E+00, 6.81361E-01 },  /* Z = 55 */
        { 1.72814E-01, 6.84485E-01, 2.23966E+01, 3.45951E+00, 8.07311E-01 },  /* Z = 56 */
        { 1.94726E-01, 6.38429E-01, 2.07637E+01, 3.46574E+00, 8.91057E-01 },  /* Z = 57 */
        { 1.91338E-01, 6.46684E-01, 2.12350E+01, 3.48193E+00, 9.01112E-01 },  /* Z = 58 */
        { 1.86776E-01, 6.55810E-01, 2.18033E+01, 3.50982E+00, 9.10636E-01 },  /* Z = 59 */
        { 1.66461E-01, 7.05677E-01, 2.39492E+01, 3.51987E+00, 8.48620E-01 },  /* Z = 60 */
        { 1.62350E-01, 7.13311E-01, 2.45984E+01, 3.55603E+00, 8.56929E-01 },  /* Z = 61 */
        { 1.58016E-01, 7.20978E-01, 2.52966E+01, 3.59628E+00, 8.65025E-01 },  /* Z = 62 */
        { 1.53759E-01, 7.28385E-01, 2.60169E+01, 3.63834E+00, 8.73083E-01 },  /* Z = 63 */
        { 1.58729E-01, 7.02414E-01, 2.54973E+01, 3.73639E+00, 9.54998E-01 },  /* Z = 64 */
        { 1.45327E-01, 7.42619E-01, 2.75466E+01, 3.72882E+00, 8.88981E-01 },  /* Z = 65 */
        { 1.41260E-01, 7.49352E-01, 2.83460E+01, 3.77625E+00, 8.96917E-01 },  /* Z = 66 */
        { 1.37360E-01, 7.55797E-01, 2.91604E+01, 3.82444E+00, 9.04803E-01 },  /* Z = 67 */
        { 1.33614E-01, 7.61947E-01, 2.99904E+01, 3.87344E+00, 9.12768E-01 },  /* Z = 68 */
        { 1.29853E-01, 7.68005E-01, 3.08345E+01, 3.92327E+00, 9.20306E-01 },  /* Z = 69 */
        { 1.26659E-01, 7.73365E-01, 3.16806E+01, 3.97271E+00, 9.28838E-01 },  /* Z = 70 */
        { 1.28806E-01, 7.52781E-01, 3.13526E+01, 4.09040E+00, 1.00717E+00 },  /* Z = 71 */
        { 1.30256E-01, 7.32428E-01, 3.12166E+01, 4.20492E+00, 1.09456E+00 },  /* Z = 72 */
        { 1.38420E-01, 7.09596E-01, 3.00767E+01, 4.24918E+00, 1.16966E+00 },  /* Z = 73 */
        { 1.50030E-01, 6.87141E-01, 2.86302E+01, 4.24261E+00, 1.23403E+00 },  /* Z = 74 */
        { 1.60803E-01, 6.65932E-01, 2.75684E+01, 4.23412E+00, 1.29699E+00 },  /* Z = 75 */
        { 1.72164E-01, 6.46849E-01, 2.65861E+01, 4.19992E+00, 1.35350E+00 },  /* Z = 76 */
        { 1.83411E-01, 6.30598E-01, 2.57339E+01, 4.14615E+00, 1.40374E+00 },  /* Z = 77 */
        { 2.23043E-01, 6.17575E-01, 2.29939E+01, 3.73461E+00, 1.44284E+00 },  /* Z = 78 */
        { 2.28909E-01, 6.11402E-01, 2.28644E+01, 3.69138E+00, 1.48856E+00 },  /* Z = 79 */
        { 2.09753E-01, 6.00426E-01, 2.44080E+01, 3.96429E+00, 1.53432E+00 },  /* Z = 80 */
        { 2.70821E-01, 6.42829E-01, 2.09409E+01, 3.24563E+00, 1.11214E+00 },  /* Z = 81 */
        { 2.37958E-01, 6.30789E-01, 2.29872E+01, 3.62172E+00, 1.23735E+00 },  /* Z = 82 */
        { 2.28771E-01, 6.21959E-01, 2.37917E+01, 3.77959E+00, 1.25338E+00 },  /* Z = 83 */
        { 1.94059E-01, 6.10455E-01, 2.66951E+01, 4.25824E+00, 1.35772E+00 },  /* Z = 84 */
        { 1.49995E-01, 6.03147E-01, 3.18397E+01, 4.92848E+00, 1.46828E+00 },  /* Z = 85 */
        { 9.55262E-02, 6.05994E-01, 4.34890E+01, 5.85205E+00, 1.57359E+00 },  /* Z = 86 */
        { 3.19155E-01, 6.23324E-01, 2.00150E+01, 2.90906E+00, 7.20714E-01 },  /* Z = 87 */
        { 2.40406E-01, 6.56665E-01, 2.45012E+01, 3.55241E+00, 8.37599E-01 },  /* Z = 88 */
        { 2.26579E-01, 6.42246E-01, 2.56843E+01, 3.79223E+00, 9.33468E-01 },  /* Z = 89 */
        { 2.17619E-01, 6.24013E-01, 2.65542E+01, 4.00437E+00, 1.02385E+00 },  /* Z = 90 */
        { 2.41294E-01, 6.30394E-01, 2.51930E+01, 3.67795E+00, 9.69895E-01 },  /* Z = 91 */
        { 2.44758E-01, 6.29816E-01, 2.52522E+01, 3.63966E+00, 9.82474E-01 },  /* Z = 92 */
        { 2.46231E-01, 6.31596E-01, 2.54271E+01, 3.61328E+00, 9.92527E-01 },  /* Z = 93 */
        { 2.55572E-01, 6.49005E-01, 2.51526E+01, 3.43021E+00, 9.32751E-01 },  /* Z = 94 */
        { 2.53567E-01, 6.53604E-01, 2.55959E+01, 3.43474E+00, 9.41671E-01 },  /* Z = 95 */
        { 2.43832E-01, 6.43738E-01, 2.65567E+01, 3.59089E+00, 1.01827E+00 },  /* Z = 96 */
        { 2.41898E-01, 6.48850E-01, 2.70360E+01, 3.59411E+00, 1.02554E+00 },  /* Z = 97 */
        { 2.44050E-01, 6.70318E-01, 2.72673E+01, 3.48061E+00, 9.66447E-01 },  /* Z = 98 */
        { 2.40237E-01, 6.76319E-01, 2.79152E+01, 3.50331E+00, 9.74347E-01 },  /* Z = 99 */
        { 2.34997E-01, 6.65571E-01, 2.86446E+01, 3.61870E+00, 1.04137E+00 },  /* Z = 100 */
        { 2.32114E-01, 6.88406E-01, 2.93353E+01, 3.55697E+00, 9.90568E-01 },  /* Z = 101 */
        { 2.27937E-01, 6.94394E-01, 3.01040E+01, 3.58685E+00, 9.98878E-01 },  /* Z = 102 */
        { 2.29571E-01, 6.82014E-01, 3.02650E+01, 3.64085E+00, 1.04473E+00 },  /* Z = 103 */
};

/* Radiation logarithms for Z = 1..92, 0 if unset (pumas.c:13709-13738). */
static const double radiation_log_table[92] = {
        202.4, 151.9, 159.9, 172.3, 177.9, 178.3, 176.6, 173.4,
        170.0, 165.8, 165.8, 167.1, 169.1, 170.8, 172.2, 173.4,
        174.3, 174.8, 175.1, 175.6, 176.2, 176.8, 0.0, 0.0,
        0.0, 175.8, 0.0, 0.0, 173.1, 0.0, 0.0, 173.0,
        0.0, 0.0, 173.5, 0.0, 0.0, 0.0, 0.0, 0.0,
        0.0, 175.9, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
        0.0, 177.4, 0.0, 0.0, 178.6, 0.0, 0.0, 0.0,
        0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
        0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
        0.0, 177.6, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
        0.0, 178.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
        0.0, 0.0, 0.0, 179.8,
};

static double nuclear_radius(double Z, double A)
{
        int iN = (int)Z;
        const int nN = 120;
        if (iN >= nN - 1)
                iN = nN - 2;
        else if ((iN == 1) && (A >= 1.5))
                iN = 0;
        else if ((iN == 11) && (A == 22.))
                iN = nN - 1;
        return nuclear_radius_fm[iN] * 1E-15;
}

static double radiation_logarithm(double Z)
{
        const int i = (int)Z;
        if ((i >= 1) && (i <= 92)) {
                const double l = radiation_log_table[i - 1];
                if (l > 0) return l;
        }
        return 182.7;
}

/* Per element constants, with the expressions of the reference. */
static void element_constants(struct gp_element * e, double mass)
{
        const double Z = e->Z, A = e->A;
        int iZ = (int)Z - 1;
        if (iZ >= 103) iZ = 102;
        if (iZ < 0) iZ = 0;
        const double * row = salvat_screening[iZ];
        if (row[4] == 1.) {
                if (iZ == 0) {
                        e->n_screen = 1;
                        e->amplitude[0] = 1.;
                } else {
                        e->n_screen = 2;
                        e->amplitude[0] = row[0];
                        e->amplitude[1] = 1. - e->amplitude[0];
                }
        } else {
                e->n_screen = 3;
                e->amplitude[0] = row[0];
                e->amplitude[1] = row[1];
                e->amplitude[2] = 1. - (e->amplitude[0] + e->amplitude[1]);
        }
        for (int i = 0; i < 3; i++) e->a_screen[i] = row[2 + i] / BOHR_RADIUS;
        e->RN = nuclear_radius(Z, A);
        e->Ma = Z * PROTON_MASS + (A - Z) * NEUTRON_MASS;
        e->z13 = pow(Z, 1. / 3.);
        e->z13_inv = 1. / e->z13;
        e->zm13 = pow(Z, -1. / 3.);
        e->z23 = pow(Z, 2. / 3.);
        e->dn = 1.54 * pow(A, 0.27);
        e->rad_log = radiation_logarithm(Z);
        {
                const double sqrte = 1.6487212707;
                e->qmax_m_pair = 1. - 0.75 * sqrte * e->z13;
        }
        e->qmax_m_brems = 1. - 0.75 * 1.648721270700128 * e->z13;
        {
                const double tmp2 = mass * e->RN / HBAR_C;
                e->muni = tmp2 * tmp2 / 6.;
        }
        {
                /* dcs_bremsstrahlung_SSR (pumas.c:13950-13958). */
                const double m = mass * 1E+03;
                const double MMU = 105.6583745;
                const double mu_qc = m / (MMU * exp(1.) / e->dn);
                const double rho = sqrt(1. + 4. * mu_qc * mu_qc);
                const double log_rho = log((rho + 1.) / (rho - 1.));
                e->mu_qc = mu_qc;
                e->ssr_delta1 = log(mu_qc) + 0.5 * rho * log_rho;
                e->ssr_delta2 = log(mu_qc) +
                    0.25 * (3. * rho - rho * rho * rho) * log_rho +
                    2. * mu_qc * mu_qc;
        }
        {
                /* dcs_pair_production_d2_SSR (pumas.c:14418-14421). */
                const double RE = 2.8179403227E-13;
                const double ME = 0.5109989461;
                const double m = mass * 1E+03;
                e->pair_pref = 4. / (3. * 3.14159265358979323846) * Z *
                    pow(ALPHA_EM * RE, 2.);
                e->pair_medn2 = pow(ME / m * e->dn, 2.);
        }
        e->log_A = log(A);
        e->shadow_low = exp(-0.1 * log(A));
}

/* Bake the cubic Hermite rows of (x, y, m) as in table_interpolate_pchip
 * (pumas.c:4146-4157), with the row 0 rule of m1 unless `no_row0_rule`
 * (table_get_msc, pumas.c:4097-4110, never uses row 0). */
static void bake(const double * x, const double * y, const double * m, int n,
    struct gp_coef * out, int no_row0_rule)
{
        for (int i1 = 0; i1 < n - 1; i1++) {
                const int i2 = i1 + 1;
                const double dX = x[i2] - x[i1];
                const double m1 = m[i1] * dX;
                const double m2 = ((i2 > 1) || no_row0_rule) ? m[i2] * dX : m1;
                const double p0 = y[i1], p1 = y[i2];
                out[i1].p0 = p0;
                out[i1].m0 = m1;
                out[i1].c2 = -3 * (p0 - p1) - 2 * m1 - m2;
                out[i1].c3 = 2 * (p0 - p1) + m1 + m2;
        }
        out[n - 1].p0 = y[n - 1];
        out[n - 1].m0 = out[n - 1].c2 = out[n - 1].c3 = 0.;
}

static void bake_nodes(const double * x, int n, struct gp_node * out)
{
        for (int i = 0; i < n - 1; i++) {
                out[i].x = x[i];
                out[i].dx = x[i + 1] - x[i];
                out[i].inv_dx = 1. / out[i].dx;
                out[i].pad = 0.;
        }
        out[n - 1].x = x[n - 1];
        out[n - 1].inv_dx = out[n - 1].dx = out[n - 1].pad = 0.;
}

struct parsed {
        int n_energies, n_materials, n_composites, n_elements, n_components;
        int max_components, n_table_dcs, particle;
        int model_brems, model_pair, model_photo;
        double ctau, mass, cutoff, elastic_ratio;
        int64_t off[53];
};

/* Parse the header and pointer table of a physics blob of `size` bytes. */
static int parse_blob(const char * b, int64_t size, struct parsed * p)
{
        if (size < 528) return GPUMAS_RETURN_FORMAT_ERROR;
        int hdr[11];
        memcpy(hdr, b, sizeof(hdr));
        if (hdr[0] != size) return GPUMAS_RETURN_FORMAT_ERROR;
        p->n_energies = hdr[1];
        p->n_materials = hdr[2];
        p->n_composites = hdr[3];
        p->n_elements = hdr[4];
        p->n_components = hdr[5];
        p->max_components = hdr[6];
        p->n_table_dcs = hdr[9];
        p->particle = hdr[10];
        double dbl[4];
        memcpy(dbl, b + 48, sizeof(dbl));
        p->ctau = dbl[0];
        p->mass = dbl[1];
        p->cutoff = dbl[2];
        p->elastic_ratio = dbl[3];
        uint64_t ptr[53];
        memcpy(ptr, b + 80, sizeof(ptr));
        for (int i = 0; i < 53; i++) {
                p->off[i] = (int64_t)(ptr[i] - ptr[0]) + 528;
                if ((p->off[i] < 528) || (p->off[i] > size))
                        return GPUMAS_RETURN_FORMAT_ERROR;
        }
        if ((p->n_energies < 3) || (p->n_materials < 1) ||
            (p->n_elements < 1) || (p->max_components > GP_MAX_COMPONENTS))
                return GPUMAS_RETURN_FORMAT_ERROR;
        /* The DCS models of the dump (pumas.c:2167-2196). */
        const char * brems = b + p->off[50];
        const char * pair = b + p->off[51];
        const char * photo = b + p->off[52];
        p->model_brems = (strcmp(brems, "SSR") == 0) ? 0 :
            (strcmp(brems, "KKP") == 0) ? 1 :
            (strcmp(brems, "ABB") == 0) ? 2 : -1;
        p->model_pair = (strcmp(pair, "SSR") == 0) ? 0 :
            (strcmp(pair, "KKP") == 0) ? 1 : -1;
        p->model_photo = (strcmp(photo, "DRSS") == 0) ? 0 :
            (strcmp(photo, "BBKS") == 0) ? 1 :
            (strcmp(photo, "BM") == 0) ? 2 : -1;
        if ((p->model_brems < 0) || (p->model_pair < 0) ||
            (p->model_photo < 0))
                return GPUMAS_RETURN_MODEL_ERROR;
        /* Muons or taus (enum pumas_particle, pumas.h:45-50). */
        if ((p->particle != GPUMAS_PARTICLE_MUON) &&
            (p->particle != GPUMAS_PARTICLE_TAU))
                return GPUMAS_RETURN_UNKNOWN_PARTICLE;
        return GPUMAS_RETURN_SUCCESS;
}

static inline const char * rebase(
    const char * b, const struct parsed * p, uint64_t address)
{
        uint64_t base;
        memcpy(&base, b + 80, 8);
        return b + (int64_t)(address - base) + 528;
}

static size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

static inline int64_t lut_key(double v)
{
        int64_t b;
        memcpy(&b, &v, 8);
        return b >> GP_LUT_SHIFT;
}

/* Bucket index of a non-decreasing table of n rows, appended to `out`.
 * Returns the number of entries, 0 if the table is not suitable (then the
 * device bisects). */
static int lut_build(const double * table, int n, unsigned short * out,
    int capacity, int * key0)
{
        const int imax = n - 1;
        if ((table[0] < 0.) || !(table[1] > 0.) || !(table[imax] > 0.))
                return 0;
        for (int i = 0; i < imax; i++)
                if (!(table[i] <= table[i + 1])) return 0;
        const int64_t k0 = lut_key(table[1]);
        const int64_t k1 = lut_key(table[imax]);
        const int64_t m = k1 - k0 + 1;
        if ((m <= 0) || (m > capacity)) return 0;
        int i = 0;
        for (int64_t k = 0; k < m; k++) {
                const int64_t bits = (k0 + k) << GP_LUT_SHIFT;
                double lo;
                memcpy(&lo, &bits, 8);
                while ((i + 1 < imax) && (table[i + 1] <= lo)) i++;
                out[k] = (unsigned short)i;
        }
        *key0 = (int)k0;
        return (int)m;
}

static int physics_from_blob(
    struct gpumas_physics ** out, const char * b, int64_t size)
{
        *out = NULL;
        struct parsed p;
        int rc = parse_blob(b, size, &p);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;

        /* Host side staging of the extra arrays. */
        const int nm = p.n_materials, ne = p.n_elements, nc = p.n_components;
        const int * elements_in = (const int *)(b + p.off[41]);
        const uint64_t * eptr = (const uint64_t *)(b + p.off[46]);
        const uint64_t * cptr = (const uint64_t *)(b + p.off[47]);
        const uint64_t * nptr = (const uint64_t *)(b + p.off[49]);

        const size_t off_elements = align256(size);
        const size_t off_comp_start =
            align256(off_elements + ne * sizeof(struct gp_element));
        const size_t off_comp_element =
            align256(off_comp_start + nm * sizeof(int));
        const size_t off_comp_fraction =
            align256(off_comp_element + nc * sizeof(int));
        const int n_lut = GP_N_LUT(nm);
        const size_t off_lut = align256(off_comp_fraction + nc * sizeof(double));
        const int lut_capacity = 1 << 16;
        const size_t off_lut_idx = align256(off_lut + n_lut * sizeof(gp_lut));
        const size_t off_node = align256(off_lut_idx +
            (size_t)n_lut * lut_capacity * sizeof(unsigned short));
        const size_t off_coef = align256(off_node +
            (size_t)n_lut * p.n_energies * sizeof(gp_node));
        const size_t total = align256(off_coef +
            (size_t)GP_N_COEF(nm) * p.n_energies * sizeof(gp_coef));

        char * host = (char *)calloc(1, total);
        if (host == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
        memcpy(host, b, size);
        struct gp_element * el = (struct gp_element *)(host + off_elements);
        for (int i = 0; i < ne; i++) {
                const char * e = rebase(b, &p, eptr[i]);
                memcpy(&el[i].Z, e, 8);
                memcpy(&el[i].A, e + 8, 8);
                memcpy(&el[i].I, e + 16, 8);
                memcpy(&el[i].index, e + 24, 4);
                element_constants(el + i, p.mass);
        }
        int * comp_start = (int *)(host + off_comp_start);
        int * comp_element = (int *)(host + off_comp_element);
        double * comp_fraction = (double *)(host + off_comp_fraction);
        int ic = 0;
        for (int i = 0; i < nm; i++) {
                comp_start[i] = ic;
                if (elements_in[i] > GP_MAX_COMPONENTS) {
                        free(host);
                        return GPUMAS_RETURN_FORMAT_ERROR;
                }
                const char * c = rebase(b, &p, cptr[i]);
                for (int j = 0; j < elements_in[i]; j++, ic++) {
                        if (ic >= nc) {
                                free(host);
                                return GPUMAS_RETURN_FORMAT_ERROR;
                        }
                        memcpy(comp_element + ic, c + 16 * j, 4);
                        memcpy(comp_fraction + ic, c + 16 * j + 8, 8);
                }
        }

        /* Bucket indices of the searched tables (device addresses are set
         * once the allocation is made). */
        gp_lut * luts = (gp_lut *)(host + off_lut);
        {
                const int ne_ = p.n_energies;
                const double * K = (const double *)(b + p.off[3]);
                const double * X = (const double *)(b + p.off[7]);
                const double * Tt = (const double *)(b + p.off[10]);
                const double * NIi = (const double *)(b + p.off[18]);
                const double * NIe = (const double *)(b + p.off[16]);
                for (int id = 0; id < n_lut; id++) {
                        const double * tab;
                        if (id == 0) {
                                tab = K;
                        } else if (id <= 2 * nm) {
                                tab = X + (size_t)(id - 1) * ne_;
                        } else if (id <= 4 * nm) {
                                tab = Tt + (size_t)(id - 1 - 2 * nm) * ne_;
                        } else if (id <= 5 * nm) {
                                tab = NIi + (size_t)(id - 1 - 4 * nm) * ne_;
                        } else {
                                tab = NIe + (size_t)(id - 1 - 5 * nm) * ne_;
                        }
                        unsigned short * out = (unsigned short *)(host +
                            off_lut_idx) + (size_t)id * lut_capacity;
                        luts[id].n = lut_build(tab, ne_, out, lut_capacity,
                            &luts[id].key0);
                        luts[id].idx = (const unsigned short *)(
                            (size_t)off_lut_idx +
                            (size_t)id * lut_capacity * sizeof(unsigned short));
                }
        }

        /* Baked interpolants and node grids. */
        {
                const int ne_ = p.n_energies;
                const int M = nm;
#define TAB(k) ((const double *)(b + p.off[k]))
                const double * K = TAB(3);
                gp_node * node = (gp_node *)(host + off_node);
                gp_coef * coef = (gp_coef *)(host + off_coef);
                bake_nodes(K, ne_, node + (size_t)GP_LUT_K * ne_);
                for (int m = 0; m < M; m++) {
                        for (int sc = 0; sc < 2; sc++) {
                                const size_t r = (size_t)(sc * M + m) * ne_;
                                const double * X = TAB(7) + r;
                                const double * Tt = TAB(10) + r;
                                const double * NIe = TAB(16) + r;
                                bake_nodes(X, ne_, node +
                                    (size_t)(1 + sc * M + m) * ne_);
                                bake_nodes(Tt, ne_, node +
                                    (size_t)(1 + (2 + sc) * M + m) * ne_);
                                bake_nodes(NIe, ne_, node +
                                    (size_t)(1 + (5 + sc) * M + m) * ne_);
                                bake(K, X, TAB(8) + r, ne_,
                                    coef + (size_t)GP_C_X(M, sc, m) * ne_, 0);
                                bake(K, Tt, TAB(11) + r, ne_,
                                    coef + (size_t)GP_C_T(M, sc, m) * ne_, 0);
                                bake(K, TAB(12) + r, TAB(13) + r, ne_,
                                    coef + (size_t)GP_C_DE(M, sc, m) * ne_, 0);
                                bake(K, NIe, TAB(17) + r, ne_,
                                    coef + (size_t)GP_C_NI_EL(M, sc, m) * ne_,
                                    0);
                                bake(X, K, TAB(4) + r, ne_, coef +
                                    (size_t)GP_C_K_OF_X(M, sc, m) * ne_, 0);
                                bake(Tt, X, TAB(9) + r, ne_, coef +
                                    (size_t)GP_C_X_OF_T(M, sc, m) * ne_, 0);
                                bake(NIe, K, TAB(6) + r, ne_, coef +
                                    (size_t)GP_C_K_OF_NI_EL(M, sc, m) * ne_,
                                    0);
                        }
                        const size_t r = (size_t)m * ne_;
                        const double * NIi = TAB(18) + r;
                        bake_nodes(NIi, ne_, node +
                            (size_t)(1 + 4 * M + m) * ne_);
                        bake(K, TAB(14) + r, TAB(15) + r, ne_,
                            coef + (size_t)GP_C_OMEGA(M, m) * ne_, 0);
                        bake(K, TAB(20) + r, TAB(21) + r, ne_,
                            coef + (size_t)GP_C_CS(M, m) * ne_, 0);
                        bake(K, NIi, TAB(19) + r, ne_,
                            coef + (size_t)GP_C_NI_IN(M, m) * ne_, 0);
                        bake(NIi, K, TAB(5) + r, ne_,
                            coef + (size_t)GP_C_K_OF_NI_IN(M, m) * ne_, 0);
                        bake(K, TAB(35) + r, TAB(36) + r, ne_,
                            coef + (size_t)GP_C_MU0(M, m) * ne_, 1);
                        for (int s3 = 0; s3 < 3; s3++) {
                                const size_t r3 = (size_t)(s3 * M + m) * ne_;
                                bake(K, TAB(39) + r3, TAB(40) + r3, ne_,
                                    coef + (size_t)GP_C_MS1(M, s3, m) * ne_,
                                    1);
                        }
                }
#undef TAB
        }

        struct gpumas_physics * ph =
            (struct gpumas_physics *)calloc(1, sizeof(*ph));
        if (ph == NULL) {
                free(host);
                return GPUMAS_RETURN_MEMORY_ERROR;
        }
        ph->material_name = (char **)calloc(nm, sizeof(char *));
        for (int i = 0; i < nm; i++) {
                const char * name = rebase(b, &p, nptr[i]);
                ph->material_name[i] = strdup(name);
        }
        ph->n_materials = nm;
        ph->n_elements = ne;
        ph->particle = p.particle;
        cudaGetDevice(&ph->device);

        if (cudaMalloc(&ph->device_blob, total) != cudaSuccess) {
                free(host);
                gpumas_physics_destroy(&ph);
                return GPUMAS_RETURN_DEVICE_ERROR;
        }
        ph->device_size = total;
        for (int id = 0; id < n_lut; id++)
                luts[id].idx = (const unsigned short *)((char *)ph->device_blob +
                    (size_t)luts[id].idx);
        if (cudaMemcpy(ph->device_blob, host, total, cudaMemcpyHostToDevice) !=
            cudaSuccess) {
                free(host);
                gpumas_physics_destroy(&ph);
                return GPUMAS_RETURN_DEVICE_ERROR;
        }
        free(host);

        const char * d = (const char *)ph->device_blob;
        struct gp_tables * t = &ph->tables;
        t->n_energies = p.n_energies;
        t->n_materials = nm;
        t->n_elements = ne;
        t->n_components = nc;
        t->n_table_dcs = p.n_table_dcs;
        t->model_brems = p.model_brems;
        t->model_pair = p.model_pair;
        t->model_photo = p.model_photo;
        t->ctau = p.ctau;
        t->mass = p.mass;
        t->cutoff = p.cutoff;
        t->elastic_ratio = p.elastic_ratio;
#define DD(k) ((const double *)(d + p.off[k]))
#define DF(k) ((const float *)(d + p.off[k]))
        t->K = DD(3);
        t->K_dX = DD(4);
        t->K_dNI_in = DD(5);
        t->K_dNI_el = DD(6);
        t->X = DD(7);
        t->X_dK = DD(8);
        t->X_dT = DD(9);
        t->T = DD(10);
        t->T_dK = DD(11);
        t->dE = DD(12);
        t->dE_dK = DD(13);
        t->Omega = DD(14);
        t->Omega_dK = DD(15);
        t->NI_el = DD(16);
        t->NI_el_dK = DD(17);
        t->NI_in = DD(18);
        t->NI_in_dK = DD(19);
        t->CS = DD(20);
        t->CS_dK = DD(21);
        t->CSf = DD(22);
        t->CSf_dK = DD(23);
        t->CSn = DD(24);
        t->CSn_dK = DD(25);
        t->DCS = DF(26);
        t->DCS_x = DF(27);
        t->DCS_env = DF(28);
        t->Kt = DD(30);
        t->Li = DD(31);
        t->a_max = DD(33);
        t->b_max = DD(34);
        t->Mu0 = DD(35);
        t->Mu0_dK = DD(36);
        t->Lb = DD(37);
        t->Lb_dK = DD(38);
        t->Ms1 = DD(39);
        t->Ms1_dK = DD(40);
        t->elements_in = (const int *)(d + p.off[41]);
        t->material_density = DD(42);
#undef DD
#undef DF
        t->element = (const struct gp_element *)(d + off_elements);
        t->comp_start = (const int *)(d + off_comp_start);
        t->comp_element = (const int *)(d + off_comp_element);
        t->comp_fraction = (const double *)(d + off_comp_fraction);
        t->lut = (const gp_lut *)(d + off_lut);
        t->node = (const gp_node *)(d + off_node);
        t->coef = (const gp_coef *)(d + off_coef);

        /* Constants of the DCS models, with the reference's expressions. */
        t->k.exp1 = exp(1.);
        t->k.exp_half = exp(0.5);
        t->k.exp_m16 = exp(-1. / 6.);
        t->k.exp_13 = exp(1. / 3.);
        t->k.exp_m13 = exp(-1. / 3.);
        t->k.allm_lq0 = log(0.52544 / 0.06527);
        t->k.pair_me_m2 = pow(0.5109989461 / (p.mass * 1E+03), 2.);

        /* Reserve the slot pool of the allocation free entry point on this
         * device now, while the caller allocates anyway. */
        if (gp_static_reserve() != GPUMAS_RETURN_SUCCESS) {
                gpumas_physics_destroy(&ph);
                return GPUMAS_RETURN_DEVICE_ERROR;
        }

        *out = ph;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_physics_load(
    struct gpumas_physics ** physics, const void * dump, size_t size)
{
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        *physics = NULL;
        if ((dump == NULL) || (size < 8)) return GPUMAS_RETURN_FORMAT_ERROR;
        int tag, blob_size;
        memcpy(&tag, dump, 4);
        memcpy(&blob_size, (const char *)dump + 4, 4);
        if ((tag != 13) || (blob_size < 528) ||
            ((size_t)blob_size + 8 > size))
                return GPUMAS_RETURN_FORMAT_ERROR;
        return physics_from_blob(
            physics, (const char *)dump + 8, blob_size);
}

extern "C" int gp_api_physics_upload(
    struct gpumas_physics ** physics, const void * pumas_physics)
{
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        *physics = NULL;
        if (pumas_physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        int size;
        memcpy(&size, pumas_physics, 4);
        return physics_from_blob(
            physics, (const char *)pumas_physics, size);
}

extern "C" void gpumas_physics_destroy(struct gpumas_physics ** physics)
{
        if ((physics == NULL) || (*physics == NULL)) return;
        struct gpumas_physics * ph = *physics;
        if (ph->device_blob != NULL) cudaFree(ph->device_blob);
        if (ph->material_name != NULL) {
                for (int i = 0; i < ph->n_materials; i++)
                        free(ph->material_name[i]);
                free(ph->material_name);
        }
        free(ph);
        *physics = NULL;
}

extern "C" int gp_api_physics_material_index(
    const struct gpumas_physics * physics, const char * name, int * index)
{
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        for (int i = 0; i < physics->n_materials; i++) {
                if (strcmp(physics->material_name[i], name) == 0) {
                        if (index != NULL) *index = i;
                        return GPUMAS_RETURN_SUCCESS;
                }
        }
        return GPUMAS_RETURN_UNKNOWN_MATERIAL;
}

extern "C" int gp_api_physics_info(const struct gpumas_physics * physics,
    int * n_materials, int * n_elements, double * cutoff, double * mass)
{
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        if (n_materials != NULL) *n_materials = physics->n_materials;
        if (n_elements != NULL) *n_elements = physics->n_elements;
        if (cutoff != NULL) *cutoff = physics->tables.cutoff;
        if (mass != NULL) *mass = physics->tables.mass;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" double gpumas_physics_cutoff(const struct gpumas_physics * physics)
{
        return (physics == NULL) ? 0. : physics->tables.cutoff;
}

extern "C" double gpumas_physics_elastic_ratio(
    const struct gpumas_physics * physics)
{
        return (physics == NULL) ? 0. : physics->tables.elastic_ratio;
}

extern "C" int gp_api_physics_particle(const struct gpumas_physics * physics,
    int * particle, double * lifetime, double * mass)
{
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        if (particle != NULL) *particle = physics->particle;
        if (lifetime != NULL) *lifetime = physics->tables.ctau;
        if (mass != NULL) *mass = physics->tables.mass;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_physics_tables(
    const struct gpumas_physics * physics, struct gp_tables * tables)
{
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        *tables = physics->tables;
        return GPUMAS_RETURN_SUCCESS;
}

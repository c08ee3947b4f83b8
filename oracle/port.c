/*
 * port.c -- plain C restatement of the reference transport hot path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle that the GPU engine is checked
 * against on machines where the reference sources are not available, and
 * the CPU baseline of the benchmark. The product never links it.
 *
 * It restates, function by function, the muon transport of the reference
 * library src/pumas.c (PUMAS 1.2.3): `pumas_context_transport` with its CSDA
 * and stepping engines, the table interpolants, the DEL and EHS samplers, the
 * Coulomb scattering functions and the default DCS models (SSR
 * bremsstrahlung, SSR pair production, DRSS photonuclear, ionisation).
 * Floating point expressions keep the reference's evaluation order, so that
 * with the same compiler settings the results are bit-identical. Each
 * function cites the reference lines it follows.
 *
 * Physics tables are read from a `pumas_physics_dump` stream
 * (pumas.c:2167-2196), whose layout mirrors `struct pumas_physics`
 * (pumas.c:660-806) on an LP64 little-endian host.
 *
 * Media with local properties (density profiles and uniform fields of
 * struct gpumas_locals) follow transport_set_locals (pumas.c:5528-5552),
 * the magnetic steps (pumas.c:6352-6382, 6833-6911) and the closed form
 * CSDA deflection (pumas.c:4968-5171). Muon and tau dumps both load.
 *
 * DCS models: bremsstrahlung SSR, KKP, ABB; pair production SSR, KKP;
 * photonuclear DRSS, BBKS, BM (pumas.h:742-771). Not restated: the
 * recorder.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "gp_math.cuh"
#include "gp_models.cuh"
#include "oracle.h"
#include "philox.h"

/* The reference computes the Coulomb pole reduction and transport
 * coefficients in long double (pumas.c:7524-7683): 80 bit extended on
 * x86-64, IEEE quad in software on aarch64. ORACLE_COULOMB_DOUBLE builds a
 * copy in double, used only to show how much of the CPU baseline's time that
 * costs on a given host; the oracle itself is the long double build. */
#ifdef ORACLE_COULOMB_DOUBLE
typedef double coulomb_real;
#define coulomb_log log
#else
typedef long double coulomb_real;
#define coulomb_log logl
#endif

/* ------------------------------------------------------------------------ */
/* Constants (pumas.c:53-200) and public enum values (pumas.h:90-278).      */
/* ------------------------------------------------------------------------ */
#define N_DEL 4
#define BMC_ALPHA 2.0
#define EPSILON_X 3E-03
#define STEP_MIN 1E-07
#define ALPHA_EM 7.2973525693E-03
#define HBAR_C 1.973269804E-16
#define BOHR_RADIUS 0.529177210903E-10
#define ELECTRON_MASS 0.510998910E-03
#define ELECTRON_RADIUS 2.817940285E-15
#define PROTON_MASS 0.938272
#define NEUTRON_MASS 0.939565
#define PION_MASS 0.13957018
#define AVOGADRO_NUMBER 6.02214076E+23
#define PI_ 3.14159265358979323846
#define LARMOR_FACTOR 0.299792458

#define MODE_DISABLED -1
#define MODE_CSDA 0
#define MODE_MIXED 1
#define MODE_STRAGGLED 2
#define MODE_WEIGHTED 0
#define MODE_RANDOMISED 1
#define MODE_FORWARD 0
#define MODE_BACKWARD 1

#define EV_NONE 0
#define EV_LIMIT_ENERGY 1
#define EV_LIMIT_DISTANCE 2
#define EV_LIMIT_GRAMMAGE 4
#define EV_LIMIT_TIME 8
#define EV_LIMIT 15
#define EV_MEDIUM 16
#define EV_BREMSSTRAHLUNG 32
#define EV_PAIR_CREATION 64
#define EV_PHOTONUCLEAR 128
#define EV_DELTA_RAY 256
#define EV_DEL 480
#define EV_COULOMB 512
#define EV_DECAY 1024
#define EV_VERTEX 2016
#define EV_WEIGHT 2048

#define RC_SUCCESS 0
#define RC_ACCURACY_ERROR 1
#define RC_DECAY_ERROR 3
#define RC_DENSITY_ERROR 4
#define RC_DIRECTION_ERROR 5
#define RC_FORMAT_ERROR 11
#define RC_INDEX_ERROR 7
#define RC_PHYSICS_ERROR 8
#define RC_INTERNAL_ERROR 9
#define RC_MEDIUM_ERROR 12
#define RC_MEMORY_ERROR 13
#define RC_MODEL_ERROR 14
#define RC_MISSING_LIMIT 15
#define RC_UNKNOWN_MATERIAL 22
#define RC_VALUE_ERROR 24

/* ------------------------------------------------------------------------ */
/* Physics tables.                                                          */
/* ------------------------------------------------------------------------ */
struct port_element {
        double Z;
        double A;
        double I;
        int index;
};

struct port_physics {
        char * blob;
        int n_energies, n_materials, n_composites, n_elements, n_components;
        int max_components, n_table_dcs, particle;
        /* DCS models: bremsstrahlung 0 SSR, 1 KKP, 2 ABB; pair production
         * 0 SSR, 1 KKP (the names of the dump, pumas.c:2167-2196). */
        int model_brems, model_pair;
        /* Photonuclear: 0 DRSS, 1 BBKS, 2 BM. */
        int model_photo;
        double ctau, mass, cutoff, elastic_ratio;
        const double *K, *K_dX, *K_dNI_in, *K_dNI_el;
        const double *X, *X_dK, *X_dT, *T, *T_dK, *dE, *dE_dK;
        const double *Omega, *Omega_dK, *NI_el, *NI_el_dK, *NI_in, *NI_in_dK;
        const double *CS, *CS_dK, *CSf, *CSf_dK, *CSn, *CSn_dK;
        const float *DCS, *DCS_x, *DCS_env;
        const double *Xt, *Kt, *a_max, *b_max, *Mu0, *Mu0_dK, *Lb, *Lb_dK;
        const double *Ms1, *Ms1_dK;
        const double * Li;
        const int * elements_in;
        const double * material_density;
        struct port_element * element;
        int * comp_start;
        int * comp_element;
        double * comp_fraction;
        const char ** material_name;
};

static struct port_physics * ph = NULL;

static void port_free(struct port_physics * p)
{
        if (p == NULL) return;
        free(p->blob);
        free(p->element);
        free(p->comp_start);
        free(p->comp_element);
        free(p->comp_fraction);
        free(p->material_name);
        free(p);
}

/*
 * Parse a physics dump (pumas.c:2049-2165). The blob starts with the struct
 * header: 10 ints and the particle enum (44 bytes + 4 padding), 4 doubles,
 * then 53 data pointers and 3 DCS function pointers; the data segment starts
 * at byte 528. Pointers are absolute addresses of the dumping process: the
 * first one (mdf_path) is the address of the data segment, which gives the
 * offsets of all others.
 */
int oracle_port_load(const void * dump, int64_t size)
{
        const char * bytes = dump;
        if (size < 8 + 528) return RC_FORMAT_ERROR;
        int tag, blob_size;
        memcpy(&tag, bytes, 4);
        memcpy(&blob_size, bytes + 4, 4);
        if ((tag != 13) || (blob_size + 8 > size) || (blob_size < 528))
                return RC_FORMAT_ERROR;
        struct port_physics * p = calloc(1, sizeof(*p));
        if (p == NULL) return RC_MEMORY_ERROR;
        p->blob = malloc(blob_size);
        if (p->blob == NULL) {
                free(p);
                return RC_MEMORY_ERROR;
        }
        memcpy(p->blob, bytes + 8, blob_size);
        const char * b = p->blob;
        int hdr[11];
        memcpy(hdr, b, sizeof(hdr));
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
        const uint64_t base = ptr[0];
        int64_t off[53];
        int i;
        for (i = 0; i < 53; i++) {
                off[i] = (int64_t)(ptr[i] - base) + 528;
                if ((off[i] < 528) || (off[i] > blob_size)) {
                        port_free(p);
                        return RC_FORMAT_ERROR;
                }
        }
#define D(k) ((const double *)(b + off[k]))
#define F(k) ((const float *)(b + off[k]))
        p->K = D(3);
        p->K_dX = D(4);
        p->K_dNI_in = D(5);
        p->K_dNI_el = D(6);
        p->X = D(7);
        p->X_dK = D(8);
        p->X_dT = D(9);
        p->T = D(10);
        p->T_dK = D(11);
        p->dE = D(12);
        p->dE_dK = D(13);
        p->Omega = D(14);
        p->Omega_dK = D(15);
        p->NI_el = D(16);
        p->NI_el_dK = D(17);
        p->NI_in = D(18);
        p->NI_in_dK = D(19);
        p->CS = D(20);
        p->CS_dK = D(21);
        p->CSf = D(22);
        p->CSf_dK = D(23);
        p->CSn = D(24);
        p->CSn_dK = D(25);
        p->DCS = F(26);
        p->DCS_x = F(27);
        p->DCS_env = F(28);
        p->Xt = D(29);
        p->Kt = D(30);
        p->Li = D(31);
        p->a_max = D(33);
        p->b_max = D(34);
        p->Mu0 = D(35);
        p->Mu0_dK = D(36);
        p->Lb = D(37);
        p->Lb_dK = D(38);
        p->Ms1 = D(39);
        p->Ms1_dK = D(40);
        p->elements_in = (const int *)(b + off[41]);
        p->material_density = D(42);
#undef D
#undef F
        /* Elements: struct atomic_element {double Z, A, I; int index;
         * char * name;} (pumas.c:510-522). */
        p->element = calloc(p->n_elements, sizeof(*p->element));
        const uint64_t * eptr = (const uint64_t *)(b + off[46]);
        for (i = 0; i < p->n_elements; i++) {
                const char * e = b + (int64_t)(eptr[i] - base) + 528;
                memcpy(&p->element[i].Z, e, 8);
                memcpy(&p->element[i].A, e + 8, 8);
                memcpy(&p->element[i].I, e + 16, 8);
                memcpy(&p->element[i].index, e + 24, 4);
        }
        /* Compositions: struct material_component {int element;
         * double fraction;} (pumas.c:527-532). */
        p->comp_start = calloc(p->n_materials, sizeof(int));
        p->comp_element = calloc(p->n_components, sizeof(int));
        p->comp_fraction = calloc(p->n_components, sizeof(double));
        const uint64_t * cptr = (const uint64_t *)(b + off[47]);
        int ic = 0;
        for (i = 0; i < p->n_materials; i++) {
                p->comp_start[i] = ic;
                const char * c = b + (int64_t)(cptr[i] - base) + 528;
                int j;
                for (j = 0; j < p->elements_in[i]; j++, ic++) {
                        memcpy(p->comp_element + ic, c + 16 * j, 4);
                        memcpy(p->comp_fraction + ic, c + 16 * j + 8, 8);
                }
        }
        p->material_name = calloc(p->n_materials, sizeof(char *));
        const uint64_t * nptr = (const uint64_t *)(b + off[49]);
        for (i = 0; i < p->n_materials; i++)
                p->material_name[i] = b + (int64_t)(nptr[i] - base) + 528;
        /* The restated DCS models. */
        const char * brems = b + off[50];
        const char * pair = b + off[51];
        p->model_brems = (strcmp(brems, "SSR") == 0) ? 0 :
            (strcmp(brems, "KKP") == 0) ? 1 :
            (strcmp(brems, "ABB") == 0) ? 2 : -1;
        p->model_pair = (strcmp(pair, "SSR") == 0) ? 0 :
            (strcmp(pair, "KKP") == 0) ? 1 : -1;
        const char * photo = b + off[52];
        p->model_photo = (strcmp(photo, "DRSS") == 0) ? 0 :
            (strcmp(photo, "BBKS") == 0) ? 1 :
            (strcmp(photo, "BM") == 0) ? 2 : -1;
        if ((p->model_brems < 0) || (p->model_pair < 0) ||
            (p->model_photo < 0) ||
            ((p->particle != 0) && (p->particle != 1))) {
                port_free(p);
                return RC_MODEL_ERROR;
        }
        port_free(ph);
        ph = p;
        return RC_SUCCESS;
}

int oracle_port_material_index(const char * name, int * index)
{
        if (ph == NULL) return RC_PHYSICS_ERROR;
        int i;
        for (i = 0; i < ph->n_materials; i++) {
                if (strcmp(ph->material_name[i], name) == 0) {
                        *index = i;
                        return RC_SUCCESS;
                }
        }
        return RC_UNKNOWN_MATERIAL;
}

/* Table accessors (pumas.c:4260-4752): scheme clamping rules. */
static inline int sch(int scheme)
{
        return (scheme > MODE_MIXED) ? MODE_MIXED : scheme;
}
#define ROW(s, m) ((long)((s) * ph->n_materials + (m)) * ph->n_energies)
#define MROW(m) ((long)(m) * ph->n_energies)

/* table_index + table_bracket (pumas.c:4174-4233), without the per context
 * cache of the last indices, which never changes the result. */
static int table_index(const double * table, double value)
{
        const int imax = ph->n_energies - 1;
        if (value < table[0]) return -1;
        if (value >= table[imax]) return imax;
        int i1 = 0, i2 = imax;
        do {
                const int i3 = (i1 + i2) / 2;
                if (value >= table[i3])
                        i1 = i3;
                else
                        i2 = i3;
        } while (i2 - i1 >= 2);
        return i1;
}

/* math_pchip_interpolate (pumas.c:4118-4125). */
static double pchip(double t, double p0, double p1, double m0, double m1)
{
        const double c2 = -3 * (p0 - p1) - 2 * m0 - m1;
        const double c3 = 2 * (p0 - p1) + m0 + m1;
        return p0 + t * (m0 + t * (c2 + t * c3));
}

/* table_interpolate_pchip (pumas.c:4146-4157). */
static double interpolate(
    const double * X, const double * Y, const double * M, double x)
{
        const int i1 = table_index(X, x);
        const int i2 = i1 + 1;
        const double dX = X[i2] - X[i1];
        const double t = (x - X[i1]) / dX;
        const double m1 = M[i1] * dX;
        const double m2 = (i2 > 1) ? M[i2] * dX : m1;
        return pchip(t, Y[i1], Y[i2], m1, m2);
}

/* ------------------------------------------------------------------------ */
/* CEL, DEL and EHS interpolants (pumas.c:3644-4111, 7446-7466).            */
/* ------------------------------------------------------------------------ */
static double cel_grammage(int scheme, int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        if (kinetic < ph->K[0]) return 0.;
        const int s = sch(scheme);
        if (kinetic >= ph->K[imax]) {
                const double a = ph->a_max[material];
                const double b = ph->b_max[s * ph->n_materials + material];
                const double K0 = ph->K[imax];
                const double K1 = a / b + ph->mass;
                return ph->X[ROW(s, material) + imax] +
                    1. / b * log((kinetic + K1) / (K0 + K1));
        }
        return interpolate(ph->K, ph->X + ROW(s, material),
            ph->X_dK + ROW(s, material), kinetic);
}

static double cel_grammage_as_time(int scheme, int material, double time)
{
        const int imax = ph->n_energies - 1;
        const int s = sch(scheme);
        const double * T = ph->T + ROW(s, material);
        if (time < T[0]) return 0.;
        if (time >= T[imax]) {
                const double a = ph->a_max[material];
                const double b = ph->b_max[s * ph->n_materials + material];
                const double E0 = ph->K[imax] + ph->mass;
                const double tmax = T[imax];
                const double r =
                    E0 / (a + b * E0) * exp(a * (time - tmax) / ph->mass);
                const double kinetic = a * r / (1. - b * r) - ph->mass;
                const double K1 = a / b + ph->mass;
                return ph->X[ROW(s, material) + imax] +
                    1. / b * log((kinetic + K1) / (E0 - ph->mass + K1));
        }
        return interpolate(T, ph->X + ROW(s, material),
            ph->X_dT + ROW(s, material), time);
}

static double cel_proper_time(int scheme, int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        if (kinetic < ph->K[0]) return 0.;
        const int s = sch(scheme);
        if (kinetic >= ph->K[imax]) {
                const double a = ph->a_max[material];
                const double b = ph->b_max[s * ph->n_materials + material];
                const double E0 = ph->K[imax] + ph->mass;
                const double E1 = kinetic + ph->mass;
                return ph->T[ROW(s, material) + imax] +
                    ph->mass / a * log((E1 / E0) * (a + b * E0) / (a + b * E1));
        }
        return interpolate(ph->K, ph->T + ROW(s, material),
            ph->T_dK + ROW(s, material), kinetic);
}

static double cel_kinetic_energy(int scheme, int material, double grammage)
{
        const int imax = ph->n_energies - 1;
        const int s = sch(scheme);
        const double * X = ph->X + ROW(s, material);
        if (grammage < X[0]) return 0.;
        if (grammage >= X[imax]) {
                const double a = ph->a_max[material];
                const double b = ph->b_max[s * ph->n_materials + material];
                const double K0 = ph->K[imax];
                const double K1 = a / b + ph->mass;
                return (K0 + K1) * exp(b * (grammage - X[imax])) - K1;
        }
        return interpolate(X, ph->K, ph->K_dX + ROW(s, material), grammage);
}

static double cel_energy_loss(int scheme, int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        if (kinetic < ph->K[0]) return 0.;
        const int s = sch(scheme);
        if (kinetic >= ph->K[imax]) {
                return ph->a_max[material] +
                    ph->b_max[s * ph->n_materials + material] *
                    (kinetic + ph->mass);
        }
        return interpolate(ph->K, ph->dE + ROW(s, material),
            ph->dE_dK + ROW(s, material), kinetic);
}

static double cel_straggling(int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        if (kinetic < ph->K[0]) return 0.;
        const double Kmax = ph->K[imax];
        if (kinetic >= Kmax) {
                const double r = (kinetic + ph->mass) / (Kmax + ph->mass);
                return ph->Omega[MROW(material) + imax] * r * r;
        }
        return interpolate(ph->K, ph->Omega + MROW(material),
            ph->Omega_dK + MROW(material), kinetic);
}

static double del_cross_section(int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        if (kinetic < ph->K[0]) return 0.;
        if (kinetic >= ph->K[imax]) return ph->CS[MROW(material) + imax];
        return interpolate(ph->K, ph->CS + MROW(material),
            ph->CS_dK + MROW(material), kinetic);
}

static double del_interaction_length(int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        if (kinetic < ph->K[0]) return 0.;
        if (kinetic >= ph->K[imax]) {
                const double k0 = ph->K[imax];
                const double a0 = ph->a_max[material];
                const double b0 = ph->b_max[ph->n_materials + material];
                const double cs = ph->CS[MROW(material) + imax];
                const double dZ =
                    cs / b0 * log((a0 + b0 * (kinetic + ph->mass)) /
                                  (a0 + b0 * (k0 + ph->mass)));
                return ph->NI_in[MROW(material) + imax] + dZ;
        }
        return interpolate(ph->K, ph->NI_in + MROW(material),
            ph->NI_in_dK + MROW(material), kinetic);
}

static double del_kinetic_from_interaction_length(int material, double nI)
{
        const int imax = ph->n_energies - 1;
        const double * NI = ph->NI_in + MROW(material);
        if (nI < NI[0]) return 0.;
        if (nI >= NI[imax]) {
                const double k0 = ph->K[imax];
                const double a0 = ph->a_max[material];
                const double b0 = ph->b_max[ph->n_materials + material];
                const double cs = ph->CS[MROW(material) + imax];
                const double nI0 = NI[imax];
                return ((a0 + b0 * (k0 + ph->mass)) *
                               exp(b0 * (nI - nI0) / cs) -
                           a0) /
                    b0 -
                    ph->mass;
        }
        return interpolate(NI, ph->K, ph->K_dNI_in + MROW(material), nI);
}

static inline int sch_el(int scheme)
{
        return (scheme >= MODE_MIXED) ? MODE_MIXED : MODE_CSDA;
}

static double ehs_interaction_length(int scheme, int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        if (kinetic < ph->K[0]) return 0.;
        const double * NI = ph->NI_el + ROW(sch_el(scheme), material);
        if (kinetic >= ph->K[imax]) {
                const double k0 = ph->K[imax - 1];
                const double k1 = ph->K[imax];
                const double nI0 = NI[imax - 1];
                const double nI1 = NI[imax];
                return nI1 + (kinetic - k1) * (nI1 - nI0) / (k1 - k0);
        }
        return interpolate(ph->K, NI,
            ph->NI_el_dK + ROW(sch_el(scheme), material), kinetic);
}

static double ehs_kinetic_from_interaction_length(
    int scheme, int material, double nI)
{
        const int imax = ph->n_energies - 1;
        const double * NI = ph->NI_el + ROW(sch_el(scheme), material);
        if (nI < NI[0]) return 0.;
        if (nI >= NI[imax]) {
                const double k0 = ph->K[imax - 1];
                const double k1 = ph->K[imax];
                const double nI0 = NI[imax - 1];
                const double nI1 = NI[imax];
                return k1 + (nI - nI1) * (k1 - k0) / (nI1 - nI0);
        }
        return interpolate(NI, ph->K,
            ph->K_dNI_el + ROW(sch_el(scheme), material), nI);
}

/* table_get_msc (pumas.c:4077-4111); Ms1 rows are offset by one scheme. */
static void table_get_msc(int energy_loss, int material, double kinetic,
    double * mu0, double * invlb1)
{
        const int imax = ph->n_energies - 1;
        const int s = sch(energy_loss);
        const double * Mu0 = ph->Mu0 + MROW(material);
        const double * Ms1 = ph->Ms1 + ROW(s + 1, material);
        if (kinetic < ph->K[1]) {
                *mu0 = Mu0[1];
                *invlb1 = Ms1[1] * sqrt(ph->K[1] / kinetic);
        } else if (kinetic >= ph->K[imax]) {
                *mu0 = Mu0[imax];
                *invlb1 = Ms1[imax] * ph->K[imax] / kinetic;
        } else {
                const double * x = ph->K;
                const int i1 = table_index(x, kinetic);
                x += i1;
                const double * y0 = Mu0 + i1;
                const double * m0 = ph->Mu0_dK + MROW(material) + i1;
                const double * y1 = Ms1 + i1;
                const double * m1 = ph->Ms1_dK + ROW(s + 1, material) + i1;
                const double dx = x[1] - x[0];
                const double t = (kinetic - x[0]) / dx;
                *mu0 = pchip(t, y0[0], y0[1], m0[0] * dx, m0[1] * dx);
                *invlb1 = pchip(t, y1[0], y1[1], m1[0] * dx, m1[1] * dx);
        }
}

static double coulomb_ehs_length(int material, double kinetic)
{
        const double p2 = kinetic * (kinetic + 2. * ph->mass);
        const int imax = ph->n_energies - 1;
        const double * Lb = ph->Lb + MROW(material);
        if (kinetic < ph->K[1]) {
                return Lb[1] / p2;
        } else if (kinetic >= ph->K[imax]) {
                return Lb[imax] / p2;
        } else {
                const int i1 = table_index(ph->K, kinetic);
                const int i2 = i1 + 1;
                double h = (kinetic - ph->K[i1]) / (ph->K[i2] - ph->K[i1]);
                return (Lb[i1] + h * (Lb[i2] - Lb[i1])) / p2;
        }
}

/* ------------------------------------------------------------------------ */
/* Per event context (the relevant part of struct simulation_context,       */
/* pumas.c:426-477, plus the stepping locals of pumas.c:5235-5262).         */
/* ------------------------------------------------------------------------ */
struct port_ctx {
        const struct oracle_config * cfg;
        const struct gpumas_geometry * geometry;
        struct oracle_stream rng;
        double lifetime;
        int step_first;
        int step_event;
        int step_foreseen;
        double step_X_limit;
        double step_invlb1;
        int randn_done;
        double randn_next;
        int steps;
        /* Field of the current medium (struct medium_locals,
         * pumas.c:396-403). */
        double magnet[3];
        int magnetized;
};

static inline double rnd(struct port_ctx * c)
{
        return oracle_stream_draw(&c->rng);
}

/* Medium callback equivalent: locate and step proposal. */
static int medium_locate(struct port_ctx * c, const struct oracle_state * s)
{
        return gpumas_geometry_locate(c->geometry, s->position);
}

static double medium_step(
    struct port_ctx * c, const struct oracle_state * s, int medium)
{
        const double sgn =
            (c->cfg->direction == MODE_FORWARD) ? 1. : -1.;
        const double u[3] = { sgn * s->direction[0], sgn * s->direction[1],
                sgn * s->direction[2] };
        c->steps++;
        return gpumas_geometry_step(c->geometry, s->position, u, medium);
}

/* transport_set_locals (pumas.c:5528-5552) for a uniform medium. */
static double medium_density(const struct port_ctx * c, int medium)
{
        const struct gpumas_medium * m = c->geometry->media + medium;
        return (m->density > 0.) ? m->density :
                                   ph->material_density[m->material];
}

static inline int medium_material(const struct port_ctx * c, int medium)
{
        return c->geometry->media[medium].material;
}

/* transport_set_locals (pumas.c:5528-5552) with the locals callback of the
 * media's descriptors (struct gpumas_locals), evaluated as the reference
 * harness's callback does: sets *density and the field, returns the step
 * limit (0 for a uniform medium). */
static double set_locals(struct port_ctx * c, int medium,
    const struct oracle_state * s, double * density)
{
        const struct gpumas_locals * l = c->geometry->locals;
        c->magnet[0] = c->magnet[1] = c->magnet[2] = 0.;
        c->magnetized = 0;
        if (l == NULL) {
                *density = medium_density(c, medium);
                return 0.;
        }
        l += medium;
        double size = 0.;
        *density = c->geometry->media[medium].density;
        if (l->model == GPUMAS_DENSITY_EXPONENTIAL) {
                *density = l->rho0 * gp_exp(gpumas_locals_exponent(l,
                                         s->position));
                size = gpumas_locals_size(l, s->direction);
        }
        if (*density <= 0.)
                *density = ph->material_density[medium_material(c, medium)];
        memcpy(c->magnet, l->magnet, sizeof(c->magnet));
        c->magnetized = ((l->magnet[0] != 0.) || (l->magnet[1] != 0.) ||
                            (l->magnet[2] != 0.)) ? 1 : 0;
        return size * c->cfg->accuracy;
}

/* ------------------------------------------------------------------------ */
/* Deterministic CSDA transport in an infinite uniform medium, with the     */
/* closed form deflection of a uniform field (pumas.c:3849-3883,            */
/* 4777-5171).                                                              */
/* ------------------------------------------------------------------------ */
/* cel_magnetic_rotation (pumas.c:3849-3883). */
static double cel_magnetic_rotation(int material, double kinetic)
{
        const int imax = ph->n_energies - 1;
        const double factor = LARMOR_FACTOR / ph->mass;
        const double * T = ph->T + ROW(0, material);
        if (kinetic <= ph->K[0]) return T[imax] * factor;
        if (kinetic >= ph->K[imax]) return 0.;
        const double t = interpolate(ph->K, T, ph->T_dK + ROW(0, material),
            kinetic);
        return (T[imax] - t) * factor;
}

/* csda_magnetic_transport (pumas.c:5095-5171), with the reference's
 * polynomial fits of cos and sin. */
static int csda_magnetic_transport(int material, double density,
    double magnet, double charge, double kinetic, double phase, double * x,
    double * y, double * z)
{
        const int imax = ph->n_energies - 1;
        double k0 = kinetic;
        int i1, i2;
        if (kinetic <= ph->K[0]) {
                k0 = ph->K[0];
                i1 = 0;
                i2 = 1;
        } else if (kinetic >= ph->K[imax]) {
                *y = 0.0;
                *x = *z = -(cel_grammage(MODE_CSDA, material, kinetic) -
                    ph->X[ROW(0, material) + imax]);
                return RC_SUCCESS;
        } else {
                i1 = table_index(ph->K, k0);
                i2 = i1 + 1;
        }
        static const double poly_x[8] = { 1.000000000e+000, 0.000000000e+000,
                -5.000000000e-001, -1.048969541e-002, 5.597396438e-002,
                -6.401353612e-003, -4.495849930e-004, 6.583532135e-005 };
        static const double poly_y[8] = { 0.000000000e+000, 1.000000000e+000,
                -1.400755143e-002, -1.350173383e-001, -2.838778336e-002,
                2.123237056e-002, -3.094290091e-003, 1.409012754e-004 };
        if (fabs(phase) > 2.0 * PI_) return RC_VALUE_ERROR;
        const double * L = ph->Li + (long)material * 8 * ph->n_energies;
        const double a = -magnet * charge / density;
        double x1 = 0., x2 = 0., y1 = 0., y2 = 0., u = 1.;
        int j;
        for (j = 0; j < 8; j++) {
                const double l1 = L[j * ph->n_energies + i1];
                const double l2 = L[j * ph->n_energies + i2];
                x1 += u * poly_x[j] * l1;
                y1 += u * poly_y[j] * l1;
                x2 += u * poly_x[j] * l2;
                y2 += u * poly_y[j] * l2;
                u *= a;
        }
        const double z1 = L[i1], z2 = L[i2];
        const double h = (k0 - ph->K[i1]) / (ph->K[i2] - ph->K[i1]);
        *x = (x1 + h * (x2 - x1)) / density;
        *y = (y1 + h * (y2 - y1)) / density;
        *z = (z1 + h * (z2 - z1)) / density;
        return RC_SUCCESS;
}

/* transport_csda_deflect (pumas.c:4968-5075). */
static int csda_deflect(struct port_ctx * c, struct oracle_state * state,
    int material, double density, double ki, double distance)
{
        const double charge = state->charge;
        const double kf = state->energy;
        double * const position = state->position;
        double * const direction = state->direction;
        const double * const m = c->magnet;
        const double b0 = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        const double b0_i = 1.0 / b0;
        double ex[3], ey[3], ez[3];
        ey[0] = (direction[2] * m[1] - direction[1] * m[2]) * b0_i;
        ey[1] = (direction[0] * m[2] - direction[2] * m[0]) * b0_i;
        ey[2] = (direction[1] * m[0] - direction[0] * m[1]) * b0_i;
        const double d = b0_i * b0_i * (m[0] * direction[0] +
                                           m[1] * direction[1] +
                                           m[2] * direction[2]);
        int k;
        for (k = 0; k < 3; k++) {
                ez[k] = m[k] * d;
                ex[k] = direction[k] - ez[k];
        }
        const double a = -b0 * charge / density;
        const double pi = a * cel_magnetic_rotation(material, ki);
        const double pf = a * cel_magnetic_rotation(material, kf);
        const double dp = pf - pi;
        const double ps = fabs(pi + pf);
        if (ps == 0.) return RC_SUCCESS;
        const double dp0 = fabs(dp);
        double dx, dy, dz;
        if ((dp0 < 1E-02) && (dp0 / ps < 1E-02)) {
                dz = (ki >= kf) ? distance : -distance;
                const double sixth = 1 / 6.0;
                dx = dz * (1.0 - sixth * dp * dp);
                dy = 0.5 * dz * dp;
        } else {
                double xi, yi, zi, xf, yf, zf;
                int rc = csda_magnetic_transport(material, density, b0, charge,
                    ki, pi, &xi, &yi, &zi);
                if (rc != RC_SUCCESS) return rc;
                rc = csda_magnetic_transport(material, density, b0, charge, kf,
                    pf, &xf, &yf, &zf);
                if (rc != RC_SUCCESS) return rc;
                const double si = sin(pi);
                const double ci = cos(pi);
                xf -= xi;
                yf -= yi;
                dx = ci * xf + si * yf;
                dy = -si * xf + ci * yf;
                dz = zf - zi;
        }
        for (k = 0; k < 3; k++)
                position[k] += dx * ex[k] + dy * ey[k] + dz * ez[k];
        const double sn = sin(dp);
        const double cs = cos(dp);
        for (k = 0; k < 3; k++)
                direction[k] = cs * ex[k] + sn * ey[k] + ez[k];
        return RC_SUCCESS;
}

/* transport_with_csda (pumas.c:4777-4949): with a field, the closed form
 * deflection; *status gets its return code. */
static int transport_with_csda(struct port_ctx * c, struct oracle_state * state,
    int material, double density, int * status)
{
        const struct oracle_config * cfg = c->cfg;
        const double ki = state->energy;
        const double di = state->distance;
        const double ti = state->time;
        const double xi = cel_grammage(MODE_CSDA, material, ki);
        const double Ti = cel_proper_time(MODE_CSDA, material, ki);

        int event = EV_NONE;
        double xB;
        if (cfg->event & EV_LIMIT_GRAMMAGE) {
                xB = cfg->limit_grammage - state->grammage;
                event = EV_LIMIT_GRAMMAGE;
        } else
                xB = DBL_MAX;
        if (cfg->event & EV_LIMIT_DISTANCE) {
                const double xD = density * (cfg->limit_distance - di);
                if (xD < xB) {
                        xB = xD;
                        event = EV_LIMIT_DISTANCE;
                }
        }
        int decayed = 0;
        double time_max =
            (cfg->event & EV_LIMIT_TIME) ? cfg->limit_time : 0.;
        if (cfg->decay == MODE_RANDOMISED) {
                if ((time_max <= 0.) || (c->lifetime < time_max)) {
                        time_max = c->lifetime;
                        decayed = 1;
                }
        }
        if (time_max > 0.) {
                const double dt = time_max - ti;
                if (dt <= 0.) {
                        xB = 0.;
                        event = EV_LIMIT_TIME;
                } else {
                        const double sgn =
                            (cfg->direction == MODE_FORWARD) ? 1. : -1.;
                        const double Tf = Ti - sgn * dt * density;
                        if (Tf > 0.) {
                                const double xT = fabs(xi -
                                    cel_grammage_as_time(
                                        MODE_CSDA, material, Tf));
                                if (xT < xB) {
                                        xB = xT;
                                        event = EV_LIMIT_TIME;
                                }
                        }
                }
        }
        if (xB <= 0.) return event;

        double xf, kf;
        if (cfg->direction == MODE_FORWARD) {
                if (xi > xB) {
                        xf = xi - xB;
                        if (xB < EPSILON_X * xi) {
                                kf = ki - cel_energy_loss(
                                    MODE_CSDA, material, ki) * xB;
                                if (kf < 0.) kf = 0.;
                        } else {
                                kf = cel_kinetic_energy(
                                    MODE_CSDA, material, xf);
                        }
                } else {
                        xf = kf = 0.;
                        event = EV_LIMIT_ENERGY;
                }
                if (cfg->event & EV_LIMIT_ENERGY) {
                        if (ki <= cfg->limit_energy) return EV_LIMIT_ENERGY;
                        if (kf < cfg->limit_energy) {
                                kf = cfg->limit_energy;
                                xf = cel_grammage(MODE_CSDA, material, kf);
                                event = EV_LIMIT_ENERGY;
                        }
                }
        } else {
                if (xB == DBL_MAX) {
                        xf = xB;
                        kf = DBL_MAX;
                } else {
                        xf = xB + xi;
                        if (xB < EPSILON_X * xi) {
                                kf = ki + cel_energy_loss(
                                    MODE_CSDA, material, ki) * xB;
                        } else {
                                kf = cel_kinetic_energy(
                                    MODE_CSDA, material, xf);
                        }
                }
                if (cfg->event & EV_LIMIT_ENERGY) {
                        if (ki >= cfg->limit_energy) return EV_LIMIT_ENERGY;
                        if (kf > cfg->limit_energy) {
                                kf = cfg->limit_energy;
                                xf = cel_grammage(MODE_CSDA, material, kf);
                                event = EV_LIMIT_ENERGY;
                        }
                }
        }

        const double distance = fabs(xf - xi) / density;
        state->energy = kf;
        if (event == EV_LIMIT_DISTANCE)
                state->distance = cfg->limit_distance;
        else
                state->distance += distance;
        if (event == EV_LIMIT_GRAMMAGE)
                state->grammage = cfg->limit_grammage;
        else
                state->grammage += distance * density;
        if (event == EV_LIMIT_TIME) {
                state->time = time_max;
                state->decayed = decayed;
                if (decayed) event = EV_DECAY;
        } else
                state->time += fabs(Ti -
                    cel_proper_time(MODE_CSDA, material, kf)) / density;
        if (cfg->direction == MODE_BACKWARD)
                state->weight *= cel_energy_loss(MODE_CSDA, material, kf) /
                    cel_energy_loss(MODE_CSDA, material, ki);
        if (cfg->decay == MODE_WEIGHTED)
                state->weight *= exp(-fabs(ti - state->time) / ph->ctau);

        if (c->magnetized) {
                *status = csda_deflect(c, state, material, density, ki,
                    distance);
                return event;
        }
        const double path =
            (cfg->direction == MODE_FORWARD) ? distance : -distance;
        state->position[0] += path * state->direction[0];
        state->position[1] += path * state->direction[1];
        state->position[2] += path * state->direction[2];
        return event;
}

/* ------------------------------------------------------------------------ */
/* Random helpers (pumas.c:7016-7095).                                      */
/* ------------------------------------------------------------------------ */
static double step_randn(struct port_ctx * c)
{
        c->randn_done = !c->randn_done;
        if (!c->randn_done) return c->randn_next;
        const double r = sqrt(-2. * log(rnd(c)));
        const double phi = 2. * PI_ * rnd(c);
        const double co = cos(phi);
        const double si = sin(phi);
        c->randn_next = r * co;
        return r * si;
}

static void step_rotate_direction(
    struct port_ctx * c, struct oracle_state * state, double mu)
{
        double * const direction = state->direction;
        const double cos_theta = 1 - 2 * mu;
        const double stsq = 4 * mu * (1. - mu);
        if (stsq <= 0.) return;
        const double st = sqrt(stsq);

        double u0x = 0., u0y = 0., u0z = 0.;
        const double a0 = fabs(direction[0]);
        const double a1 = fabs(direction[1]);
        const double a2 = fabs(direction[2]);
        if (a0 > a1) {
                if (a0 > a2) {
                        const double nrm =
                            1. / sqrt(direction[0] * direction[0] +
                                     direction[2] * direction[2]);
                        u0x = -direction[2] * nrm, u0z = direction[0] * nrm;
                } else {
                        const double nrm =
                            1. / sqrt(direction[1] * direction[1] +
                                     direction[2] * direction[2]);
                        u0y = direction[2] * nrm, u0z = -direction[1] * nrm;
                }
        } else {
                if (a1 > a2) {
                        const double nrm =
                            1. / sqrt(direction[0] * direction[0] +
                                     direction[1] * direction[1]);
                        u0x = direction[1] * nrm, u0y = -direction[0] * nrm;
                } else {
                        const double nrm =
                            1. / sqrt(direction[1] * direction[1] +
                                     direction[2] * direction[2]);
                        u0y = direction[2] * nrm, u0z = -direction[1] * nrm;
                }
        }
        const double u1x = u0y * direction[2] - u0z * direction[1];
        const double u1y = u0z * direction[0] - u0x * direction[2];
        const double u1z = u0x * direction[1] - u0y * direction[0];

        const double phi = PI_ * (1. - 2. * rnd(c));
        const double cp = cos(phi);
        const double sp = sin(phi);
        direction[0] = cos_theta * direction[0] + st * (cp * u0x + sp * u1x);
        direction[1] = cos_theta * direction[1] + st * (cp * u0y + sp * u1y);
        direction[2] = cos_theta * direction[2] + st * (cp * u0z + sp * u1z);
}

/* ------------------------------------------------------------------------ */
/* Coulomb scattering (pumas.c:7143-7683).                                  */
/* ------------------------------------------------------------------------ */

/* Nuclear r.m.s. charge radii in fm, indexed as in data_nuclear_radius
 * (pumas.c:7143-7175): entry 0 is deuterium-like hydrogen, entry Z is
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

static double data_nuclear_radius(double Z, double A)
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

/* Atomic screening of Salvat et al. (1987), one row per element Z = 1..103:
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

/* coulomb_screening_parameters (pumas.c:7203-7387). */
static void coulomb_screening_parameters(double Z, double A, double mass,
    double kinetic, double kinetic0, int * n_parameters, double * amplitude,
    double * screening)
{
        const double aZE = ALPHA_EM * Z * (kinetic + mass);
        const double p2 = kinetic * (kinetic + 2. * mass);
        const double zeta2 = aZE * aZE / p2;
        double f;
        if (zeta2 < 1) {
                f = 1. / (1. + zeta2) + 0.20205690315959424 -
                    0.03692775514336999 * zeta2 +
                    0.008349277381922926 * zeta2 * zeta2;
                f *= zeta2;
        } else {
                const double r2i = 1. / (1. + zeta2);
                const double phi = -atan(sqrt(zeta2));
                f = -0.5 * log(r2i) + 0.5 * (1. - r2i) +
                    1. / 12. * (1. - cos(2 * phi) * r2i) -
                    1. / 120. * (1. - cos(4 * phi) * r2i * r2i) +
                    1. / 252. * (1. - cos(6 * phi) * r2i * r2i * r2i);
        }
        const double ktv = exp(2 * f);

        const double p02 = kinetic0 * (kinetic0 + 2. * mass);
        const double d = 0.25 * HBAR_C * HBAR_C / p02 * ktv;
        int iZ = (int)Z - 1;
        if (iZ >= 103) iZ = 102;
        const double * row = salvat_screening[iZ];
        int n;
        if (row[4] == 1.) {
                if (iZ == 0) {
                        n = 1;
                        amplitude[0] = 1.;
                } else {
                        n = 2;
                        amplitude[0] = row[0];
                        amplitude[1] = 1. - amplitude[0];
                }
        } else {
                n = 3;
                amplitude[0] = row[0];
                amplitude[1] = row[1];
                amplitude[2] = 1. - (amplitude[0] + amplitude[1]);
        }
        int i;
        for (i = 0; i < n; i++) {
                const double a = row[2 + i] / BOHR_RADIUS;
                screening[i] = d * a * a;
        }
        const double RN = data_nuclear_radius(Z, A);
        screening[n++] = 12. * d / (RN * RN);
        *n_parameters = n;
}

/* coulomb_nuclear_form_factor (pumas.c:7396-7416). */
static double coulomb_nuclear_form_factor(double mu, double N)
{
        if (mu <= 0.)
                return 1.;
        else if (mu > 1.)
                return 0.;
        const double x2 = 10. * mu / N;
        double d;
        if (x2 <= 1E-04) {
                d = 1. / (1. + 0.1 * x2);
        } else {
                const double x = sqrt(x2);
                d = 3 * (sin(x) - x * cos(x)) / (x2 * x);
        }
        return d * d;
}

/* coulomb_normalisation (pumas.c:7428-7435). */
static double coulomb_normalisation(
    double Z, double A, double mass, double kinetic, double kinetic0)
{
        const double p2 = kinetic * (kinetic + 2. * mass);
        const double p02 = kinetic0 * (kinetic0 + 2. * mass);
        double d = ALPHA_EM * Z * HBAR_C * (kinetic + mass);
        return A * 1E-03 * p2 * p02 / (d * d * PI_ * AVOGADRO_NUMBER);
}

/* coulomb_spin_factor (pumas.c:7475-7479). */
static double coulomb_spin_factor(double mass, double kinetic)
{
        const double e = kinetic + mass;
        return kinetic * (e + mass) / (e * e);
}

/* coulomb_frame_parameters (pumas.c:7492-7508). */
static void coulomb_frame_parameters(double Z, double A, double mass,
    double kinetic, double * kinetic0, double * parameters)
{
        const double Ma = Z * PROTON_MASS + (A - Z) * NEUTRON_MASS;
        double M2 = mass + Ma;
        M2 *= M2;
        const double sCM12i = 1. / sqrt(M2 + 2. * Ma * kinetic);
        parameters[0] = (kinetic + mass + Ma) * sCM12i;
        *kinetic0 = (kinetic * Ma + mass * (mass + Ma)) * sCM12i - mass;
        if (*kinetic0 < 1E-09) *kinetic0 = 1E-09;
        const double etot = kinetic + mass + Ma;
        const double betaCM2 = kinetic * (kinetic + 2. * mass) / (etot * etot);
        double rM2 = mass / Ma;
        rM2 *= rM2;
        parameters[1] = sqrt(rM2 * (1. - betaCM2) + betaCM2);
}

/* coulomb_pole_reduction (pumas.c:7524-7576), in extended precision. */
static void coulomb_pole_reduction(int n_parameters, const double * amplitude,
    const double * screening, coulomb_real * a, coulomb_real * b,
    coulomb_real * c)
{
        const int n = n_parameters - 1;
        int i, j;
        for (i = 0; i < n; i++) a[i] = b[i] = 0;
        for (i = 0; i < 4; i++) c[i] = 0;
        for (i = 0; i < n; i++) {
                const coulomb_real Ai = amplitude[i];
                const coulomb_real Bi = screening[i];
                b[i] = Ai * Ai;
                for (j = i + 1; j < n; j++) {
                        const coulomb_real Aj = amplitude[j];
                        const coulomb_real Bj = screening[j];
                        const coulomb_real d = 2 * Ai * Aj / (Bj - Bi);
                        a[i] += d;
                        a[j] -= d;
                }
        }
        const coulomb_real N = screening[n];
        coulomb_real Sa[4] = { 0, 0, 0, 0 }, Sb[4] = { 0, 0, 0, 0 };
        for (i = 0; i < n; i++) {
                const coulomb_real Bi = screening[i];
                const coulomb_real x = 1. - Bi / N;
                coulomb_real r = x;
                for (j = 0; j < 4; j++) {
                        Sa[j] += a[i] / r;
                        r *= x;
                        Sb[j] += b[i] / r;
                }
        }
        coulomb_real tmp = 1;
        for (i = 0; i < 4; i++) {
                c[i] = ((4 - i) * Sb[3 - i] / N - Sa[3 - i]) * tmp;
                tmp *= N;
        }
        for (i = 0; i < n; i++) {
                const coulomb_real Bi = screening[i];
                coulomb_real d = 1. - Bi / N;
                d *= d;
                d *= d;
                a[i] = (a[i] - 4 * b[i] / (N - Bi)) / d;
                b[i] /= d;
        }
}

/* coulomb_transport_coefficients (pumas.c:7623-7683). */
static void coulomb_transport_coefficients(double mu_, double fspin,
    int n_parameters, const double * screening, const coulomb_real * a,
    const coulomb_real * b, const coulomb_real * c, double * coefficient)
{
        const coulomb_real S = fspin;
        const coulomb_real mu = mu_;
        const int n = n_parameters - 1;
        double cs0 = 0., cs1 = 0.;
        int i;
        for (i = 0; i < n; i++) {
                const coulomb_real alp = screening[i];
                const coulomb_real r = mu / (mu + alp);
                const coulomb_real L = coulomb_log(1. + mu / alp);
                const coulomb_real I0 = r / alp;
                const coulomb_real J0 = L;
                const coulomb_real I1 = L - r;
                const coulomb_real J1 = -alp * L;
                const coulomb_real I2 = mu + alp * (r - 2. * L);
                const coulomb_real J2 = alp * (alp * L - mu);
                cs0 += a[i] * (J0 - S * J1) + b[i] * (I0 - S * I1);
                cs1 += a[i] * (J1 - S * J2) + b[i] * (I1 - S * I2);
        }
        const coulomb_real N = screening[n];
        const coulomb_real r = mu / (mu + N);
        const coulomb_real L = coulomb_log(1. + mu / N);
        const coulomb_real I0 = r / N;
        const coulomb_real J0 = L;
        const coulomb_real I1 = L - r;
        const coulomb_real J1 = -N * L;
        const coulomb_real I2 = mu + N * (r - 2. * L);
        const coulomb_real J2 = N * (N * L - mu);
        const coulomb_real rn = 1. / (1. + mu / N);
        const coulomb_real K0 = (1. - rn) * (1. + rn) / (2 * N * N);
        const coulomb_real L0 =
            (1. - rn) * ((1. + rn) * (1. + rn) - rn) / (3 * N * N * N);
        const coulomb_real K1 = I0 - N * K0;
        const coulomb_real L1 = K0 - N * L0;
        const coulomb_real K2 = I1 - N * K1;
        const coulomb_real L2 = K1 - N * L1;
        cs0 += c[0] * (J0 - S * J1) + c[1] * (I0 - S * I1) +
            c[2] * (K0 - S * K1) + c[3] * (L0 - S * L1);
        cs1 += c[0] * (J1 - S * J2) + c[1] * (I1 - S * I2) +
            c[2] * (K1 - S * K2) + c[3] * (L1 - S * L2);
        coefficient[0] = cs0;
        coefficient[1] = 2 * cs1;
}

/* coulomb_restricted_cs (pumas.c:7591-7609). */
static double coulomb_restricted_cs(double mu, double fspin, int n_parameters,
    const double * screening, const coulomb_real * a, const coulomb_real * b,
    const coulomb_real * c)
{
        if ((mu >= 1.) || (mu >= 1E+06 * screening[n_parameters - 1]))
                return 0.;
        double coefficients[2];
        coulomb_transport_coefficients(
            1., fspin, n_parameters, screening, a, b, c, coefficients);
        const double cs0 = coefficients[0];
        coulomb_transport_coefficients(
            mu, fspin, n_parameters, screening, a, b, c, coefficients);
        if (coefficients[0] > cs0)
                return 0;
        else
                return cs0 - coefficients[0];
}

/* ------------------------------------------------------------------------ */
/* Numerical helpers (pumas.c:12105-12325, 12463-12673).                    */
/* ------------------------------------------------------------------------ */

/* Gauss-Legendre nodes and weights on [0, 1] for 9 and 12 points, as
 * tabulated in math_gauss_quad_coefficients (pumas.c:12463-12561). */
static const double gl9_x[9] = {
        0.0159198802461870, 0.0819844463366821, 0.1933142836497048,
        0.3378732882980955, 0.5000000000000000, 0.6621267117019045,
        0.8066857163502952, 0.9180155536633179, 0.9840801197538130,
};
static const double gl9_w[9] = {
        0.0406371941807872, 0.0903240803474287, 0.1303053482014677,
        0.1561735385200015, 0.1651196775006299, 0.1561735385200015,
        0.1303053482014677, 0.0903240803474287, 0.0406371941807872,
};
static const double gl12_x[12] = {
        0.0092196828766404, 0.0479413718147625, 0.1150486629028477,
        0.2063410228566913, 0.3160842505009099, 0.4373832957442655,
        0.5626167042557344, 0.6839157494990901, 0.7936589771433087,
        0.8849513370971523, 0.9520586281852375, 0.9907803171233596,
};
static const double gl12_w[12] = {
        0.0235876681932559, 0.0534696629976592, 0.0800391642716731,
        0.1015837133615330, 0.1167462682691774, 0.1245735229067014,
        0.1245735229067014, 0.1167462682691774, 0.1015837133615330,
        0.0800391642716731, 0.0534696629976592, 0.0235876681932559,
};

/* Chebyshev expansion of the dilogarithm, CERNLIB RDILOG (C332), as used by
 * math_dilog (pumas.c:12609-12673). */
static const double dilog_c[20] = {
        0.42996693560813697, 0.40975987533077105, -0.01858843665014592,
        0.00145751084062268, -0.00014304184442340, 0.00001588415541880,
        -0.00000190784959387, 0.00000024195180854, -0.00000003193341274,
        0.00000000434545063, -0.00000000060578480, 0.00000000008612098,
        -0.00000000001244332, 0.00000000000182256, -0.00000000000027007,
        0.00000000000004042, -0.00000000000000610, 0.00000000000000093,
        -0.00000000000000014, 0.00000000000000002,
};

static double math_dilog(double x)
{
        const double PI3 = PI_ * PI_ / 3.;
        const double PI6 = PI_ * PI_ / 6.;
        const double PI12 = PI_ * PI_ / 12.;
        if (x == 10) {
                return PI6;
        } else if ((x == -1.) || (1. - x == 0.)) {
                return -PI12;
        } else {
                double T = -x;
                double A, S, Y;
                if (T <= -2) {
                        Y = -1. / (1. + T);
                        S = 1.;
                        A = -PI3 + 0.5 * (pow(log(-T), 2.) -
                                             pow(log(1. + 1. / T), 2.));
                } else if (T < -1.) {
                        Y = -1. - T;
                        S = -1.;
                        A = log(-T);
                        A = -PI6 + A * (A + log(1. + 1. / T));
                } else if (T <= -0.5) {
                        Y = -(1. + T) / T;
                        S = 1.;
                        A = log(-T);
                        A = -PI6 + A * (-0.5 * A + log(1. + T));
                } else if (T < 0.) {
                        Y = -T / (1. + T);
                        S = -1.;
                        A = 0.5 * pow(log(1 + T), 2.);
                } else if (T <= 1.) {
                        Y = T;
                        S = 1.;
                        A = 0.;
                } else {
                        Y = 1. / T;
                        S = -1.;
                        A = PI6 + 0.5 * pow(log(T), 2);
                }
                const double H = Y + Y - 1;
                const double ALFA = H + H;
                double B0 = 0., B1 = 0., B2 = 0.;
                int i;
                for (i = 19; i >= 0; i--) {
                        B0 = dilog_c[i] + ALFA * B1 - B2;
                        B2 = B1;
                        B1 = B0;
                }
                return -(S * (B0 - H * B2) + A);
        }
}

/* ------------------------------------------------------------------------ */
/* Default DCS models.                                                      */
/* ------------------------------------------------------------------------ */

/* Radiation logarithms (Kelner, Kokoulin & Petrukhin), for Z = 1..92, as in
 * radiation_logarithm (pumas.c:13709-13738); 0 means unset. */
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

static double radiation_logarithm(double Z)
{
        const int i = (int)Z;
        if ((i >= 1) && (i <= 92)) {
                const double l = radiation_log_table[i - 1];
                if (l > 0) return l;
        }
        return 182.7;
}

/* dcs_bremsstrahlung_SSR (pumas.c:13915-14005), constants of
 * pumas.c:13827-13830. */
#define SSR_SQRTE 1.648721270700128
#define SSR_ME 0.5109989461
#define SSR_RE 2.8179403227E-13
#define SSR_MMU 105.6583745
static double dcs_bremsstrahlung_SSR(
    double Z, double A, double m, double K, double q)
{
        if ((Z <= 0) || (A <= 0) || (m <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        const double z13 = pow(Z, 1. / 3.);
        if (q >= K + m * (1. - 0.75 * SSR_SQRTE * z13)) return 0.;
        const double a[3] = { -0.00349, 148.84, -987.531 };
        const double b[4] = { 0.1642, 132.573, -585.361, 1407.77 };
        const double c[6] = { -2.8922, -19.0156, 57.698, -63.418, 14.1166,
                1.84206 };
        const double d[6] = { 2134.19, 581.823, -2708.85, 4767.05, 1.52918,
                0.361933 };
        const double energy = (K + m) * 1E+03;
        const double v = q * 1E+03 / energy;
        m *= 1E+03;
        const double Z13 = 1. / z13;
        const double rad_log = radiation_logarithm(Z);
        const double rad_log_inel = (Z == 1.) ? 446. : 1429.;
        const double Dn = 1.54 * pow(A, 0.27);
        const double mu_qc = m / (SSR_MMU * exp(1.) / Dn);
        const double rho = sqrt(1. + 4. * mu_qc * mu_qc);
        const double log_rho = log((rho + 1.) / (rho - 1.));
        const double delta1 = log(mu_qc) + 0.5 * rho * log_rho;
        const double delta2 = log(mu_qc) +
            0.25 * (3. * rho - rho * rho * rho) * log_rho +
            2. * mu_qc * mu_qc;
        const double delta = m * m * v / (2. * energy * (1. - v));
        double phi1 = log(rad_log * Z13 * (m / SSR_ME) /
            (1. + rad_log * Z13 * exp(0.5) * delta / SSR_ME));
        double phi2 = log(rad_log * Z13 * exp(-1. / 6.) * (m / SSR_ME) /
            (1. + rad_log * Z13 * exp(1. / 3.) * delta / SSR_ME));
        phi1 -= delta1 * (1. - 1. / Z);
        phi2 -= delta2 * (1. - 1. / Z);
        const double s_atomic_1 =
            log(m / delta / (m * delta / (SSR_ME * SSR_ME) + SSR_SQRTE));
        const double s_atomic_2 = log(1. + SSR_ME /
            (delta * rad_log_inel * Z13 * Z13 * SSR_SQRTE));
        const double s_atomic =
            (4. / 3. * (1. - v) + v * v) * (s_atomic_1 - s_atomic_2);
        double s_rad;
        if (v < .0 || v > 1.) {
                s_rad = 0.;
        } else if (v < 0.02) {
                s_rad = a[0] + a[1] * v + a[2] * v * v;
        } else if (v >= 0.02 && v < 0.1) {
                s_rad = b[0] + b[1] * v + b[2] * v * v + b[3] * v * v * v;
        } else if (v >= 0.01 && v < 0.9) {
                s_rad = c[0] + c[1] * v + c[2] * v * v;
                const double tmp = log(1. - v);
                s_rad += c[3] * v * log(v) + c[4] * tmp + c[5] * tmp * tmp;
        } else {
                s_rad = d[0] + d[1] * v + d[2] * v * v;
                const double tmp = log(1. - v);
                s_rad += d[3] * v * log(v) + d[4] * tmp + d[5] * tmp * tmp;
        }
        const double result =
            ((2. - 2. * v + v * v) * phi1 - 2. / 3. * (1. - v) * phi2) +
            1. / Z * s_atomic + 0.25 * ALPHA_EM * phi1 * s_rad;
        if (result <= 0.) return 0.;
        const double aux = 2 * (SSR_ME / m) * SSR_RE * Z;
        return aux * aux * (ALPHA_EM / q) * result * 1E-04;
}

/* dcs_pair_production_range (pumas.c:14230-14240). */
static void dcs_pair_production_range(
    double Z, double m, double K, double * qmin, double * qmax)
{
        if (qmax != NULL) {
                const double sqrte = 1.6487212707;
                const double Z13 = pow(Z, 1. / 3.);
                *qmax = K + m * (1. - 0.75 * sqrte * Z13);
        }
        if (qmin != NULL) *qmin = 4. * ELECTRON_MASS;
}

/* dcs_pair_production_d2_SSR (pumas.c:14394-14544). */
static double dcs_pair_production_d2_SSR(
    double Z, double A, double m, double K, double q, double rho)
{
        if ((Z <= 0) || (A <= 0) || (m <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        double qmin, qmax;
        dcs_pair_production_range(Z, m, K, &qmin, &qmax);
        if ((q < qmin) || (q > qmax)) return 0.;
        const double energy = (K + m) * 1E+03;
        const double v = q / (K + m);
        m *= 1E+03;
        const double rad_log = radiation_logarithm(Z);
        const double const_prefactor =
            4. / (3. * PI_) * Z * pow(ALPHA_EM * SSR_RE, 2.);
        const double Z13 = pow(Z, -1. / 3.);
        const double d_n = 1.54 * pow(A, 0.27);
        rho = 1 - rho;
        const double rho2 = rho * rho;
        double g1, g2;
        if (Z == 1.) {
                g1 = 4.4E-05;
                g2 = 4.8E-05;
        } else {
                g1 = 1.95E-05;
                g2 = 5.3E-05;
        }
        const double zeta1 = (0.073 * log(energy / m /
                                     (1. + g1 * pow(Z, 2. / 3.) * energy / m)) -
            0.26);
        const double zeta2 =
            (0.058 * log(energy / m / (1 + g2 / Z13 * energy / m)) - 0.14);
        double zeta;
        if ((zeta1 > 0.) && (zeta2 > 0.))
                zeta = zeta1 / zeta2;
        else
                zeta = 0.;
        const double beta = v * v / (2. * (1. - v));
        const double xi = pow(m * v / (2. * SSR_ME), 2.) * (1. - rho2) / (1. - v);

        const double Be = ((2. + rho2) * (1. + beta) + xi * (3. + rho2)) *
                log(1. + 1. / xi) +
            (1. - rho2 - beta) / (1. + xi) - (3. + rho2);
        const double Ce2 = ((1. - rho2) * (1. + beta) + xi * (3. - rho2)) *
                log(1. + 1. / xi) +
            2. * (1. - beta - rho2) / (1. + xi) - (3. - rho2);
        const double Ce1 = Be - Ce2;
        const double De = ((2. + rho2) * (1. + beta) + xi * (3. + rho2)) *
                math_dilog(1. / (1. + xi)) -
            (2. + rho2) * xi * log(1. + 1. / xi) -
            (xi + rho2 + beta) / (1. + xi);
        double Le1, Le2;
        if (De / Be > 0.) {
                const double tmp = De / Be;
                const double Xe = (tmp < 100) ? exp(-tmp) : 0.;
                Le1 = log(rad_log * Z13 * sqrt(1. + xi) /
                          (Xe + 2. * SSR_ME * exp(0.5) * rad_log * Z13 *
                                  (1. + xi) / (energy * v * (1. - rho2)))) -
                    tmp -
                    0.5 * log(Xe + pow(SSR_ME / m * d_n, 2.) * (1. + xi));
                Le2 = log(rad_log * Z13 * exp(-1. / 6.) * sqrt(1 + xi) /
                          (Xe + 2. * SSR_ME * exp(1. / 3.) * rad_log * Z13 *
                                  (1. + xi) / (energy * v * (1. - rho2)))) -
                    tmp -
                    0.5 * log(Xe + pow(SSR_ME / m * d_n, 2.) * exp(-1. / 3.) *
                                  (1. + xi));
        } else {
                const double tmp = De / Be;
                const double Xe_inv = (tmp > -100) ? exp(De / Be) : 0;
                Le1 = log(rad_log * Z13 * sqrt(1. + xi) /
                          (1. + Xe_inv * 2. * SSR_ME * exp(0.5) * rad_log *
                                    Z13 * (1. + xi) /
                                    (energy * v * (1. - rho2)))) -
                    0.5 * De / Be -
                    0.5 * log(1. + Xe_inv * pow(SSR_ME / m * d_n, 2.) *
                                       (1. + xi));
                Le2 = log(rad_log * Z13 * exp(-1. / 6.) * sqrt(1 + xi) /
                          (1. + Xe_inv * 2. * SSR_ME * exp(1. / 3.) * rad_log *
                                    Z13 * (1. + xi) /
                                    (energy * v * (1. - rho2)))) -
                    0.5 * De / Be -
                    0.5 * log(1. + Xe_inv * pow(SSR_ME / m * d_n, 2.) *
                                       exp(-1. / 3.) * (1. + xi));
        }
        double diagram_e = const_prefactor * (Z + zeta) * (1. - v) / v *
            (Ce1 * Le1 + Ce2 * Le2);
        if (diagram_e < 0.) diagram_e = 0.;

        const double Bm = ((1. + rho2) * (1. + (3. * beta) / 2) -
                              1. / xi * (1. + 2. * beta) * (1. - rho2)) *
                log(1. + xi) +
            xi * (1. - rho2 - beta) / (1. + xi) +
            (1. + 2. * beta) * (1. - rho2);
        const double Cm2 =
            ((1. - beta) * (1. - rho2) - xi * (1. + rho2)) * log(1. + xi) /
                xi -
            2. * (1. - beta - rho2) / (1. + xi) + 1. - beta -
            (1. + beta) * rho2;
        const double Cm1 = Bm - Cm2;
        const double Dm = ((1. + rho2) * (1. + (3. * beta) / 2.) -
                              1. / xi * (1. + 2. * beta) * (1. - rho2)) *
                math_dilog(xi / (1. + xi)) +
            (1. + (3. * beta) / 2.) * (1. - rho2) / xi * log(1. + xi) +
            (1. - rho2 - beta / 2. * (1. + rho2) +
                (1. - rho2) / (2. * xi) * beta) *
                xi / (1. + xi);
        double Lm1, Lm2;
        if (Dm / Bm > 0.) {
                const double tmp = Dm / Bm;
                const double Xm = (tmp < 100) ? exp(-tmp) : 0.;
                Lm1 = log(m / SSR_ME * rad_log * Z13 / d_n /
                          (Xm + 2. * SSR_ME * exp(0.5) * rad_log * Z13 *
                                  (1. + xi) / (energy * v * (1. - rho2)))) -
                    tmp;
                Lm2 = log(m / SSR_ME * rad_log * Z13 / d_n /
                          (Xm + 2. * SSR_ME * exp(1. / 3.) * rad_log * Z13 *
                                  (1. + xi) / (energy * v * (1. - rho2)))) -
                    tmp;
        } else {
                const double tmp = Dm / Bm;
                const double Xmv = (tmp > -100) ? exp(tmp) : 0.;
                Lm1 = log(m / SSR_ME * rad_log * Z13 / d_n /
                    (1. + 2. * SSR_ME * exp(0.5) * rad_log * Z13 * (1. + xi) /
                            (energy * v * (1. - rho2)) * Xmv));
                Lm2 = log(m / SSR_ME * rad_log * Z13 / d_n /
                    (1. + 2. * SSR_ME * exp(1. / 3.) * rad_log * Z13 *
                            (1. + xi) / (energy * v * (1. - rho2)) * Xmv));
        }
        double diagram_mu = const_prefactor * (Z + zeta) * (1. - v) / v *
            pow(SSR_ME / m, 2.) * (Cm1 * Lm1 + Cm2 * Lm2);
        if (diagram_mu < 0.) diagram_mu = 0.;
        return (diagram_e + diagram_mu) * 1E-01 / energy;
}

/* dcs_pair_production_SSR (pumas.c:14560-14604). */
static double dcs_pair_production_SSR(
    double Z, double A_, double mass, double K, double q)
{
        if ((Z <= 0) || (A_ <= 0) || (mass <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        if (q <= 4. * ELECTRON_MASS) return 0.;
        const double sqrte = 1.6487212707;
        const double Z13 = pow(Z, 1. / 3.);
        if (q >= K + mass * (1. - 0.75 * sqrte * Z13)) return 0.;
        const double gamma = 1. + K / mass;
        const double x0 = 1. - 4. * ELECTRON_MASS / q;
        const double x1 = 1. - 6. / (gamma * (gamma - q / mass));
        double rmax;
        if ((x0 > 0) && (x1 > 0))
                rmax = sqrt(x0) * x1;
        else
                return 0.;
        const double ri = 1. - rmax;
        if ((ri <= 0.) || (ri >= 1.)) return 0.;
        const double tmin = log(ri);
        double I = 0.;
        int i;
        for (i = 0; i < 12; i++) {
                const double rho = exp(gl12_x[i] * tmin);
                I -= dcs_pair_production_d2_SSR(Z, A_, mass, K, q, rho) * rho *
                    gl12_w[i] * tmin;
        }
        return (I < 0) ? 0. : I;
}


/* dcs_photonuclear_f2p_ALLM97 (pumas.c:14626-14673). */
static double dcs_photonuclear_f2p_ALLM97(double x, double Q2)
{
        const double m02 = 0.31985;
        const double mP2 = 49.457;
        const double mR2 = 0.15052;
        const double Q02 = 0.52544;
        const double Lambda2 = 0.06527;
        const double cP1 = 0.28067;
        const double cP2 = 0.22291;
        const double cP3 = 2.1979;
        const double aP1 = -0.0808;
        const double aP2 = -0.44812;
        const double aP3 = 1.1709;
        const double bP1 = 0.36292;
        const double bP2 = 1.8917;
        const double bP3 = 1.8439;
        const double cR1 = 0.80107;
        const double cR2 = 0.97307;
        const double cR3 = 3.4942;
        const double aR1 = 0.58400;
        const double aR2 = 0.37888;
        const double aR3 = 2.6063;
        const double bR1 = 0.01147;
        const double bR2 = 3.7582;
        const double bR3 = 0.49338;
        const double M = 0.5 * (PROTON_MASS + NEUTRON_MASS);
        const double M2 = M * M;
        const double W2 = M2 + Q2 * (1.0 / x - 1.0);
        const double t = log(log((Q2 + Q02) / Lambda2) / log(Q02 / Lambda2));
        const double xP = (Q2 + mP2) / (Q2 + mP2 + W2 - M2);
        const double xR = (Q2 + mR2) / (Q2 + mR2 + W2 - M2);
        const double cP =
            cP1 + (cP1 - cP2) * (1.0 / (1.0 + pow(t, cP3)) - 1.0);
        const double aP =
            aP1 + (aP1 - aP2) * (1.0 / (1.0 + pow(t, aP3)) - 1.0);
        const double bP = bP1 + bP2 * pow(t, bP3);
        const double cR = cR1 + cR2 * pow(t, cR3);
        const double aR = aR1 + aR2 * pow(t, aR3);
        const double bR = bR1 + bR2 * pow(t, bR3);
        const double F2P = cP * exp(aP * log(xP) + bP * log(1 - x));
        const double F2R = cR * exp(aR * log(xR) + bR * log(1 - x));
        return Q2 / (Q2 + m02) * (F2P + F2R);
}

/* dcs_photonuclear_shadowing_DRSS (pumas.c:14688-14699). */
static double dcs_photonuclear_shadowing_DRSS(double Z, double A, double x)
{
        if (Z == 1.) return 1.;
        if (x < 0.0014)
                return exp(-0.1 * log(A));
        else if (x < 0.04)
                return exp((0.069 * log10(x) + 0.097) * log(A));
        else
                return 1.;
}

/* dcs_photonuclear_f2a_DRSS (pumas.c:14716-14721). */
static double dcs_photonuclear_f2a_DRSS(
    double Z, double A, double F2p, double shadowing, double x)
{
        return F2p * shadowing *
            (Z + (A - Z) * (1.0 + x * (-1.85 + x * (2.45 + x * (-2.35 + x)))));
}

/* dcs_photonuclear_d2_DRSS (pumas.c:14923-14943). */
static double dcs_photonuclear_d2_DRSS(
    double Z, double A, double ml, double K, double q, double Q2)
{
        const double cf = 4 * PI_ * ALPHA_EM * ALPHA_EM * HBAR_C * HBAR_C;
        const double M = 0.5 * (PROTON_MASS + NEUTRON_MASS);
        const double E = K + ml;
        const double y = q / E;
        const double x = 0.5 * Q2 / (M * q);
        const double F2p = dcs_photonuclear_f2p_ALLM97(x, Q2);
        const double shadowing = dcs_photonuclear_shadowing_DRSS(Z, A, x);
        const double F2A = dcs_photonuclear_f2a_DRSS(Z, A, F2p, shadowing, x);
        const double R = 0.;
        const double dds = (1 - y +
                               0.5 * (1 - 2 * ml * ml / Q2) *
                                   (y * y + Q2 / (E * E)) / (1 + R)) /
                (Q2 * Q2) -
            0.25 / (E * E * Q2);
        return cf * F2A * dds / q;
}

typedef double photonuclear_ddcs_t(
    double Z, double A, double ml, double K, double q, double Q2);

/* The doubly differential cross section of the photonuclear polar angle
 * sampler: BM for the BM model, else DRSS (dcs_photonuclear_ddcs,
 * pumas.c:15159-15170). */
static photonuclear_ddcs_t * photonuclear_ddcs(void);

/* dcs_photonuclear_integrated for mode 0 (pumas.c:15002-15060), with the
 * logarithmic Gauss nodes of math_gauss_quad_initialise
 * (pumas.c:12575-12602). */
static double photonuclear_integrated(photonuclear_ddcs_t * ddcs,
    double Z, double A, double ml, double K, double q)
{
        if ((Z <= 0) || (A <= 0) || (ml <= 0) || (K <= 0)) return 0.;
        const double M = 0.5 * (NEUTRON_MASS + PROTON_MASS);
        const double mpi = PION_MASS;
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
                const double Q2 = exp(xmin + dx * gl9_x[i]);
                const double w = gl9_w[i] * (dx * Q2);
                double tmp = ddcs(Z, A, ml, K, q, Q2);
                if (tmp <= 0.) continue;
                ds += tmp * w;
        }
        return (ds < 0.) ? 0. : ds;
}

/* dcs_photonuclear_DRSS and dcs_photonuclear_BM (pumas.c:15078-15103). */
static double dcs_photonuclear_DRSS(
    double Z, double A, double ml, double K, double q)
{
        return photonuclear_integrated(
            &dcs_photonuclear_d2_DRSS, Z, A, ml, K, q);
}

static photonuclear_ddcs_t * photonuclear_ddcs(void)
{
        return (ph->model_photo == 2) ? &gpm_photonuclear_d2_BM :
                                        &dcs_photonuclear_d2_DRSS;
}


/* dcs_photonuclear_range (pumas.c:11058-11065). */
static void dcs_photonuclear_range(
    double m, double K, double * qmin, double * qmax)
{
        const double M = 0.5 * (NEUTRON_MASS + PROTON_MASS);
        const double mpi = PION_MASS;
        if (qmin != NULL) *qmin = mpi + 0.5 * mpi * mpi / M;
        if (qmax != NULL) *qmax = K + m - 0.5 * (M + m * m / M);
}

/* pumas_electronic_dcs (pumas.c:11082-11101). */
static double electronic_dcs(double Z, double I, double m, double K, double q)
{
        const double P2 = K * (K + 2. * m);
        const double E = K + m;
        const double Wmax = 2. * ELECTRON_MASS * P2 /
            (m * m + ELECTRON_MASS * (ELECTRON_MASS + 2. * E));
        if (q > Wmax) return 0.;
        const double Wmin = (13.6 / 19.2) * I;
        if (q <= Wmin) return 0.;
        const double E2 = E * E;
        const double beta2 = P2 / E2;
        const double a0 = 0.5 / E2;
        const double a1 = beta2 / Wmax;
        const double cs = 2 * PI_ * ELECTRON_MASS * ELECTRON_RADIUS *
            ELECTRON_RADIUS * Z * (a0 + 1. / q * (1 / q - a1)) / beta2;
        return cs;
}

/* Process wrappers dcs_bremsstrahlung, dcs_pair_production,
 * dcs_photonuclear and dcs_ionisation (pumas.c:11003-11122), in m^2/kg. */
static double dcs_process(int process, const struct port_element * e,
    double K, double q)
{
        switch (process) {
        case 0: {
                const double m = ph->mass;
                const double d = (ph->model_brems == 1) ?
                    gpm_bremsstrahlung_KKP(e->Z, e->A, m, K, q,
                        radiation_logarithm(e->Z)) :
                    (ph->model_brems == 2) ?
                    gpm_bremsstrahlung_ABB(e->Z, e->A, m, K, q) :
                    dcs_bremsstrahlung_SSR(e->Z, e->A, m, K, q);
                return d * 1E+03 * AVOGADRO_NUMBER * (m + K) / e->A;
        }
        case 1: {
                const double m = ph->mass;
                const double d = (ph->model_pair == 1) ?
                    gpm_pair_production_KKP(e->Z, e->A, m, K, q,
                        radiation_logarithm(e->Z), gl12_x, gl12_w) :
                    dcs_pair_production_SSR(e->Z, e->A, m, K, q);
                return d * 1E+03 * AVOGADRO_NUMBER * (m + K) / e->A;
        }
        case 2: {
                double qmin, qmax;
                dcs_photonuclear_range(ph->mass, K, &qmin, &qmax);
                if ((q < qmin) || (q > qmax)) return 0.;
                const double m = ph->mass;
                const double d = (ph->model_photo == 1) ?
                    gpm_photonuclear_BBKS(e->Z, e->A, m, K, q) :
                    (ph->model_photo == 2) ?
                    gpm_photonuclear_BM(e->Z, e->A, m, K, q, gl9_x, gl9_w) :
                    dcs_photonuclear_DRSS(e->Z, e->A, m, K, q);
                return d * 1E+03 * AVOGADRO_NUMBER * (m + K) / e->A;
        }
        default:
                return electronic_dcs(e->Z, e->I, ph->mass, K, q) *
                    (ph->mass + K) * AVOGADRO_NUMBER / (e->A * 1E-03);
        }
}

/* Float index bracketing, table_bracketf (pumas.c:4236-4244). */
static void table_bracketf(const float * table, float value, int * p1, int * p2)
{
        do {
                const int i3 = (*p1 + *p2) / 2;
                if (value >= table[i3])
                        *p1 = i3;
                else
                        *p2 = i3;
        } while (*p2 - *p1 >= 2);
}

/* dcs_evaluate (pumas.c:11243-11347): single precision interpolation of the
 * tabulated log DCS, or the exact model. */
static double dcs_evaluate(
    int process, const struct port_element * element, double K, double q)
{
        const double wj = K / (K + ph->mass);
        if (process == 3) return dcs_process(process, element, K, q) * wj;

        double qlow = 0;
        if (process == 2) {
                double qmin, qmax;
                dcs_photonuclear_range(ph->mass, K, &qmin, &qmax);
                if ((q < qmin) || (q > qmax))
                        return 0.;
                else
                        qlow = 2 * qmin;
        } else {
                double qmin, qmax;
                dcs_pair_production_range(element->Z, ph->mass, K, &qmin, &qmax);
                if (process == 1)
                        qlow = 4 * qmin;
                else
                        qmin = 0.;
                if ((q < qmin) || (q > qmax)) return 0.;
        }
        if (q < qlow) return dcs_process(process, element, K, q) * wj;

        const int nx = ph->n_table_dcs;
        const float xmin = ph->DCS_x[0];
        const float xmax = ph->DCS_x[nx - 1];
        const float x = logf((float)(q / K));
        if ((x < xmin) || (x >= xmax))
                return dcs_process(process, element, K, q) * wj;
        int ix = 0, tmpi = nx - 1;
        table_bracketf(ph->DCS_x, x, &ix, &tmpi);
        if ((ix < 0) || (ix >= nx - 1))
                return dcs_process(process, element, K, q) * wj;

        float p00, p01, m00, m01, p10, p11, m10, m11, h0, h1;
        const int imax = ph->n_energies - 1;
        const double Kmax = ph->K[imax];
        const long stride = (long)ph->n_table_dcs * 2;
        const float * base = ph->DCS +
            stride * ((long)(process * ph->n_elements + element->index) *
                         ph->n_energies);
        int i0;
        if ((K >= Kmax) || ((i0 = table_index(ph->K, K)) >= imax)) {
                const float * data = base + stride * imax;
                p00 = p10 = data[2 * ix];
                m00 = m10 = data[2 * ix + 1];
                p01 = p11 = data[2 * ix + 2];
                m01 = m11 = data[2 * ix + 3];
                h0 = 1.f;
                h1 = 0.f;
        } else {
                const float * data = base + stride * i0;
                p00 = data[2 * ix];
                m00 = data[2 * ix + 1];
                p01 = data[2 * ix + 2];
                m01 = data[2 * ix + 3];
                data += 2 * nx;
                p10 = data[2 * ix];
                m10 = data[2 * ix + 1];
                p11 = data[2 * ix + 2];
                m11 = data[2 * ix + 3];
                const float K0 = (float)(ph->K[i0]);
                const float K1 = (float)(ph->K[i0 + 1]);
                h1 = logf(((float)K) / K0) / logf(K1 / K0);
                h0 = 1.f - h1;
        }
        if (((p00 == 0.f) && (m00 == 0.f)) || ((p01 == 0.f) && (m01 == 0.f)) ||
            ((p10 == 0.f) && (m10 == 0.f)) || ((p11 == 0.f) && (m11 == 0.f)))
                return dcs_process(process, element, K, q) * wj;

        const float x0 = ph->DCS_x[ix];
        const float x1 = ph->DCS_x[ix + 1];
        const float dx = x1 - x0;
        m00 *= dx;
        m01 *= dx;
        const float t = (x - x0) / dx;
        const float c02 = -3 * (p00 - p01) - 2 * m00 - m01;
        const float c03 = 2 * (p00 - p01) + m00 + m01;
        float r = expf(p00 + t * (m00 + t * (c02 + t * c03))) * h0;
        if (h1 > 0.f) {
                m10 *= dx;
                m11 *= dx;
                const float c12 = -3 * (p10 - p11) - 2 * m10 - m11;
                const float c13 = 2 * (p10 - p11) + m10 + m11;
                r += expf(p10 + t * (m10 + t * (c12 + t * c13))) * h1;
        }
        return r * wj;
}

/* ------------------------------------------------------------------------ */
/* Polar angle samplers (pumas.c:11736-11976).                              */
/* ------------------------------------------------------------------------ */

/* polar_bremsstrahlung (pumas.c:11759-11830); also used for pairs. */
static double polar_bremsstrahlung(struct port_ctx * c,
    const struct port_element * element, double ki, double kf)
{
        const double m = ph->mass;
        const double E = ki + m;
        const double nu = ki - kf;
        const double y = nu / E;
        const double tmp = 0.5 * m * nu / (E * (E - nu));
        const double mu0 = tmp * tmp;
        const double c1 = (2 * (1. - y) + y * y) * mu0;
        const double c2 = 4 * (1. - y) * mu0 * mu0;
        const double RN = data_nuclear_radius(element->Z, element->A);
        const double tmp2 = m * RN / HBAR_C;
        const double muni = tmp2 * tmp2 / 6.;
        const double muc = sqrt(mu0) - mu0;
        if (muc < 0) return 0;
        double x0;
        {
                const double q = muni;
                const double r = mu0;
                const double qr = q * r;
                x0 = (1. + 2 * qr) * log((1. + qr) / (r + qr)) -
                    (1. - r) * (1 + 2 * q) / (1 + q);
        }
        int i;
        for (i = 0; i < 100; i++) {
                const double r0 = rnd(c);
                const double r1 = rnd(c);
                const double mu = r0 * mu0 / (mu0 + 1. - r0);
                const double mus = mu0 + mu;
                const double mu2 = mus * mus;
                const double d1 = 1 / mu2;
                const double d2 = d1 * d1;
                const double score = r1 * c1 * d1;
                double pdf = c1 * d1 - mu * c2 * d2;
                if (score > pdf) continue;
                const double l2 = mu2 / (mu0 * mu0);
                const double q = muni * l2;
                const double r = mu0 * l2;
                const double qr = q * r;
                if (qr > 1E+05) continue;
                const double x = (1. + 2 * qr) * log((1. + qr) / (r + qr)) -
                    (1. - r) * (1 + 2 * q) / (1 + q);
                pdf *= x / x0;
                if (score <= pdf) return mu;
        }
        return 0.;
}

/* Objective of the photonuclear polar sampling (pumas.c:11855-11862). */
struct polar_args {
        double Z, A, K, q;
};

static double polar_objective(double lnQ2, const struct polar_args * p)
{
        const double Q2 = exp(lnQ2);
        return -photonuclear_ddcs()(p->Z, p->A, ph->mass, p->K, p->q, Q2) *
            Q2;
}

/* math_find_minimum_brent (pumas.c:12233-12325). The upper bracket of the
 * search is the initial minimiser xb, as in the reference. */
static int find_minimum_brent(double xa, double xb, double xc,
    const double * fb_p, double tol, int max_iter,
    const struct polar_args * params, double * xopt, double * fopt)
{
#define EPS 1E-15
#define GOLD 0.3819660
#define SIGN(a, b) ((b) >= 0.0 ? fabs(a) : -fabs(a))
        double fb = *fb_p;
        tol *= fabs(xc - xa);
        double x = xb, w = xb, v = xb;
        double fw = fb, fv = fb, fx = fb;
        double d = 0., e = 0.;
        int i;
        for (i = 0; i < max_iter; i++) {
                const double xm = 0.5 * (xa + xb);
                const double tol1 = tol * fabs(x) + EPS;
                const double tol2 = 2 * tol1;
                if (fabs(x - xm) <= (tol2 - 0.5 * (xb - xa))) break;
                if (fabs(e) > tol1) {
                        const double r = (x - w) * (fx - fv);
                        double q = (x - v) * (fx - fw);
                        double p = (x - v) * q - (x - w) * r;
                        q = 2. * (q - r);
                        if (q > 0.) p = -p;
                        q = fabs(q);
                        const double etemp = e;
                        e = d;
                        if (fabs(p) >= fabs(0.5 * q * etemp) ||
                            (p <= q * (xa - x)) || (p >= q * (xb - x))) {
                                e = (x >= xm) ? xa - x : xb - x;
                                d = GOLD * e;
                        } else {
                                d = p / q;
                                const double u = x + d;
                                if ((u - xa < tol2) || (xb - u < tol2))
                                        d = SIGN(tol1, xm - x);
                        }
                } else {
                        e = (x >= xm) ? xa - x : xb - x;
                        d = GOLD * e;
                }
                const double u =
                    (fabs(d) >= tol1) ? x + d : x + SIGN(tol1, d);
                const double fu = polar_objective(u, params);
                if (fu <= fx) {
                        if (u >= x)
                                xa = x;
                        else
                                xb = x;
                        v = w, w = x, x = u;
                        fv = fw, fw = fx, fx = fu;
                } else {
                        if (u < x)
                                xa = u;
                        else
                                xb = u;
                        if ((fu <= fw) || (w == x)) {
                                v = w;
                                w = u;
                                fv = fw;
                                fw = fu;
                        } else if ((fu <= fv) || (v == x) || (v == w)) {
                                v = u;
                                fv = fu;
                        }
                }
        }
        *xopt = x;
        *fopt = fx;
        return (i < max_iter) ? i : -1;
#undef EPS
#undef GOLD
#undef SIGN
}

/* math_find_minimum with Brent refinement (pumas.c:12105-12206). */
static int find_minimum(double xa, double xc, double tol, int max_iter,
    const struct polar_args * params, double * xopt, double * fopt)
{
        double fa = polar_objective(xa, params);
        double fc = polar_objective(xc, params);
        const double atol = tol * fabs(xc - xa);
        double xb = 0, fb = 0;
        int i;
        for (i = 0; i < max_iter; i++) {
                xb = 0.5 * (xa + xc);
                fb = polar_objective(xb, params);
                if ((fb < fa) && (fb < fc)) break;
                if (fabs(xc - xa) <= atol) {
                        *xopt = xb;
                        *fopt = fb;
                        return i;
                }
                if (fb < fc) {
                        xc = xb;
                        fc = fb;
                } else {
                        xa = xb;
                        fa = fb;
                }
        }
        if (i == max_iter) {
                if (fa < fb) {
                        fb = fa;
                        xb = xa;
                } else if (fc < fb) {
                        fb = fc;
                        xb = xc;
                }
                *xopt = xb;
                *fopt = fb;
                return -1;
        }
        const int status = find_minimum_brent(
            xa, xb, xc, &fb, tol, max_iter - i, params, xopt, fopt);
        if (status < 0)
                return -2;
        else
                return status + i;
}

/* polar_photonuclear (pumas.c:11874-11950). */
static double polar_photonuclear(struct port_ctx * c,
    const struct port_element * element, double ki, double kf)
{
        const double M = 0.5 * (PROTON_MASS + NEUTRON_MASS);
        const double q = ki - kf;
        const double ml = ph->mass;
        const double E = ki + ml;
        const double ml2 = ml * ml;
        const double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
        const double Q2max = 2.0 * M * (q - PION_MASS) - PION_MASS * PION_MASS;
        if ((Q2max < Q2min) | (Q2min < 0)) return 0.;
        const struct polar_args args = { element->Z, element->A, ki, q };
        double fopt = 0., xopt = 0.;
        const double lnQ2min = log(Q2min);
        const double lnQ2max = log(Q2max);
        const int status =
            find_minimum(lnQ2min, lnQ2max, 1E-06, 100, &args, &xopt, &fopt);
        fopt = -fopt;
        if (status == -2) return 0.;
        const double x = exp(xopt) / (2 * q * M);
        const double lne = 0.1;
        if ((x <= 0.04) && (xopt + lne < lnQ2max)) {
                double f2, x2;
                const int status2 = find_minimum(
                    xopt + lne, lnQ2max, 1E-06, 100, &args, &x2, &f2);
                if (status2 >= 0) {
                        f2 = -f2;
                        if (f2 > fopt) {
                                xopt = x2;
                                fopt = f2;
                        }
                }
        }
        const double rQ2 = lnQ2max - lnQ2min;
        double Q2 = 0.;
        int i;
        for (i = 0; i < 100; i++) {
                const double u = rnd(c);
                Q2 = Q2min * exp(rQ2 * u);
                const double r = photonuclear_ddcs()(
                                     element->Z, element->A, ml, ki, q, Q2) *
                    Q2;
                if (rnd(c) * fopt <= r) break;
        }
        if (i == 100) return 0.;
        const double p = sqrt(ki * (ki + 2 * ml));
        const double E1 = E - q;
        const double eps = ml / E1;
        const double p1 = E1 * sqrt((1. + eps) * (1. - eps));
        const double p2 = p * p1;
        double tmp = p2 + ml * ml - E * E1;
        if (fabs(tmp) <= 3 * DBL_EPSILON * p2) tmp = 0.;
        const double a_mu = 0.5 * tmp / p2;
        const double b_mu = 0.25 / p2;
        double mu = a_mu + b_mu * Q2;
        if (mu < 0)
                mu = 0.;
        else if (mu > 1.)
                mu = 1.;
        return mu;
}

/* polar_ionisation (pumas.c:11965-11976). */
static double polar_ionisation(double ki, double kf)
{
        const double nu = ki - kf;
        const double p2 = ki * (ki + 2 * ph->mass);
        const double E = ki + ph->mass;
        const double co = (p2 - nu * (E + ELECTRON_MASS)) /
            sqrt(p2 * (p2 + nu * nu - 2 * nu * E));
        return 0.5 * (1. - co);
}

static double polar_sample(struct port_ctx * c, int process,
    const struct port_element * element, double ki, double kf)
{
        if (process <= 1)
                return polar_bremsstrahlung(c, element, ki, kf);
        else if (process == 2)
                return polar_photonuclear(c, element, ki, kf);
        else
                return polar_ionisation(ki, kf);
}

/* ------------------------------------------------------------------------ */
/* DEL sampling (pumas.c:5887-6270, 11185-11226).                           */
/* ------------------------------------------------------------------------ */

/* dcs_ionisation_randomise (pumas.c:11185-11226). */
static double dcs_ionisation_randomise(struct port_ctx * c,
    const struct port_element * element, double K, double xlow)
{
        const double P2 = K * (K + 2. * ph->mass);
        const double E = K + ph->mass;
        const double Wmax = 2. * ELECTRON_MASS * P2 /
            (ph->mass * ph->mass +
                ELECTRON_MASS * (ELECTRON_MASS + 2. * E));
        if (Wmax < ph->cutoff * K) return K;
        double Wmin = (13.6 / 19.2) * element->I;
        const double qlow = K * xlow;
        if (qlow >= Wmin) Wmin = qlow;
        const double E2 = E * E;
        const double beta2 = P2 / E2;
        const double a0 = 0.5 / E2;
        const double a1 = beta2 / Wmax;
        const double p0 = a0 * (Wmax - Wmin);
        const double p2 = 1. / Wmin - 1. / Wmax;
        double q;
        for (;;) {
                double z = rnd(c) * (p0 + p2);
                if (z <= p0) {
                        z /= p0;
                        q = (Wmax - Wmin) * z;
                } else {
                        z = (z - p0) / p2;
                        q = Wmin * Wmax / (Wmax - z * (Wmax - Wmin));
                }
                const double r0 = a0 + 1 / (q * q);
                const double r1 = r0 - a1 / q;
                if (rnd(c) * r0 <= r1) break;
        }
        return K - q;
}

static inline double envelope_norm(double a, double xmin, double xmax)
{
        if (a == 1)
                return log(xmax / xmin);
        else
                return (pow(xmin, 1. - a) - pow(xmax, 1. - a)) / (a - 1.);
}

/* del_randomise_target (pumas.c:6154-6270). Sets *process, *element and,
 * in backward mode, *weight. */
static void del_randomise_target(struct port_ctx * c,
    const struct oracle_state * state, int material, double Q, int * process,
    int * element, double * weight)
{
        int i1, i2;
        double h, dk;
        i1 = table_index(ph->K, state->energy);
        if (i1 < 0) {
                i1 = i2 = 0;
                h = dk = 0.;
        } else if (i1 >= ph->n_energies - 1) {
                i1 = i2 = ph->n_energies - 1;
                h = dk = 0.;
        } else {
                i2 = i1 + 1;
                const double K1 = ph->K[i1];
                dk = ph->K[i2] - K1;
                h = (state->energy - K1) / dk;
        }
        (void)i2;
        const int ic0 = ph->comp_start[material];
        const int nc = ph->elements_in[material];
        int ic, ip;
        if (c->cfg->direction == MODE_FORWARD) {
                const double zeta = rnd(c);
                for (ic = ic0; ic < ic0 + nc; ic++) {
                        for (ip = 0; ip < N_DEL; ip++) {
                                const double * f = ph->CSf +
                                    (long)(ip * ph->n_components + ic) *
                                        ph->n_energies + i1;
                                const double * df = ph->CSf_dK +
                                    (long)(ip * ph->n_components + ic) *
                                        ph->n_energies + i1;
                                const double csf = pchip(
                                    h, f[0], f[1], df[0] * dk, df[1] * dk);
                                if (!(zeta > csf)) {
                                        *element = ph->comp_element[ic];
                                        *process = ip;
                                        return;
                                }
                        }
                }
                /* Not reached for consistent tables (pumas.c:6209). */
                *element = ph->comp_element[ic0 + nc - 1];
                *process = N_DEL - 1;
                c->step_event = -1;
                return;
        } else {
                double stot = 0.;
                for (ip = 0; ip < N_DEL; ip++) {
                        for (ic = ic0; ic < ic0 + nc; ic++) {
                                const struct port_element * e =
                                    ph->element + ph->comp_element[ic];
                                const double d =
                                    dcs_evaluate(ip, e, state->energy, Q);
                                stot += d * ph->comp_fraction[ic];
                        }
                }
                if (stot == 0.) {
                        *weight = 0.;
                        return;
                } else {
                        *weight = stot;
                }
                if (c->cfg->scattering == MODE_DISABLED) {
                        *element = ph->n_elements;
                        *process = N_DEL;
                        return;
                }
                double zeta;
                for (;;) {
                        zeta = rnd(c) * stot;
                        if ((zeta > 0.) && (zeta < stot)) break;
                }
                /* In the reference the energy transfer and the weight share
                 * a union (struct del_info, pumas.c:643-655). The weight was
                 * just written, hence the DCS below is evaluated at an
                 * energy transfer equal to stot (pumas.c:6228, 6250). */
                const double Q_union = stot;
                double s = 0.;
                for (ic = ic0; ic < ic0 + nc; ic++) {
                        for (ip = 0; ip < N_DEL; ip++) {
                                const int iel = ph->comp_element[ic];
                                const double si = dcs_evaluate(ip,
                                    ph->element + iel, state->energy,
                                    Q_union) * ph->comp_fraction[ic];
                                s += si;
                                if (!(zeta > s)) {
                                        *element = iel;
                                        *process = ip;
                                        return;
                                }
                        }
                }
                *element = ph->comp_element[ic0 + nc - 1];
                *process = N_DEL - 1;
                c->step_event = -1;
        }
}

/* del_randomise_forward (pumas.c:5912-6017). Returns the process index with
 * a polar angle to sample, or -1 for none; *target is the element. */
static int del_randomise_forward(struct port_ctx * c,
    struct oracle_state * state, int material, int * process, int * target)
{
        if (state->energy <= ph->Kt[material]) return -1;
        int ip = 0, iel = 0;
        double w = 0.;
        del_randomise_target(c, state, material, 0., &ip, &iel, &w);
        const struct port_element * element = ph->element + iel;
        *target = iel;
        *process = ip;
        if (ip == 3) {
                state->energy = dcs_ionisation_randomise(
                    c, element, state->energy, ph->cutoff);
                return ip;
        }
        double qmin, qmax;
        if (ip == 2) {
                dcs_photonuclear_range(ph->mass, state->energy, &qmin, &qmax);
        } else {
                dcs_pair_production_range(
                    element->Z, ph->mass, state->energy, &qmin, &qmax);
                if (ip == 0) qmin = 0.;
        }
        double xmin = qmin / state->energy;
        if (xmin < ph->cutoff) xmin = ph->cutoff;
        const double xmax = qmax / state->energy;
        if (xmin >= xmax) return -1;

        double a0, a1, b0, b1, p0;
        const int imax = ph->n_energies - 1;
        const float * env = ph->DCS_env +
            2 * ((long)(ip * ph->n_elements + element->index) * ph->n_energies);
        if (state->energy >= ph->K[imax]) {
                const float * envelope = env + 2 * imax;
                a0 = (double)envelope[0];
                b0 = (double)envelope[1];
                p0 = 1.;
                a1 = b1 = 0.;
        } else {
                const int row = table_index(ph->K, state->energy);
                const float * envelope0 = env + 2 * row;
                const float * envelope1 = env + 2 * (row + 1);
                a0 = (double)envelope0[0];
                b0 = (double)envelope0[1];
                a1 = (double)envelope1[0];
                b1 = (double)envelope1[1];
                const double k0 = ph->K[row];
                const double k1 = ph->K[row + 1];
                const double h1 = (state->energy - k0) / (k1 - k0);
                const double h0 = 1. - h1;
                b0 *= h0;
                b1 *= h1;
                p0 = envelope_norm(a0, xmin, xmax) * b0;
                const double p1 = envelope_norm(a1, xmin, xmax) * b1;
                p0 /= p0 + p1;
        }
        double x = 0.;
        int i;
        for (i = 0; i < 100; i++) {
                double u = rnd(c);
                double a;
                if (u < p0) {
                        a = a0;
                        u = u / p0;
                } else {
                        a = a1;
                        u = (u - p0) / (1. - p0);
                }
                if (a == 1) {
                        x = xmin * exp(u * log(xmax / xmin));
                } else {
                        const double am = a - 1.;
                        const double pmin = pow(xmin, -am);
                        const double pmax = pow(xmax, -am);
                        x = pow(pmin - u * (pmin - pmax), -1. / am);
                }
                const double penv = b0 * pow(x, -a0) + b1 * pow(x, -a1);
                const double d = dcs_evaluate(
                    ip, element, state->energy, state->energy * x);
                if (rnd(c) * penv <= d) break;
        }
        if (i == 100) return -1;
        state->energy *= (1. - x);
        return ip;
}

/* del_randomise_power_law (pumas.c:6109-6138) for alpha != 1. */
static void del_randomise_power_law(struct port_ctx * c, double alpha,
    double xmin, double xmax, double * p_r, double * p_w)
{
        double r = 0., w_bias;
        const double a1 = 1. - alpha;
        const double x0 = pow(xmin, a1);
        const double x1 = pow(xmax, a1);
        for (;;) {
                const double z = rnd(c);
                const double tmp = x0 + z * (x1 - x0);
                r = pow(tmp, 1. / a1);
                if ((r < xmin) || (r >= xmax)) continue;
                w_bias = (x1 - x0) * r / (a1 * tmp);
                break;
        }
        *p_r = 1. - r;
        *p_w = w_bias;
}

/* del_randomise_reverse (pumas.c:6036-6093). */
static int del_randomise_reverse(struct port_ctx * c,
    struct oracle_state * state, int material, int * process, int * target)
{
        const double lnq0 = -log(ph->cutoff);
        const double kt = ph->Kt[material];
        const double kf = state->energy;
        const double pCEL =
            (kf >= kt) ? 0. : lnq0 / (lnq0 + log(kt / (kt - kf)));
        if (pCEL && (rnd(c) < pCEL)) {
                state->weight /= pCEL;
                return -1;
        }
        const double xf =
            (kf >= kt * (1. - ph->cutoff)) ? ph->cutoff : 1. - kf / kt;
        double xmax;
        const double m1 = ph->mass - ELECTRON_MASS;
        if (state->energy < 0.5 * m1 * m1 / ELECTRON_MASS) {
                const double m2 = ph->mass + ELECTRON_MASS;
                xmax = 2. * ELECTRON_MASS * (state->energy + 2. * ph->mass) /
                    (m2 * m2);
                if (xmax < xf)
                        return -1;
                else if (xmax > 1.)
                        xmax = 1.;
        } else {
                xmax = 1.;
        }
        double r, w_bias;
        del_randomise_power_law(c, BMC_ALPHA, xf, xmax, &r, &w_bias);
        w_bias /= r;
        state->energy /= r;

        int ip = 0, iel = 0;
        double weight = 0.;
        del_randomise_target(
            c, state, material, state->energy - kf, &ip, &iel, &weight);
        if (weight <= 0) {
                state->weight = 0.;
                return -1;
        }
        state->weight *= w_bias * weight /
            (del_cross_section(material, kf) * (1. - pCEL));
        *process = ip;
        if (c->cfg->scattering == MODE_DISABLED) {
                *target = -1;
                return -2;
        } else {
                *target = iel;
                return ip;
        }
}

/* transport_do_del (pumas.c:5706-5757). */
static void transport_do_del(
    struct port_ctx * c, struct oracle_state * state, int material)
{
        double ki, kf;
        int process = -1, target = -1, polar;
        if (c->cfg->direction == MODE_FORWARD) {
                ki = state->energy;
                polar = del_randomise_forward(
                    c, state, material, &process, &target);
                kf = state->energy;
        } else {
                kf = state->energy;
                polar = del_randomise_reverse(
                    c, state, material, &process, &target);
                ki = state->energy;
        }
        if (c->step_event < 0) return;
        if (process < 0) {
                if (state->weight > 0)
                        c->step_event = EV_NONE;
                else
                        c->step_event = EV_WEIGHT;
        } else {
                static const int event_for[N_DEL + 1] = { EV_BREMSSTRAHLUNG,
                        EV_PAIR_CREATION, EV_PHOTONUCLEAR, EV_DELTA_RAY,
                        EV_VERTEX };
                c->step_event = event_for[process];
        }
        if ((c->cfg->scattering == MODE_MIXED) && (polar >= 0)) {
                if (kf > ki) {
                        const double tmp = kf;
                        kf = ki;
                        ki = tmp;
                }
                const double mu =
                    polar_sample(c, polar, ph->element + target, ki, kf);
                step_rotate_direction(c, state, mu);
        }
}

/* ------------------------------------------------------------------------ */
/* Elastic hard scattering (transport_do_ehs, pumas.c:5768-5885).           */
/* ------------------------------------------------------------------------ */
struct coulomb_data {
        double cs_hard;
        double normalisation;
        int n_parameters;
        double amplitude[3];
        double screening[4];
        coulomb_real a[3], b[3], c[4];
        double fspin;
        double fCM[2];
};

static void transport_do_ehs(
    struct port_ctx * c, struct oracle_state * state, int material)
{
        struct coulomb_data data_[16];
        const double kinetic = state->energy;
        double mu0 = 0., invlb1 = 0.;
        table_get_msc(c->cfg->energy_loss, material, kinetic, &mu0, &invlb1);
        const int n_el = ph->elements_in[material];
        const int ic0 = ph->comp_start[material];
        int i;
        struct coulomb_data * data;
        double cs_tot = 0.;
        for (i = 0, data = data_; i < n_el; i++, data++) {
                const struct port_element * element =
                    ph->element + ph->comp_element[ic0 + i];
                double kinetic0;
                coulomb_frame_parameters(element->Z, element->A, ph->mass,
                    kinetic, &kinetic0, data->fCM);
                data->fspin = coulomb_spin_factor(ph->mass, kinetic);
                coulomb_screening_parameters(element->Z, element->A, ph->mass,
                    kinetic, kinetic0, &data->n_parameters, data->amplitude,
                    data->screening);
                coulomb_pole_reduction(data->n_parameters, data->amplitude,
                    data->screening, data->a, data->b, data->c);
                data->normalisation = ph->comp_fraction[ic0 + i] /
                    coulomb_normalisation(
                        element->Z, element->A, ph->mass, kinetic, kinetic0);
                data->cs_hard = data->normalisation *
                    coulomb_restricted_cs(mu0, data->fspin,
                        data->n_parameters, data->screening, data->a,
                        data->b, data->c);
                cs_tot += data->cs_hard;
        }
        const double cc0 = rnd(c) * cs_tot;
        int ihard = n_el - 1;
        double cs = 0.;
        for (i = 0, data = data_; i < n_el; i++, data++) {
                cs += data->cs_hard;
                if (cs >= cc0) {
                        ihard = i;
                        break;
                }
        }
        data = data_ + ihard;
        const int n = data->n_parameters - 1;
        double A = data->screening[0];
        for (i = 1; i < n; i++) {
                const double Ai = data->screening[i];
                if (Ai < A) A = Ai;
        }
        double mu1;
        for (;;) {
                const double zeta = rnd(c);
                const double tmp = 1. + A - zeta * (1 - mu0);
                if (tmp <= 0.) continue;
                mu1 = (A + mu0) * (A + 1.) / tmp - A;
                if (mu1 < mu0)
                        mu1 = mu0;
                else if (mu1 > 1.)
                        mu1 = 1;
                int k;
                double ratio = 0.;
                for (k = 0; k < n; k++) {
                        ratio += data->amplitude[k] * (A + mu1) /
                            (data->screening[k] + mu1);
                }
                ratio *= coulomb_nuclear_form_factor(mu1, data->screening[n]);
                ratio *= ratio * (1. - data->fspin * mu1);
                if (rnd(c) <= ratio) break;
        }
        const double gamma = data->fCM[0];
        const double tau = data->fCM[1];
        double mu;
        if (mu1 > 1E-06) {
                const double a = gamma * (tau + 1. - 2. * mu1);
                const double ct_h = a / sqrt(4. * mu1 * (1. - mu1) + a * a);
                mu = 0.5 * (1. - ct_h);
        } else {
                const double d = gamma * (1. + tau);
                mu = mu1 / (d * d);
        }
        step_rotate_direction(c, state, mu);
}

/* ------------------------------------------------------------------------ */
/* Stepping (pumas.c:5194-5696, 6296-7005).                                 */
/* ------------------------------------------------------------------------ */

/* step_fluctuate (pumas.c:6943-7005). */
static void step_fluctuate(struct port_ctx * c,
    const struct oracle_state * state, int material, double Xtot, double dX,
    double * kf, double * ratio)
{
        const int scheme = c->cfg->energy_loss;
        const double sgn = (c->cfg->direction == MODE_FORWARD) ? 1. : -1.;
        double k1, r = 0.;
        k1 = cel_kinetic_energy(scheme, material, Xtot - sgn * dX);
        const double dk0 = fabs(state->energy - k1);
        if ((k1 > 0.) && (dk0 > 0.)) {
                const double Omega0 = cel_straggling(material, state->energy);
                const double Omega1 = cel_straggling(material, k1);
                double dk12 = 0.5 * dX * (Omega0 + Omega1);
                const double tmp = dX / Xtot;
                if (tmp > 5E-02) {
                        const double de1 = cel_energy_loss(scheme, material, k1);
                        const double de0 =
                            cel_energy_loss(scheme, material, state->energy);
                        dk12 *= 1. + sgn * dX / dk0 * (de1 - de0);
                }
                const double dk1 = sqrt(dk12);
                if (dk0 >= 3. * dk1) {
                        double u;
                        do
                                u = step_randn(c);
                        while (fabs(u) > 3.);
                        u /= 1.015387;
                        k1 += u * dk1;
                } else if (dk0 >= 1.7320508 * dk1) {
                        const double u = 1.7320508 * (1. - 2. * rnd(c));
                        k1 += u * dk1;
                } else {
                        const double dk32 = 3. * dk12;
                        const double dk02 = dk0 * dk0;
                        const double a =
                            1. - (dk32 - dk02) / (dk32 + 3. * dk02);
                        if (rnd(c) <= a) {
                                const double b =
                                    0.5 * (dk32 + 3. * dk02) / dk0;
                                const double u = rnd(c);
                                k1 = state->energy - sgn * b * u;
                                if (k1 < 0.) k1 = 0.;
                        } else {
                                k1 = state->energy;
                        }
                }
                r = fabs(state->energy - k1) / dk0;
        }
        if (r == 0.) r = 1.;
        *kf = k1;
        *ratio = r;
}

/* transport_limit (pumas.c:5569-5696). */
static void transport_limit(struct port_ctx * c,
    const struct oracle_state * state, int material, double Xi, double Xf,
    double * grammage_max)
{
        const struct oracle_config * cfg = c->cfg;
        c->step_event = c->step_foreseen = EV_NONE;
        if (state->weight <= 0.) {
                c->step_event = EV_WEIGHT;
                return;
        }
        if (cfg->direction == MODE_FORWARD) {
                const double kinetic_min =
                    (cfg->event & EV_LIMIT_ENERGY) ? cfg->limit_energy : 0.;
                if (state->energy <= kinetic_min) {
                        c->step_event = EV_LIMIT_ENERGY;
                        return;
                }
        } else if ((cfg->event & EV_LIMIT_ENERGY) &&
            (state->energy >= cfg->limit_energy)) {
                c->step_event = EV_LIMIT_ENERGY;
                return;
        }
        if (cfg->event & EV_LIMIT_GRAMMAGE) {
                *grammage_max = cfg->limit_grammage;
                c->step_foreseen = EV_LIMIT_GRAMMAGE;
        } else {
                *grammage_max = 0.;
        }
        const int scheme = cfg->energy_loss;
        if (scheme == MODE_DISABLED) {
                if (cfg->scattering == MODE_MIXED) {
                        const double X = Xi -
                            coulomb_ehs_length(material, state->energy) *
                                log(rnd(c));
                        if ((*grammage_max == 0.) || (X < *grammage_max)) {
                                *grammage_max = X;
                                c->step_foreseen = EV_COULOMB;
                                return;
                        }
                }
                return;
        }
        const double sgn = (cfg->direction == MODE_FORWARD) ? 1. : -1.;
        int foreseen = EV_NONE;
        double kinetic_limit = 0.;
        if (scheme == MODE_MIXED) {
                int i;
                for (i = 0; i < 1000; i++) {
                        const double zeta = rnd(c);
                        if ((zeta <= 0.) || (zeta >= 1.)) continue;
                        const double nI =
                            del_interaction_length(material, state->energy) +
                            sgn * log(zeta);
                        if (nI <= 0.) break;
                        const double k =
                            del_kinetic_from_interaction_length(material, nI);
                        if (cfg->direction == MODE_FORWARD) {
                                if (k >= state->energy) continue;
                        } else {
                                if (k <= state->energy) continue;
                        }
                        if ((cfg->direction == MODE_BACKWARD) ||
                            (k > ph->Kt[material])) {
                                kinetic_limit = k;
                                foreseen = EV_DEL;
                        }
                        break;
                }
        }
        if ((scheme < MODE_STRAGGLED) && (cfg->scattering == MODE_MIXED)) {
                const double nI =
                    ehs_interaction_length(scheme, material, state->energy) +
                    sgn * log(rnd(c));
                if (nI > 0.) {
                        const double k = ehs_kinetic_from_interaction_length(
                            scheme, material, nI);
                        if ((kinetic_limit <= 0.) ||
                            ((cfg->direction == MODE_FORWARD) &&
                                (k > kinetic_limit)) ||
                            ((cfg->direction == MODE_BACKWARD) &&
                                (k < kinetic_limit))) {
                                kinetic_limit = k;
                                foreseen = EV_COULOMB;
                        }
                }
        }
        if (foreseen == EV_NONE) return;
        const double X = Xi +
            sgn * (Xf - cel_grammage(scheme, material, kinetic_limit));
        if ((*grammage_max <= 0) || (X < *grammage_max)) {
                *grammage_max = X;
                c->step_foreseen = foreseen;
        }
}

/* step_transport (pumas.c:6296-6925), without magnetic field and with
 * uniform locals. Returns the end step medium index in *out_medium. */
static int step_transport(struct port_ctx * c, struct oracle_state * state,
    int straight, int medium, double density, double grammage_max,
    double step_max_medium, double * step_max_locals, double * density_end,
    int * out_medium)
{
        const struct oracle_config * cfg = c->cfg;
        const int scheme = cfg->energy_loss;
        double * const direction = state->direction;
        double * const position = state->position;
        const int material = medium_material(c, medium);
        const double density_i = 1. / density;
        const double momentum =
            sqrt(state->energy * (state->energy + 2. * ph->mass));
        const int tmp_scheme = (scheme == MODE_DISABLED) ? MODE_CSDA : scheme;
        const double Xtot = cel_grammage(tmp_scheme, material, state->energy);

        double step_loc;
        double invlb1 = 0.;
        double rLarmor0 = 0., uT0[3] = { 0., 0., 0. };
        if (!straight) {
                double r = cfg->accuracy;
                const double k_threshold = 1E+09;
                if ((scheme == MODE_STRAGGLED) &&
                    (state->energy > k_threshold)) {
                        double f = k_threshold / state->energy;
                        if (f < 0.1) f = 0.1;
                        r *= f;
                }
                step_loc = r * density_i * Xtot;
                if (cfg->scattering == MODE_MIXED) {
                        if (c->step_first != 0) {
                                double mu0;
                                table_get_msc(scheme, material, state->energy,
                                    &mu0, &invlb1);
                                invlb1 *= density;
                        } else
                                invlb1 = c->step_invlb1;
                        const double stepT = cfg->accuracy / invlb1;
                        if (stepT < step_loc) step_loc = stepT;
                }
                /* Larmor radius and deflection direction
                 * (pumas.c:6352-6382). */
                if (c->magnetized) {
                        const double * const B = c->magnet;
                        uT0[0] = direction[1] * B[2] - direction[2] * B[1];
                        uT0[1] = direction[2] * B[0] - direction[0] * B[2];
                        uT0[2] = direction[0] * B[1] - direction[1] * B[0];
                        const double BT = sqrt(uT0[0] * uT0[0] +
                            uT0[1] * uT0[1] + uT0[2] * uT0[2]);
                        if (BT != 0.) {
                                rLarmor0 = momentum / (BT * LARMOR_FACTOR);
                                const double pinv = 1. / momentum;
                                uT0[0] *= pinv;
                                uT0[1] *= pinv;
                                uT0[2] *= pinv;
                        }
                }
                if (rLarmor0 > 0.) {
                        const double stepM = cfg->accuracy * rLarmor0;
                        if (stepM < step_loc) step_loc = stepM;
                }
        } else {
                if (grammage_max <= 0.)
                        step_loc = 1E+09 * density_i;
                else
                        step_loc = grammage_max * density_i;
        }
        c->step_first = 0;

        if (step_loc < STEP_MIN) step_loc = STEP_MIN;
        double step = (step_max_medium <= 0) ?
            step_loc :
            (step_max_medium < step_loc ? step_max_medium : step_loc);
        if ((*step_max_locals > 0.) && (step > *step_max_locals))
                step = *step_max_locals;

        *out_medium = medium;
        int event = EV_NONE;
        if (cfg->event & EV_LIMIT_DISTANCE) {
                const double d = cfg->limit_distance - state->distance;
                if (d <= step) {
                        step = d;
                        event = EV_LIMIT_DISTANCE;
                }
        }

        const double sgn = (cfg->direction == MODE_FORWARD) ? 1. : -1.;
        position[0] += step * sgn * direction[0];
        position[1] += step * sgn * direction[1];
        position[2] += step * sgn * direction[2];

        int end_medium = medium_locate(c, state);
        double end_position[3] = { position[0], position[1], position[2] };
        if (end_medium != medium) {
                /* Boundary check for a PUMAS_STEP_CHECK geometry. */
                const double step_min = (step < STEP_MIN) ? step : STEP_MIN;
                double pi[3];
                memcpy(pi, position, sizeof(pi));
                double s1 = 0., s2 = -step_min;
                position[0] = pi[0] + s2 * sgn * direction[0];
                position[1] = pi[1] + s2 * sgn * direction[1];
                position[2] = pi[2] + s2 * sgn * direction[2];
                int tmp_medium = medium_locate(c, state);
                if (tmp_medium != medium) {
                        if (tmp_medium != end_medium) end_medium = tmp_medium;
                        s1 = s2;
                        s2 = -step;
                        while (fabs(s1 - s2) > STEP_MIN) {
                                double s3 = 0.5 * (s1 + s2);
                                position[0] = pi[0] + s3 * sgn * direction[0];
                                position[1] = pi[1] + s3 * sgn * direction[1];
                                position[2] = pi[2] + s3 * sgn * direction[2];
                                tmp_medium = medium_locate(c, state);
                                if (tmp_medium == medium) {
                                        s2 = s3;
                                } else {
                                        s1 = s3;
                                        if (tmp_medium != end_medium)
                                                end_medium = tmp_medium;
                                }
                        }
                        position[0] = pi[0] + s2 * sgn * direction[0];
                        position[1] = pi[1] + s2 * sgn * direction[1];
                        position[2] = pi[2] + s2 * sgn * direction[2];
                        step += s1;
                        end_position[0] = pi[0] + s1 * sgn * direction[0];
                        end_position[1] = pi[1] + s1 * sgn * direction[1];
                        end_position[2] = pi[2] + s1 * sgn * direction[2];
                }
                event = EV_MEDIUM;
                *out_medium = end_medium;
        }

        /* End step locals (pumas.c:6488-6503), at the last point inside
         * the medium when the step crosses a boundary. */
        double Bi[3] = { 0., 0., 0. };
        if (c->magnetized) memcpy(Bi, c->magnet, sizeof(Bi));
        double density1 = density;
        if (*step_max_locals > 0.) {
                *step_max_locals = set_locals(c, medium, state, &density1);
                if (density1 <= 0.) return RC_DENSITY_ERROR;
        }
        if (event & EV_MEDIUM) {
                position[0] = end_position[0];
                position[1] = end_position[1];
                position[2] = end_position[2];
        }

        double k1 = state->energy, dk = 0.;
        const double dX = 0.5 * step * (density + density1);
        if ((scheme >= MODE_CSDA) && (scheme <= MODE_MIXED)) {
                const double X = Xtot - sgn * dX;
                if ((cfg->direction == MODE_FORWARD) &&
                    (X <= c->step_X_limit)) {
                        k1 = (cfg->event & EV_LIMIT_ENERGY) ?
                            cfg->limit_energy : 0.;
                        const double grammage =
                            state->grammage + Xtot - c->step_X_limit;
                        if ((grammage_max <= 0.) || (grammage < grammage_max)) {
                                grammage_max = grammage;
                                event = EV_LIMIT_ENERGY;
                        }
                } else if ((cfg->direction == MODE_BACKWARD) &&
                    (c->step_X_limit > 0.) && (X > c->step_X_limit)) {
                        k1 = (cfg->event & EV_LIMIT_ENERGY) ?
                            cfg->limit_energy : 0.;
                        const double grammage =
                            state->grammage + c->step_X_limit - Xtot;
                        if ((grammage_max <= 0.) || (grammage < grammage_max)) {
                                grammage_max = grammage;
                                event = EV_LIMIT_ENERGY;
                        }
                } else if (dX < EPSILON_X * Xtot) {
                        k1 -= sgn * cel_energy_loss(scheme, material, k1) * dX;
                        if ((cfg->event & EV_LIMIT_ENERGY) &&
                            (cfg->limit_energy > 0.)) {
                                if (((cfg->direction == MODE_FORWARD) &&
                                        (k1 < cfg->limit_energy)) ||
                                    ((cfg->direction == MODE_BACKWARD) &&
                                        (k1 > cfg->limit_energy))) {
                                        k1 = cfg->limit_energy;
                                        event = EV_LIMIT_ENERGY;
                                }
                        } else if (k1 < 0.) {
                                k1 = 0.;
                        }
                } else {
                        k1 = cel_kinetic_energy(scheme, material, X);
                }
        } else if (scheme == MODE_STRAGGLED) {
                double ratio;
                step_fluctuate(c, state, material, Xtot, dX, &k1, &ratio);
                dk = fabs(state->energy - k1);
                double kinetic_limit = -1.;
                if (cfg->direction == MODE_FORWARD) {
                        const double kinetic_min =
                            (cfg->event & EV_LIMIT_ENERGY) ?
                            cfg->limit_energy : 0.;
                        if (k1 <= kinetic_min) kinetic_limit = kinetic_min;
                } else {
                        if ((cfg->event & EV_LIMIT_ENERGY) &&
                            (k1 >= cfg->limit_energy))
                                kinetic_limit = cfg->limit_energy;
                }
                if (kinetic_limit >= 0.) {
                        const double grammage = state->grammage +
                            fabs(state->energy - kinetic_limit) / dk * dX;
                        k1 = kinetic_limit;
                        if ((grammage_max <= 0.) || (grammage < grammage_max)) {
                                grammage_max = grammage;
                                event = EV_LIMIT_ENERGY;
                        }
                }
                double Xmax = dX;
                if (grammage_max > 0.) {
                        const double dX1 = grammage_max - state->grammage;
                        if (Xmax > dX1) Xmax = dX1;
                }
                double k_x = -1.;
                {
                        double xs_del = del_cross_section(
                            material, state->energy);
                        const double tmp_del = del_cross_section(material, k1);
                        if (tmp_del > xs_del) xs_del = tmp_del;
                        if (xs_del <= 0.) goto no_del_event;
                        const double X_del = -log(rnd(c)) / xs_del;
                        if (X_del >= Xmax) goto no_del_event;
                        const double k_h = cel_kinetic_energy(
                            scheme, material, Xtot - sgn * X_del);
                        const double k_del = state->energy -
                            sgn * ratio * fabs(state->energy - k_h);
                        if (k_del <= 0.) goto no_del_event;
                        const double r =
                            del_cross_section(material, k_del) / xs_del;
                        if (rnd(c) > r) goto no_del_event;
                        k_x = k_del;
                        Xmax = X_del;
                        event = EV_DEL;
                }
        no_del_event:
                if (cfg->scattering == MODE_MIXED) {
                        double kmin, kmax;
                        if (k1 <= state->energy)
                                kmin = k1, kmax = state->energy;
                        else
                                kmax = k1, kmin = state->energy;
                        if (kmin < ph->K[1]) {
                                const double tmp = kmin;
                                kmin = kmax, kmax = tmp;
                        }
                        double lb_ehs = coulomb_ehs_length(material, kmin);
                        if (lb_ehs <= 0.) goto no_ehs_event;
                        const double X_ehs = -log(rnd(c)) * lb_ehs;
                        if (X_ehs >= Xmax) goto no_ehs_event;
                        const double k_h = cel_kinetic_energy(
                            scheme, material, Xtot - sgn * X_ehs);
                        const double k_ehs = state->energy -
                            sgn * ratio * fabs(state->energy - k_h);
                        if (k_ehs <= 0.) goto no_ehs_event;
                        const double r =
                            coulomb_ehs_length(material, k_ehs) / lb_ehs;
                        if ((r <= 0.) || (rnd(c) > 1. / r)) goto no_ehs_event;
                        k_x = k_ehs;
                        Xmax = X_ehs;
                        event = EV_COULOMB;
                no_ehs_event:;
                }
                if (k_x >= 0.) {
                        k1 = k_x;
                        grammage_max = state->grammage + Xmax;
                }
        }

        const double Xi = state->grammage;
        state->grammage += dX;
        const double sf0 = step;
        double h_int = 0.;
        if ((grammage_max > 0.) && (state->grammage >= grammage_max)) {
                const double dX_ = grammage_max - Xi;
                if ((fabs(density - density1) <= FLT_EPSILON) ||
                    (sf0 <= FLT_EPSILON)) {
                        step = dX_ * density_i;
                        h_int = dX_ / (state->grammage - Xi);
                } else {
                        const double drho = density1 - density;
                        double tmp = density * density + 2. * dX_ * drho / sf0;
                        tmp = (tmp > FLT_EPSILON) ? sqrt(tmp) : 0;
                        h_int = (tmp - density) / drho;
                        step *= h_int;
                }
                state->grammage = grammage_max;
                if (!(event & EV_LIMIT_ENERGY)) {
                        if (scheme <= MODE_MIXED) {
                                if (scheme != MODE_DISABLED)
                                        k1 = cel_kinetic_energy(scheme, material,
                                            Xtot - sgn * (state->grammage - Xi));
                                event = c->step_foreseen;
                        } else if (!(event & (EV_COULOMB | EV_DEL))) {
                                k1 = state->energy -
                                    sgn * (state->grammage - Xi) * dk / dX;
                                if (k1 < 0.) k1 = 0.;
                                event = EV_LIMIT_GRAMMAGE;
                        }
                }
                const double ds_ = step - sf0;
                position[0] += ds_ * sgn * direction[0];
                position[1] += ds_ * sgn * direction[1];
                position[2] += ds_ * sgn * direction[2];
        }

        int decayed = 0;
        double time_max = (cfg->event & EV_LIMIT_TIME) ? cfg->limit_time : 0.;
        if (cfg->decay == MODE_RANDOMISED) {
                if ((time_max <= 0.) || (c->lifetime < time_max)) {
                        time_max = c->lifetime;
                        decayed = 1;
                }
        }
        const double sf1 = step;
        if (straight && (scheme != MODE_DISABLED)) {
                const double Ti =
                    cel_proper_time(scheme, material, state->energy);
                if (time_max > 0.) {
                        const double Tf =
                            Ti - sgn * (time_max - state->time) * density;
                        if (Tf > 0.) {
                                const double dxT = fabs(Xtot -
                                    cel_grammage_as_time(scheme, material, Tf));
                                if (Xi + dxT < state->grammage) {
                                        event = EV_LIMIT_TIME;
                                        state->time = time_max;
                                        state->decayed = decayed;
                                        step = dxT * density_i;
                                        if (step > sf1) step = sf1;
                                        state->grammage = Xi + dxT;
                                        const double xf = Xtot - sgn * dxT;
                                        k1 = cel_kinetic_energy(
                                            scheme, material, xf);
                                }
                        }
                }
                if (event != EV_LIMIT_TIME) {
                        const double Tf = cel_proper_time(scheme, material, k1);
                        state->time += fabs(Tf - Ti) * density_i;
                }
        } else {
                const double p_f =
                    (k1 <= 0) ? momentum : sqrt(k1 * (k1 + 2. * ph->mass));
                const double ti = state->time;
                state->time +=
                    0.5 * step * ph->mass * (1. / momentum + 1. / p_f);
                if ((time_max > 0.) && (state->time >= time_max)) {
                        event = EV_LIMIT_TIME;
                        state->time = time_max;
                        state->decayed = decayed;
                        const double a = (momentum / p_f - 1.) / sf1;
                        const double cc =
                            -2. * (time_max - ti) * momentum / ph->mass;
                        if (a != 0.) {
                                double delta = 1. - a * cc;
                                if (delta < 0.) delta = 0.;
                                step = 1. / a * (sqrt(delta) - 1.);
                        } else {
                                step = -0.5 * cc;
                        }
                        if (step < 0.) step = 0.;
                        if (scheme != MODE_DISABLED) {
                                const double p1 = momentum / (1 + a * step);
                                k1 = sqrt(p1 * p1 - ph->mass * ph->mass) -
                                    ph->mass;
                                if (k1 < 0.) k1 = 0.;
                        }
                        const double Xf = Xi + dX;
                        if (density == density1)
                                state->grammage = Xi + step * density;
                        else
                                state->grammage = Xi +
                                    step * (density +
                                               0.5 * step / sf0 *
                                                   (density1 - density));
                        if (state->grammage > Xf) state->grammage = Xf;
                }
        }
        if (event == EV_LIMIT_TIME) {
                const double ds_ = step - sf1;
                position[0] += ds_ * sgn * direction[0];
                position[1] += ds_ * sgn * direction[1];
                position[2] += ds_ * sgn * direction[2];
        }

        c->step_event = event;
        state->energy = k1;
        state->distance += step;

        if (cfg->scattering == MODE_MIXED) {
                double mu0, invlb1_;
                if (state->energy <= 0.) {
                        c->step_invlb1 = invlb1;
                } else {
                        table_get_msc(
                            scheme, material, state->energy, &mu0, &invlb1_);
                        c->step_invlb1 = density1 * invlb1_;
                }
        }
        *density_end = density1;

        /* End point field and magnetic deflection (pumas.c:6833-6911). */
        double rLarmor1 = 0., uT1[3] = { 0., 0., 0. };
        if (c->magnetized) {
                double B[3] = { c->magnet[0], c->magnet[1], c->magnet[2] };
                int magnetized = c->magnetized;
                if (h_int > 0.) {
                        B[0] = Bi[0] + h_int * (B[0] - Bi[0]);
                        B[1] = Bi[1] + h_int * (B[1] - Bi[1]);
                        B[2] = Bi[2] + h_int * (B[2] - Bi[2]);
                        magnetized =
                            (B[0] * B[0] + B[1] * B[1] + B[2] * B[2] == 0.);
                }
                if (magnetized != 0) {
                        uT1[0] = direction[1] * B[2] - direction[2] * B[1];
                        uT1[1] = direction[2] * B[0] - direction[0] * B[2];
                        uT1[2] = direction[0] * B[1] - direction[1] * B[0];
                        const double BT = sqrt(uT1[0] * uT1[0] +
                            uT1[1] * uT1[1] + uT1[2] * uT1[2]);
                        if (BT != 0.) {
                                const double p = (state->energy <= 0) ?
                                    momentum :
                                    sqrt(state->energy *
                                        (state->energy + 2. * ph->mass));
                                rLarmor1 = p / (BT * LARMOR_FACTOR);
                                const double pinv = 1. / p;
                                uT1[0] *= pinv;
                                uT1[1] *= pinv;
                                uT1[2] *= pinv;
                        }
                }
        }
        if ((rLarmor0 > 0.) || (rLarmor1 > 0.)) {
                const double u[3] = { direction[0], direction[1],
                        direction[2] };
                const double theta0 =
                    (rLarmor0 > 0.) ? state->charge * step / rLarmor0 : 0.;
                const double theta1 =
                    (rLarmor1 > 0.) ? state->charge * step / rLarmor1 : 0.;
                double theta = 0.5 * (theta0 + theta1);
                if (cfg->direction == MODE_BACKWARD) theta = -theta;
                double cs = cos(theta);
                double sn = sin(theta);
                double v[3];
                int i;
                for (i = 0; i < 3; i++) v[i] = 0.5 * (uT0[i] + uT1[i]);
                double nrmv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
                if (nrmv > 0.) {
                        nrmv = 1. / sqrt(nrmv);
                        for (i = 0; i < 3; i++) v[i] *= nrmv;
                } else {
                        cs = 1.;
                        sn = 0.;
                }
                for (i = 0; i < 3; i++) direction[i] = cs * u[i] + sn * v[i];
                const double norm = 1. / sqrt(direction[0] * direction[0] +
                                             direction[1] * direction[1] +
                                             direction[2] * direction[2]);
                for (i = 0; i < 3; i++) direction[i] *= norm;
        }

        if ((invlb1 > 0.) || (c->step_invlb1 > 0.)) {
                double ilb1 = 0.25 * step * (invlb1 + c->step_invlb1);
                if (ilb1 > 1.) ilb1 = 1.;
                double mu;
                do {
                        mu = -ilb1 * log(rnd(c));
                } while (mu > 1.);
                step_rotate_direction(c, state, mu);
        }
        return RC_SUCCESS;
}

/* transport_with_stepping (pumas.c:5194-5514), uniform locals, no
 * recorder. Returns the end event and updates *medium_ptr. */
static int transport_with_stepping(struct port_ctx * c,
    struct oracle_state * state, int * medium_ptr, double density,
    double step_max_medium, double step_max_locals, int * status)
{
        const struct oracle_config * cfg = c->cfg;
        int medium = *medium_ptr;
        int material = medium_material(c, medium);
        const int scheme = cfg->energy_loss;
        int straight = ((cfg->scattering == MODE_DISABLED) &&
                           (scheme <= MODE_MIXED) &&
                           (step_max_locals <= 0.) && !c->magnetized) ? 1 : 0;
        c->step_event = EV_NONE;
        double ti = state->time;
        double wi = state->weight;
        double Xi = state->grammage;
        double dei, Xf;
        if (scheme > MODE_DISABLED) {
                const double ki = state->energy;
                Xf = cel_grammage(scheme, material, ki);
                dei = 1. / cel_energy_loss(scheme, material, ki);
        } else {
                Xf = dei = 0.;
        }
        if ((cfg->event & EV_LIMIT_DISTANCE) &&
            (state->distance >= cfg->limit_distance))
                return EV_LIMIT_DISTANCE;
        if ((cfg->event & EV_LIMIT_GRAMMAGE) &&
            (state->grammage >= cfg->limit_grammage))
                return EV_LIMIT_GRAMMAGE;
        if ((cfg->event & EV_LIMIT_TIME) && (state->time >= cfg->limit_time))
                return EV_LIMIT_TIME;
        if (state->weight <= 0.) return EV_WEIGHT;

        double grammage_max;
        c->step_event = EV_NONE;
        c->step_first = 1;
        c->step_X_limit = (cfg->event & EV_LIMIT_ENERGY) ?
            cel_grammage((scheme > MODE_DISABLED) ? scheme : MODE_CSDA,
                material, cfg->limit_energy) :
            0.;
        c->step_invlb1 = 0;
        transport_limit(c, state, material, Xi, Xf, &grammage_max);
        if (c->step_event) return c->step_event;

        int step_index = 1;
        for (;;) {
                if (step_index > 1) {
                        const int m = medium_locate(c, state);
                        step_max_medium = medium_step(c, state, m);
                        if (step_max_medium > 0.)
                                step_max_medium += 0.5 * STEP_MIN;
                }
                int new_medium = -1;
                const int rc = step_transport(c, state, straight, medium,
                    density, grammage_max, step_max_medium, &step_max_locals,
                    &density, &new_medium);
                if (rc != RC_SUCCESS) {
                        *status = rc;
                        return c->step_event;
                }
                step_index++;
                if (!c->step_event) continue;

                if ((cfg->direction == MODE_BACKWARD) &&
                    (cfg->energy_loss >= MODE_CSDA)) {
                        const double wt = (cfg->decay == MODE_WEIGHTED) ?
                            exp(-fabs(state->time - ti) / ph->ctau) :
                            1.;
                        state->weight = wi * wt * dei *
                            cel_energy_loss(scheme, material, state->energy);
                } else if (cfg->decay == MODE_WEIGHTED) {
                        state->weight =
                            wi * exp(-fabs(state->time - ti) / ph->ctau);
                }

                if (c->step_event & (EV_LIMIT | EV_WEIGHT | EV_DECAY)) {
                        break;
                } else if (c->step_event & (EV_DEL | EV_COULOMB)) {
                        if (c->step_event & EV_DEL) {
                                transport_do_del(c, state, material);
                                if (c->step_event < 0) {
                                        *status = RC_INTERNAL_ERROR;
                                        c->step_event = EV_NONE;
                                        break;
                                }
                                if ((cfg->event & c->step_event) ||
                                    c->step_event == EV_WEIGHT)
                                        break;
                                c->step_first = 1;
                                c->step_invlb1 = 0;
                        } else {
                                transport_do_ehs(c, state, material);
                                if (cfg->event & c->step_event) break;
                        }
                        /* Locals update (pumas.c:5403-5414). */
                        if (step_max_locals > 0.) {
                                step_max_locals =
                                    set_locals(c, medium, state, &density);
                                if (density <= 0.) {
                                        *status = RC_DENSITY_ERROR;
                                        return c->step_event;
                                }
                        }
                } else if (c->step_event & EV_MEDIUM) {
                        medium = new_medium;
                        if ((medium < 0) || (cfg->event & EV_MEDIUM)) break;
                        material = medium_material(c, medium);
                        step_max_locals = set_locals(c, medium, state, &density);
                        if (density <= 0.) {
                                *status = RC_DENSITY_ERROR;
                                return c->step_event;
                        }
                        straight = ((cfg->scattering == MODE_DISABLED) &&
                                       (scheme <= MODE_MIXED) &&
                                       (step_max_locals <= 0.) &&
                                       !c->magnetized) ? 1 : 0;
                        const int tmp_scheme =
                            scheme > MODE_DISABLED ? scheme : MODE_CSDA;
                        c->step_X_limit = (cfg->event & EV_LIMIT_ENERGY) ?
                            cel_grammage(
                                tmp_scheme, material, cfg->limit_energy) :
                            0.;
                        c->step_first = 1;
                        c->step_invlb1 = 0;
                } else {
                        *status = RC_INTERNAL_ERROR;
                        break;
                }

                ti = state->time;
                wi = state->weight;
                Xi = state->grammage;
                if (cfg->energy_loss >= MODE_CSDA) {
                        const double ki = state->energy;
                        Xf = cel_grammage(scheme, material, ki);
                        dei = 1. / cel_energy_loss(scheme, material, ki);
                }
                transport_limit(c, state, material, Xi, Xf, &grammage_max);
                if (c->step_event) break;
        }

        if (cfg->direction == MODE_FORWARD) {
                const double kinetic_min =
                    (cfg->event & EV_LIMIT_ENERGY) ? cfg->limit_energy : 0.;
                if (fabs(state->energy - kinetic_min) < FLT_EPSILON)
                        state->energy = kinetic_min;
        } else {
                if ((cfg->event & EV_LIMIT_ENERGY) &&
                    (fabs(state->energy - cfg->limit_energy) < FLT_EPSILON))
                        state->energy = cfg->limit_energy;
        }
        *medium_ptr = medium;
        return c->step_event;
}

/* pumas_context_transport (pumas.c:3114-3251) for one event. */
static int context_transport(struct port_ctx * c, struct oracle_state * state,
    int * event, int media[2])
{
        const struct oracle_config * cfg = c->cfg;
        *event = EV_NONE;
        media[0] = media[1] = -1;
        if (ph == NULL) return RC_PHYSICS_ERROR;
        if (state->decayed) {
                *event = EV_DECAY;
                return RC_SUCCESS;
        }
        {
                const double * const u = state->direction;
                const double norm2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
                if (fabs(norm2 - 1) > FLT_EPSILON) return RC_DIRECTION_ERROR;
        }
        if ((cfg->accuracy <= 0) || (cfg->accuracy > 1))
                return RC_ACCURACY_ERROR;
        if ((cfg->direction == MODE_BACKWARD) &&
            (cfg->energy_loss > MODE_CSDA) && (ph->cutoff < 1E-02))
                return RC_ACCURACY_ERROR;

        int medium = medium_locate(c, state);
        double step_max_medium = medium_step(c, state, medium);
        media[0] = medium;
        media[1] = -1;
        if (medium < 0) {
                *event = EV_MEDIUM;
                return RC_SUCCESS;
        } else if (step_max_medium > 0.)
                step_max_medium += 0.5 * STEP_MIN;
        double density;
        const double step_max_locals = set_locals(c, medium, state, &density);
        if ((step_max_locals > 0.) && (step_max_locals < step_max_medium))
                step_max_medium = step_max_locals;
        if (density <= 0.) return RC_DENSITY_ERROR;

        if (cfg->decay == MODE_RANDOMISED) {
                const double u = rnd(c);
                c->lifetime = state->time - ph->ctau * log(u);
        }

        int do_stepping = 1;
        int e = EV_NONE, status = RC_SUCCESS;
        if ((step_max_medium <= 0.) && (step_max_locals <= 0.) &&
            (cfg->energy_loss <= MODE_CSDA)) {
                if ((cfg->energy_loss == MODE_DISABLED) &&
                    ((cfg->event & EV_LIMIT) == 0)) {
                        return RC_MISSING_LIMIT;
                } else if ((cfg->scattering == MODE_DISABLED) &&
                    (cfg->energy_loss == MODE_CSDA)) {
                        do_stepping = 0;
                }
        }
        if (do_stepping) {
                e = transport_with_stepping(c, state, &medium, density,
                    step_max_medium, step_max_locals, &status);
        } else {
                e = transport_with_csda(
                    c, state, medium_material(c, medium), density, &status);
        }
        *event = e;
        media[1] = medium;
        return status;
}

/* The per element DEL tables of the loaded dump (the reference's own
 * pumas_physics_create output), in the dump's layout: CSn and CSn_dK
 * [4][n_elements][n_energies], the DCS tables [3][n_elements][n_energies]
 * [n_table_dcs][2], the envelope exponents [3][n_elements][n_energies] and
 * the DCS grid. Returns the sizes through dims[3] = {n_elements,
 * n_energies, n_table_dcs} when the arrays are NULL. */
int oracle_port_dcs_tables(int * dims, double * csn, double * csn_dk,
    float * dcs, float * alpha, float * x)
{
        if (ph == NULL) return RC_PHYSICS_ERROR;
        const int nel = ph->n_elements, nE = ph->n_energies;
        const int nx = ph->n_table_dcs;
        dims[0] = nel;
        dims[1] = nE;
        dims[2] = nx;
        if (csn == NULL) return RC_SUCCESS;
        const size_t n4 = 4 * (size_t)nel * nE, n3 = 3 * (size_t)nel * nE;
        memcpy(csn, ph->CSn, n4 * sizeof(double));
        memcpy(csn_dk, ph->CSn_dK, n4 * sizeof(double));
        memcpy(dcs, ph->DCS, n3 * 2 * nx * sizeof(float));
        size_t i;
        for (i = 0; i < n3; i++) alpha[i] = ph->DCS_env[2 * i];
        memcpy(x, ph->DCS_x, nx * sizeof(float));
        return RC_SUCCESS;
}

/* ------------------------------------------------------------------------ */
/* Per element DEL tables (the device table builder's CPU restatement).     */
/* ------------------------------------------------------------------------ */

/* math_diff3 (pumas.c:9944-9955). */
static double tab_diff3(
    double x0, double x1, double x2, double y0, double y1, double y2)
{
        const double h1 = x1 - x0;
        const double h2 = x2 - x0;
        const double delta = h1 * h2 * (h2 - h1);
        const double c1 = h2 * h2 / delta;
        const double c2 = -h1 * h1 / delta;
        const double c0 = -(c1 + c2);
        return c0 * y0 + c1 * y1 + c2 * y2;
}

/* math_pchip_initialise without known derivatives (pumas.c:9958-10023). */
static void tab_pchip(int n, const double * x, const double * y, double * m)
{
        if (n >= 3) {
                m[0] = (y[1] - y[0]) / (x[1] - x[0]);
                n--;
                x++;
                y++;
                m++;
        }
        if (n == 1) {
                m[0] = 0;
        } else if (n == 2) {
                const double d = (y[1] - y[0]) / (x[1] - x[0]);
                m[0] = m[1] = d;
        } else {
                int i;
                for (i = 1; i < n - 1; i++) {
                        const double h1 = x[i] - x[i - 1];
                        const double h2 = x[i + 1] - x[i];
                        const double S1 = (y[i] - y[i - 1]) / h1;
                        const double S2 = (y[i + 1] - y[i]) / h2;
                        const double tmp = S1 * S2;
                        if (tmp > 0) {
                                const double a =
                                    (h1 + 2 * h2) / (3 * (h1 + h2));
                                m[i] = tmp / ((1 - a) * S1 + a * S2);
                        } else {
                                m[i] = 0.;
                        }
                }
                m[0] = tab_diff3(x[0], x[1], x[2], y[0], y[1], y[2]);
                m[n - 1] = tab_diff3(x[n - 1], x[n - 2], x[n - 3], y[n - 1],
                    y[n - 2], y[n - 3]);
        }
}

/* The restricted cross section of a DEL process: compute_dcs_integral in
 * mode 0 with 180 points from cutoff K to K (pumas.c:10837-10888,
 * 10730-10732), a 6 point Gauss-Legendre rule on equal intervals of ln q
 * (math_gauss_quad, pumas.c:12410-12450), and the analytic integral of the
 * ionisation DCS (dcs_ionisation_integrate, pumas.c:11140-11183). */
static double tab_csn(int process, const struct port_element * e, double K)
{
        static const double xg[6] = { 0.0337652428984240, 0.1693953067668678,
                0.3806904069584016, 0.6193095930415985, 0.8306046932331322,
                0.9662347571015760 };
        static const double wg[6] = { 0.0856622461895852, 0.1803807865240693,
                0.2339569672863455, 0.2339569672863455, 0.1803807865240693,
                0.0856622461895852 };
        const double xlow = ph->cutoff, xhigh = 1.;
        if (process == 3) {
                const double P2 = K * (K + 2. * ph->mass);
                const double E = K + ph->mass;
                const double Wr = 2. * ELECTRON_MASS * P2 /
                    (ph->mass * ph->mass +
                        ELECTRON_MASS * (ELECTRON_MASS + 2. * E));
                const double qlow = K * xlow, qhigh = K * xhigh;
                double Wmax = Wr;
                if (Wmax < qlow) return 0.;
                if (Wmax > qhigh) Wmax = qhigh;
                double Wmin = (13.6 / 19.2) * e->I;
                if (qlow >= Wmin) Wmin = qlow;
                if (Wmax <= Wmin) return 0.;
                const double E2 = E * E;
                const double beta2 = P2 / E2;
                const double a0 = 0.5 / E2;
                const double a1 = beta2 / Wr;
                const double I = a0 * (Wmax - Wmin) - a1 * log(Wmax / Wmin) +
                    1. / Wmin - 1. / Wmax;
                return 2 * PI_ * ELECTRON_MASS * ELECTRON_RADIUS *
                    ELECTRON_RADIUS * e->Z * AVOGADRO_NUMBER /
                    (e->A * 1E-03 * beta2) * I;
        }
        double qmin = 0, qmax;
        if (process == 2) {
                const double M = 0.5 * (NEUTRON_MASS + PROTON_MASS);
                const double mpi = PION_MASS;
                qmin = mpi + 0.5 * mpi * mpi / M;
                qmax = K + ph->mass - 0.5 * (M + ph->mass * ph->mass / M);
        } else {
                const double Z13 = pow(e->Z, 1. / 3.);
                const double sqrte = 1.648721271;
                qmax = K + ph->mass * (1. - 0.75 * sqrte * Z13);
                if (process == 1) qmin = 4 * ELECTRON_MASS;
        }
        double qlow = xlow * K;
        if (qlow < qmin) qlow = qmin;
        double qhigh = xhigh * K;
        if (qhigh > qmax) qhigh = qmax;
        if (qlow >= qhigh) return 0.;
        const int n_itv = 30;
        double x0 = log(qlow);
        const double h = (log(qhigh) - x0) / n_itv;
        double s = 0.;
        int i, j;
        for (i = 0; i < n_itv; i++, x0 += h) {
                for (j = 0; j < 6; j++) {
                        const double xi = x0 + xg[j] * h;
                        const double wi = wg[j] * h;
                        const double qi = exp(xi);
                        const double y = dcs_process(process, e, K, qi) * qi;
                        s += y * wi;
                }
        }
        return s / (K + ph->mass);
}

/* One row of the DCS table (dcs_tabulate_row, pumas.c:11358-11438). */
static void tab_dcs_row(int process, int iel, int row, const double * x,
    double cs, float * data, float * alpha)
{
        const int n = ph->n_table_dcs;
        int i;
        if (cs <= 0.) {
                for (i = 0; i < 2 * n; i++) data[i] = 0.f;
                *alpha = 0.f;
                return;
        }
        const double K = ph->K[row];
        const struct port_element * e = ph->element + iel;
        double y[64], m[64];
        int imin = n, imax = n - 1;
        for (i = 0; i < n; i++) {
                const double d = dcs_process(process, e, K, K * exp(x[i]));
                if (d > 0) {
                        if (i < imin) imin = i;
                        y[i] = log(d);
                } else if (imin < n) {
                        imax = i - 1;
                        break;
                }
        }
        if (imin <= imax)
                tab_pchip(imax - imin + 1, x + imin, y + imin, m + imin);
        double qmin, qmax;
        if (process == 2) {
                dcs_photonuclear_range(ph->mass, K, &qmin, &qmax);
                qmin += qmin;
        } else {
                dcs_pair_production_range(e->Z, ph->mass, K, &qmin, &qmax);
                if (process == 0)
                        qmin = 0.5 * ph->cutoff * K;
                else
                        qmin *= 4;
        }
        const double qrev = 0.6 * K;
        qmax *= 0.5;
        if (qmax > qrev) qmax = qrev;
        const double xmin = log(qmin / K), xmax = log(qmax / K);
        int ia0 = imax, ia1 = imin;
        for (i = 0; i < n; i++) {
                if ((i >= imin) && (i <= imax)) {
                        data[2 * i] = (float)y[i];
                        data[2 * i + 1] = (float)m[i];
                        if ((x[i] > xmin) && (x[i] < xmax)) {
                                if (ia0 > i) ia0 = i;
                                if (ia1 < i) ia1 = i;
                        }
                } else {
                        data[2 * i] = 0.f;
                        data[2 * i + 1] = 0.f;
                }
        }
        if ((ia0 < ia1) && (ia0 < n - 1)) {
                const int ia = (3 * ia0 + ia1) / 4;
                double a = -m[ia];
                if (fabs(a - 1.) <= 0.1) a = 1.;
                *alpha = (float)a;
        } else {
                *alpha = 0.f;
        }
}

/* The per element DEL tables of the loaded physics computed from its
 * elements, energy grid and DCS models, as the device table builder does
 * (gp_tabulate.cu), with OpenMP over processes, elements and rows: CSn and
 * CSn_dK [4][n_elements][n_energies], the DCS tables and the envelope
 * exponents (layouts of oracle_port_dcs_tables). */
int oracle_port_dcs_tabulate(double * csn, double * csn_dk, float * dcs,
    float * alpha, int n_threads)
{
        if (ph == NULL) return RC_PHYSICS_ERROR;
        const int nel = ph->n_elements, nE = ph->n_energies;
        const int n = ph->n_table_dcs;
        if (n > 64) return RC_VALUE_ERROR;
        /* The DCS sampling grid of compute_dcs_table (pumas.c:11643-11672). */
        double x[64];
        const int p = 20, m = n - p;
        double xrev;
        int i;
        if (m > 0) {
                xrev = 0.6;
                const double x0 = log(ph->cutoff);
                const double dx = log(xrev / ph->cutoff) / (m - 1);
                for (i = 0; i < m; i++) x[i] = x0 + i * dx;
        } else {
                xrev = ph->cutoff;
        }
        const double dxmin = 1E-03;
        const double dx = log((0.95 - xrev) / dxmin) / ((m > 0) ? p : p - 1);
        for (i = 0; i < p; i++) x[n - 1 - i] = log(0.95 - dxmin * exp(i * dx));

        long k;
        const long n4 = 4L * nel * nE, n3 = 3L * nel * nE;
#ifdef _OPENMP
        if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(n_threads)
#endif
        for (k = 0; k < n4; k++) {
                const int row = (int)(k % nE);
                const int iel = (int)((k / nE) % nel);
                const int process = (int)(k / ((long)nE * nel));
                csn[k] = (row == 0) ? 0. :
                    tab_csn(process, ph->element + iel, ph->K[row]);
        }
        for (k = 0; k < 4L * nel; k++)
                tab_pchip(nE, ph->K, csn + k * nE, csn_dk + k * nE);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8) num_threads(n_threads)
#endif
        for (k = 0; k < n3; k++) {
                const int row = (int)(k % nE);
                const int iel = (int)((k / nE) % nel);
                const int process = (int)(k / ((long)nE * nel));
                tab_dcs_row(process, iel, row, x, csn[k],
                    dcs + k * 2 * n, alpha + k);
        }
        for (k = 0; k < 3L * nel; k++) {
                float * a = alpha + k * nE;
                int n0 = 0, row;
                float a0 = 0.f;
                for (row = 0; row < nE; row++) {
                        if (a[row] > 0.f) {
                                n0 = row;
                                a0 = a[row];
                                break;
                        }
                }
                for (row = 0; row < n0; row++) a[row] = a0;
        }
        return RC_SUCCESS;
}

int oracle_port_max_threads(void)
{
#ifdef _OPENMP
        return omp_get_max_threads();
#else
        return 1;
#endif
}

/* Transport a batch of events, one transport call per event. */
int oracle_port_transport(const struct oracle_config * cfg,
    const struct gpumas_geometry * geometry, int64_t n, uint64_t first_event,
    struct oracle_state * states, struct oracle_result * results,
    int n_threads)
{
        if (ph == NULL) return RC_PHYSICS_ERROR;
        int64_t k;
#ifdef _OPENMP
        if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(n_threads)
#endif
        for (k = 0; k < n; k++) {
                struct port_ctx c;
                memset(&c, 0, sizeof(c));
                c.cfg = cfg;
                c.geometry = geometry;
                c.rng.seed = cfg->seed;
                c.rng.event = first_event + k;
                c.rng.n = 0;
                struct oracle_result * r = results + k;
                if (cfg->carry) {
                        oracle_stream_seek(&c.rng, r->draws);
                        c.randn_done = r->randn_done;
                        c.randn_next = r->randn_next;
                }
                int event, media[2];
                const int rc = context_transport(&c, states + k, &event, media);
                r->event = event;
                r->medium_in = media[0];
                r->medium_out = media[1];
                r->status = rc;
                r->steps = c.steps;
                r->randn_done = c.randn_done;
                r->draws = c.rng.n;
                r->randn_next = c.randn_next;
        }
        return RC_SUCCESS;
}

/* Tabulated properties for known answer tests, with the same meaning as
 * oracle_ref_property. */
int oracle_port_property(int property, int scheme, int material,
    double kinetic, double * value)
{
        if (ph == NULL) return RC_PHYSICS_ERROR;
        switch (property) {
        case 0:
                *value = cel_grammage(scheme, material, kinetic);
                return RC_SUCCESS;
        case 1:
                *value = cel_proper_time(scheme, material, kinetic);
                return RC_SUCCESS;
        case 2:
                *value = cel_kinetic_energy(scheme, material, kinetic);
                return RC_SUCCESS;
        case 3:
                *value = cel_energy_loss(scheme, material, kinetic);
                return RC_SUCCESS;
        case 4:
                *value = cel_straggling(material, kinetic);
                return RC_SUCCESS;
        default:
                return RC_INDEX_ERROR;
        }
}

/* Philox stream access, for checking other implementations of it. */
double oracle_port_uniform(
    uint64_t seed, uint32_t domain, uint64_t event, uint64_t n)
{
        return oracle_uniform(seed, domain, event, n);
}

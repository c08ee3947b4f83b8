/*
 * gp_tabulate.cu -- device tabulation of the per element DEL tables of a
 * physics: the part of the reference's table builder (pumas_physics_create)
 * that evaluates the exact DCS models millions of times.
 *
 * For every DEL process (bremsstrahlung, pair production, photonuclear,
 * ionisation), atomic element and row of the kinetic energy grid:
 *
 *   - the restricted cross section CSn, the integral of the DCS over the
 *     energy transfer q from cutoff K to K (compute_dcs_integral in mode 0
 *     with 180 points, pumas.c:10837-10888 called at 10730-10732): a 6 point
 *     Gauss-Legendre rule on 30 equal intervals of ln q
 *     (math_gauss_quad, pumas.c:12410-12450), the analytic integral for
 *     ionisation (dcs_ionisation_integrate, pumas.c:11140-11183);
 *   - its PCHIP derivative coefficients over the energy grid
 *     (compute_pchip_elements_coeffs, pumas.c:10116-10137, with
 *     math_pchip_initialise, pumas.c:9958-10023);
 *   - for the three radiative processes, the DCS interpolation table: the
 *     logarithm of the DCS on the 36 point grid of x = ln(q / K) and its
 *     PCHIP slopes, stored in single precision, with the exponent of the
 *     DCS envelope (dcs_tabulate_row, pumas.c:11358-11438, and the low
 *     energy rows of compute_dcs_table, pumas.c:11683-11699).
 *
 * Each quadrature point (and each DCS table point) is one GPU thread; the
 * sums, the slopes and the table rows are then made by one thread each, in
 * the reference's order. This file is compiled without floating point
 * contraction, so that every expression rounds as the reference's C code
 * does; the DCS models are the engine's device forms (gp_device.cuh) and
 * its logarithm / exponential, so values agree with the reference's to a
 * few ulp. What this file does not build: the energy loss tables, their
 * cumulative integrals, the multiple scattering tables and the envelope
 * maxima, which the reference computes from these quantities on the host.
 */
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "gp_context.h"
#include "gp_io.cuh"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Points of the restricted cross section integrals (pumas.c:10730-10735)
 * and of the Gauss-Legendre rule of math_gauss_quad (pumas.c:12415). */
#define GP_TAB_NINT 180
#define GP_TAB_NGQ 6
#define GP_TAB_NITV ((GP_TAB_NINT + GP_TAB_NGQ - 1) / GP_TAB_NGQ)

/* The 6 point Gauss-Legendre nodes and weights on [0, 1], with the
 * reference's digits (math_gauss_quad_coefficients, pumas.c:12463-12561). */
__constant__ double gp_tab_gq_x[GP_TAB_NGQ] = { 0.0337652428984240,
        0.1693953067668678, 0.3806904069584016, 0.6193095930415985,
        0.8306046932331322, 0.9662347571015760 };
__constant__ double gp_tab_gq_w[GP_TAB_NGQ] = { 0.0856622461895852,
        0.1803807865240693, 0.2339569672863455, 0.2339569672863455,
        0.1803807865240693, 0.0856622461895852 };

/* Integration range of compute_dcs_integral for a radiative process
 * (pumas.c:10850-10874); returns 0 when it is empty. */
static __device__ int gp_tab_range(const gp_tables & T, int process,
    const gp_element & el, double K, double * x0, double * x1)
{
        const double xlow = T.cutoff, xhigh = 1.;
        double qmin = 0, qmax;
        if (process == 2) {
                const double M = 0.5 * (GP_NEUTRON_MASS + GP_PROTON_MASS);
                const double mpi = GP_PION_MASS;
                qmin = mpi + 0.5 * mpi * mpi / M;
                qmax = K + T.mass - 0.5 * (M + T.mass * T.mass / M);
        } else {
                /* Z^1/3 as evaluated on the host at load time. */
                const double sqrte = 1.648721271;
                qmax = K + T.mass * (1. - 0.75 * sqrte * el.z13);
                if (process == 1) qmin = 4 * GP_ELECTRON_MASS;
        }
        double qlow = xlow * K;
        if (qlow < qmin) qlow = qmin;
        double qhigh = xhigh * K;
        if (qhigh > qmax) qhigh = qmax;
        if (qlow >= qhigh) return 0;
        *x0 = gp_log(qlow);
        *x1 = gp_log(qhigh);
        return 1;
}

/* One quadrature point of a restricted cross section: point p of
 * (process, element, row), weighted by its Gauss weight. Row 0 (K = 0) has
 * none. */
__global__ void gp_kernel_tab_points(const gp_tables T, double * out)
{
        const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
        const int nE = T.n_energies;
        const long n = 3L * T.n_elements * nE * GP_TAB_NINT;
        if (t >= n) return;
        const int p = (int)(t % GP_TAB_NINT);
        const long r = t / GP_TAB_NINT;
        const int row = (int)(r % nE);
        const int iel = (int)((r / nE) % T.n_elements);
        const int process = (int)(r / ((long)nE * T.n_elements));
        double x0, x1;
        const double K = T.K[row];
        const gp_element & el = T.element[iel];
        if ((row == 0) || !gp_tab_range(T, process, el, K, &x0, &x1)) {
                out[t] = 0.;
                return;
        }
        /* The iterator's interval origin advances by h at each interval. */
        const double h = (x1 - x0) / GP_TAB_NITV;
        const int itv = p / GP_TAB_NGQ, j = p % GP_TAB_NGQ;
        double xa = x0;
        for (int i = 0; i < itv; i++) xa += h;
        const double xi = xa + gp_tab_gq_x[j] * h;
        const double wi = gp_tab_gq_w[j] * h;
        const double qi = gp_exp(xi);
        const double y = gp_dcs_process(T, process, el, K, qi) * qi;
        out[t] = y * wi;
}

/* The restricted cross sections CSn[process][element][row]: sums of the
 * quadrature points in their order, divided by K + m, and the analytic
 * integral of the ionisation DCS. */
__global__ void gp_kernel_tab_csn(const gp_tables T, const double * points,
    double * csn)
{
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        const int nE = T.n_energies;
        if (t >= 4 * T.n_elements * nE) return;
        const int row = t % nE;
        const int iel = (t / nE) % T.n_elements;
        const int process = t / (nE * T.n_elements);
        const double K = T.K[row];
        if (row == 0) {
                csn[t] = 0.;
                return;
        }
        if (process < 3) {
                const double * y = points + (long)t * GP_TAB_NINT;
                double s = 0.;
                for (int p = 0; p < GP_TAB_NINT; p++) s += y[p];
                csn[t] = s / (K + T.mass);
                return;
        }
        /* dcs_ionisation_integrate in mode 0 (pumas.c:11140-11183). */
        const gp_element & el = T.element[iel];
        const double xlow = T.cutoff, xhigh = 1.;
        const double P2 = K * (K + 2. * T.mass);
        const double E = K + T.mass;
        const double Wr = 2. * GP_ELECTRON_MASS * P2 /
            (T.mass * T.mass +
                GP_ELECTRON_MASS * (GP_ELECTRON_MASS + 2. * E));
        const double qlow = K * xlow;
        const double qhigh = K * xhigh;
        double Wmax = Wr;
        double I = 0.;
        if (Wmax >= qlow) {
                if (Wmax > qhigh) Wmax = qhigh;
                double Wmin = (13.6 / 19.2) * el.I;
                if (qlow >= Wmin) Wmin = qlow;
                if (Wmax > Wmin) {
                        const double E2 = E * E;
                        const double beta2 = P2 / E2;
                        const double a0 = 0.5 / E2;
                        const double a1 = beta2 / Wr;
                        I = a0 * (Wmax - Wmin) - a1 * gp_log(Wmax / Wmin) +
                            1. / Wmin - 1. / Wmax;
                        I = 2 * M_PI * GP_ELECTRON_MASS * GP_ELECTRON_RADIUS *
                            GP_ELECTRON_RADIUS * el.Z * GP_AVOGADRO /
                            (el.A * 1E-03 * beta2) * I;
                }
        }
        csn[t] = I;
}

/* math_diff3 (pumas.c:9944-9955). */
static __device__ double gp_tab_diff3(
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

/* math_pchip_initialise without known derivatives (pumas.c:9958-10023):
 * the slopes m of the monotone cubic through (x, y), n nodes. */
static __device__ void gp_tab_pchip(int n, const double * x,
    const double * y, double * m)
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
                for (int i = 1; i < n - 1; i++) {
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
                m[0] = gp_tab_diff3(x[0], x[1], x[2], y[0], y[1], y[2]);
                m[n - 1] = gp_tab_diff3(x[n - 1], x[n - 2], x[n - 3],
                    y[n - 1], y[n - 2], y[n - 3]);
        }
}

/* CSn_dK: PCHIP slopes of each CSn column over the energy grid. */
__global__ void gp_kernel_tab_csn_dk(const gp_tables T, const double * csn,
    double * dk)
{
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= 4 * T.n_elements) return;
        const long o = (long)t * T.n_energies;
        gp_tab_pchip(T.n_energies, T.K, csn + o, dk + o);
}

/* DCS values of the table points: q = K exp(x_i) for the rows whose cross
 * section is positive. */
__global__ void gp_kernel_tab_dcs_points(const gp_tables T,
    const double * x, const double * csn, double * d)
{
        const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
        const int nE = T.n_energies, nx = T.n_table_dcs;
        const long n = 3L * T.n_elements * nE * nx;
        if (t >= n) return;
        const int i = (int)(t % nx);
        const long r = t / nx;
        const int row = (int)(r % nE);
        const int iel = (int)((r / nE) % T.n_elements);
        const int process = (int)(r / ((long)nE * T.n_elements));
        if (csn[r] <= 0.) {
                d[t] = 0.;
                return;
        }
        const double K = T.K[row];
        const double q = K * gp_exp(x[i]);
        d[t] = gp_dcs_process(T, process, T.element[iel], K, q);
}

/* One row of the DCS table (dcs_tabulate_row, pumas.c:11358-11438): the
 * logarithms of the positive DCS values, their PCHIP slopes in x and the
 * envelope exponent, from the slope at a quarter of the kinematic range. */
__global__ void gp_kernel_tab_dcs_rows(const gp_tables T, const double * x,
    const double * csn, const double * d, double * work, float * table,
    float * alpha)
{
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        const int nE = T.n_energies, n = T.n_table_dcs;
        if (t >= 3 * T.n_elements * nE) return;
        const int row = t % nE;
        const int iel = (t / nE) % T.n_elements;
        const int process = t / (nE * T.n_elements);
        float * data = table + (long)t * 2 * n;
        if (csn[t] <= 0.) {
                for (int i = 0; i < 2 * n; i++) data[i] = 0.f;
                alpha[t] = 0.f;
                return;
        }
        const double K = T.K[row];
        const gp_element & el = T.element[iel];
        const double * dt = d + (long)t * n;
        double * y = work + (long)t * 2 * n;
        double * m = y + n;
        int imin = n, imax = n - 1;
        for (int i = 0; i < n; i++) {
                if (dt[i] > 0) {
                        if (i < imin) imin = i;
                        y[i] = gp_log(dt[i]);
                } else if (imin < n) {
                        imax = i - 1;
                        break;
                }
        }
        if (imin <= imax)
                gp_tab_pchip(imax - imin + 1, x + imin, y + imin, m + imin);

        /* Kinematic filter of the envelope (pumas.c:11396-11412). */
        double qmin, qmax;
        if (process == 2) {
                gp_photonuclear_range(T.mass, K, qmin, qmax);
                qmin += qmin;
        } else {
                qmin = 4. * GP_ELECTRON_MASS;
                qmax = K + T.mass * el.qmax_m_pair;
                if (process == 0)
                        qmin = 0.5 * T.cutoff * K;
                else
                        qmin *= 4;
        }
        const double qrev = 0.6 * K;
        qmax *= 0.5;
        if (qmax > qrev) qmax = qrev;
        const double xmin = gp_log(qmin / K), xmax = gp_log(qmax / K);
        int ia0 = imax, ia1 = imin;
        for (int i = 0; i < n; i++) {
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
                alpha[t] = (float)a;
        } else {
                alpha[t] = 0.f;
        }
}

/* Envelope exponent of the low energy rows: the first positive one of the
 * column (compute_dcs_table, pumas.c:11683-11699). */
__global__ void gp_kernel_tab_alpha_low(const gp_tables T, float * alpha)
{
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= 3 * T.n_elements) return;
        float * a = alpha + (long)t * T.n_energies;
        int n0 = 0;
        float a0 = 0.f;
        for (int row = 0; row < T.n_energies; row++) {
                if (a[row] > 0.f) {
                        n0 = row;
                        a0 = a[row];
                        break;
                }
        }
        for (int row = 0; row < n0; row++) a[row] = a0;
}

/* The DCS sampling grid in x = ln(q / K) (compute_dcs_table,
 * pumas.c:11643-11672), in double precision, on the host. */
static void gp_tab_grid(int n, double cutoff, double * x)
{
        const int p = 20;        /* DCS_MODEL_N_REVERSE */
        const int m = n - p;
        double xrev;
        if (m > 0) {
                xrev = 0.6;      /* DCS_MODEL_X_REVERSE */
                const double x0 = log(cutoff);
                const double dx = log(xrev / cutoff) / (m - 1);
                for (int i = 0; i < m; i++) x[i] = x0 + i * dx;
        } else {
                xrev = cutoff;
        }
        const double dxmin = 1E-03;  /* DCS_MODEL_DXMIN */
        const double dx = log((0.95 - xrev) / dxmin) / ((m > 0) ? p : p - 1);
        for (int i = 0; i < p; i++)
                x[n - 1 - i] = log(0.95 - dxmin * exp(i * dx));
}

extern "C" int gp_api_physics_tabulate(const struct gpumas_physics * physics,
    double * csn, double * csn_dk, float * dcs, float * alpha, float * ms)
{
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        if ((csn == NULL) || (csn_dk == NULL) || (dcs == NULL) ||
            (alpha == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        const gp_tables & T = physics->tables;
        const int nE = T.n_energies, nel = T.n_elements, nx = T.n_table_dcs;
        const size_t n_pts = 3 * (size_t)nel * nE * GP_TAB_NINT;
        const size_t n_csn = 4 * (size_t)nel * nE;
        const size_t n_rows = 3 * (size_t)nel * nE;
        const size_t n_dpt = n_rows * nx;
        double * hx = (double *)malloc(nx * sizeof(double));
        if (hx == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
        gp_tab_grid(nx, T.cutoff, hx);

        /* Device work space: points, cross sections and slopes, grid, DCS
         * points and row work, outputs. */
        const size_t bytes = (n_pts + 2 * n_csn + nx + n_dpt + 2 * n_dpt) *
            sizeof(double) + (2 * n_dpt + n_rows) * sizeof(float);
        char * base = NULL;
        int rc = gp_check(cudaMalloc(&base, bytes));
        if (rc != GPUMAS_RETURN_SUCCESS) {
                free(hx);
                return rc;
        }
        double * d_pts = (double *)base;
        double * d_csn = d_pts + n_pts;
        double * d_dk = d_csn + n_csn;
        double * d_x = d_dk + n_csn;
        double * d_d = d_x + nx;
        double * d_work = d_d + n_dpt;
        float * d_table = (float *)(d_work + 2 * n_dpt);
        float * d_alpha = d_table + 2 * n_dpt;
        cudaEvent_t e0 = NULL, e1 = NULL;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        rc = gp_check(cudaMemcpy(d_x, hx, nx * sizeof(double),
            cudaMemcpyHostToDevice));
        free(hx);
        const int b = 128;
        if (rc == GPUMAS_RETURN_SUCCESS) {
                cudaEventRecord(e0, 0);
                gp_kernel_tab_points<<<(unsigned int)((n_pts + b - 1) / b),
                    b>>>(T, d_pts);
                gp_kernel_tab_csn<<<(unsigned int)((n_csn + b - 1) / b), b>>>(
                    T, d_pts, d_csn);
                gp_kernel_tab_csn_dk<<<(4 * nel + b - 1) / b, b>>>(
                    T, d_csn, d_dk);
                gp_kernel_tab_dcs_points<<<(unsigned int)((n_dpt + b - 1) /
                    b), b>>>(T, d_x, d_csn, d_d);
                gp_kernel_tab_dcs_rows<<<(unsigned int)((n_rows + b - 1) / b),
                    b>>>(T, d_x, d_csn, d_d, d_work, d_table, d_alpha);
                gp_kernel_tab_alpha_low<<<(3 * nel + b - 1) / b, b>>>(
                    T, d_alpha);
                cudaEventRecord(e1, 0);
                rc = gp_check(cudaGetLastError());
        }
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpy(csn, d_csn, n_csn * sizeof(double),
                    cudaMemcpyDeviceToHost));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpy(csn_dk, d_dk, n_csn * sizeof(double),
                    cudaMemcpyDeviceToHost));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpy(dcs, d_table,
                    2 * n_dpt * sizeof(float), cudaMemcpyDeviceToHost));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpy(alpha, d_alpha,
                    n_rows * sizeof(float), cudaMemcpyDeviceToHost));
        if ((rc == GPUMAS_RETURN_SUCCESS) && (ms != NULL))
                cudaEventElapsedTime(ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(base);
        return rc;
}

/*
 * gp_batch.cu -- the slot pool engine: stepping regrouped by step kind.
 *
 * The reference transports one event per call, in a loop over steps
 * (transport_with_stepping, pumas.c:5194-5514) whose iterations differ
 * widely in cost: a continuous step, a discrete energy loss (DEL) with its
 * rejection sampling and polar angle, a hard elastic scatter (EHS) with its
 * Coulomb setup, a boundary crossing. Running one event per GPU thread from
 * start to end makes a warp wait on its slowest lane at every such branch.
 *
 * This engine keeps a pool of P event slots in device memory (structure of
 * arrays, sized to stay resident in L2) and advances all of them one
 * iteration at a time with one kernel per step kind:
 *
 *   1. gp_pool_step: every slot makes its continuous step(s). Empty slots are
 *      first refilled from the input (a device work queue: an atomic cursor
 *      over the events). Slots whose step ended on a DEL or an EHS are
 *      appended to the DEL or EHS list with warp aggregated atomics (a
 *      ballot and prefix count per warp), so that the lists are compact.
 *   2. gp_pool_del: one thread per listed DEL, full warps.
 *   3. gp_pool_ehs: one thread per listed EHS, full warps.
 *
 * Finished events are written back to the caller's arrays at their input
 * index and their slot is refilled at the next iteration. Per event results
 * are identical to the one thread per event kernel: the random stream of an
 * event depends only on (seed, event id), and an event's draws are consumed
 * in the same order whichever slot, warp or kernel executes them.
 *
 * The host runs the iterations in batches captured in a CUDA graph and reads
 * two counters (input cursor, active slots) after each batch to stop.
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "gp_context.h"
#include "gp_io.cuh"

namespace cg = cooperative_groups;

/* Minimum resident blocks per SM of the pool kernels (register budget). */
#ifndef GP_POOL_MIN_BLOCKS
#define GP_POOL_MIN_BLOCKS 1
#endif

/* Field layout of a slot: doubles, ints and 64 bit integers, each as an
 * array of P values. */
enum gp_slot_double {
        SD_CHARGE, SD_ENERGY, SD_DISTANCE, SD_GRAMMAGE, SD_TIME, SD_WEIGHT,
        SD_POS0, SD_POS1, SD_POS2, SD_DIR0, SD_DIR1, SD_DIR2,
        SD_STEP_X_LIMIT, SD_STEP_INVLB1, SD_RANDN_NEXT, SD_LIFETIME, SD_RNEXT,
        SD_DENSITY, SD_TI, SD_WI, SD_XI, SD_XF, SD_DEI, SD_GRAMMAGE_MAX,
        SD_STEP_MAX_MEDIUM, SD_POLAR_KI, SD_POLAR_KF, SD_N
};
enum gp_slot_int {
        SI_DECAYED, SI_STEP_FIRST, SI_STEP_EVENT, SI_STEP_FORESEEN,
        SI_RANDN_DONE, SI_STEPS, SI_STATUS, SI_MEDIUM, SI_MATERIAL,
        SI_STRAIGHT, SI_STEP_INDEX, SI_NEW_MEDIUM, SI_PHASE, SI_MEDIUM_IN,
        SI_N_DRAWS, SI_POLAR_PROCESS, SI_POLAR_TARGET, SI_N
};
enum gp_slot_u64 { SU_ID, SU_SRC, SU_N };

#define GP_EMPTY 0

struct gp_pool {
        double * d;
        int * i;
        uint64_t * u;
        int P;
};

struct gp_counters {
        unsigned long long cursor;
        int active;
        int pad;
        int n_del[2];
        int n_ehs[2];
        int n_polar[2];
        int polar_next[2];
        int step_next[2];
};

/* Per call launch parameters, read by the kernels from device memory so
 * that one instantiated graph serves every call. */
struct gp_launch {
        gp_config cfg;
        gp_io io;
        size_t n;
        uint64_t first_event;
        int max_inner;
};

struct gp_pool_state {
        gp_pool pool;
        gp_counters * d_counters;
        gp_counters * h_counters;
        int * del_list[2];
        int * ehs_list[2];
        int * polar_list[2];
        void * d_mem;
        size_t capacity;
        gp_launch * d_launch;
        gp_launch * h_launch;
        cudaGraph_t graph;
        cudaGraphExec_t exec;
        int graph_batch;
        const void * graph_tables;
        const void * graph_geometry;
        unsigned int step_grid;
};

#define PD(f) pool.d[(size_t)(f) * pool.P + slot]
#define PI(f) pool.i[(size_t)(f) * pool.P + slot]
#define PU(f) pool.u[(size_t)(f) * pool.P + slot]

__device__ __forceinline__ void gp_slot_load(const gp_pool & pool, int slot,
    const gp_config & cfg, gp_event & e, gp_loop & L)
{
        e.charge = PD(SD_CHARGE);
        e.energy = PD(SD_ENERGY);
        e.distance = PD(SD_DISTANCE);
        e.grammage = PD(SD_GRAMMAGE);
        e.time = PD(SD_TIME);
        e.weight = PD(SD_WEIGHT);
        e.pos[0] = PD(SD_POS0);
        e.pos[1] = PD(SD_POS1);
        e.pos[2] = PD(SD_POS2);
        e.dir[0] = PD(SD_DIR0);
        e.dir[1] = PD(SD_DIR1);
        e.dir[2] = PD(SD_DIR2);
        e.step_X_limit = PD(SD_STEP_X_LIMIT);
        e.step_invlb1 = PD(SD_STEP_INVLB1);
        e.randn_next = PD(SD_RANDN_NEXT);
        e.lifetime = PD(SD_LIFETIME);
        e.rnext = PD(SD_RNEXT);
        e.decayed = PI(SI_DECAYED);
        e.step_first = PI(SI_STEP_FIRST);
        e.step_event = PI(SI_STEP_EVENT);
        e.step_foreseen = PI(SI_STEP_FORESEEN);
        e.randn_done = PI(SI_RANDN_DONE);
        e.steps = PI(SI_STEPS);
        e.status = PI(SI_STATUS);
        e.n = (uint32_t)PI(SI_N_DRAWS);
        e.id = PU(SU_ID);
        e.k0 = (uint32_t)cfg.seed;
        e.k1 = (uint32_t)(cfg.seed >> 32);
        L.density = PD(SD_DENSITY);
        L.ti = PD(SD_TI);
        L.wi = PD(SD_WI);
        L.Xi = PD(SD_XI);
        L.Xf = PD(SD_XF);
        L.dei = PD(SD_DEI);
        L.grammage_max = PD(SD_GRAMMAGE_MAX);
        L.step_max_medium = PD(SD_STEP_MAX_MEDIUM);
        L.medium = PI(SI_MEDIUM);
        L.material = PI(SI_MATERIAL);
        L.straight = PI(SI_STRAIGHT);
        L.step_index = PI(SI_STEP_INDEX);
        L.new_medium = PI(SI_NEW_MEDIUM);
}

__device__ __forceinline__ void gp_slot_store(const gp_pool & pool, int slot,
    const gp_event & e, const gp_loop & L)
{
        PD(SD_CHARGE) = e.charge;
        PD(SD_ENERGY) = e.energy;
        PD(SD_DISTANCE) = e.distance;
        PD(SD_GRAMMAGE) = e.grammage;
        PD(SD_TIME) = e.time;
        PD(SD_WEIGHT) = e.weight;
        PD(SD_POS0) = e.pos[0];
        PD(SD_POS1) = e.pos[1];
        PD(SD_POS2) = e.pos[2];
        PD(SD_DIR0) = e.dir[0];
        PD(SD_DIR1) = e.dir[1];
        PD(SD_DIR2) = e.dir[2];
        PD(SD_STEP_X_LIMIT) = e.step_X_limit;
        PD(SD_STEP_INVLB1) = e.step_invlb1;
        PD(SD_RANDN_NEXT) = e.randn_next;
        PD(SD_LIFETIME) = e.lifetime;
        PD(SD_RNEXT) = e.rnext;
        PI(SI_DECAYED) = e.decayed;
        PI(SI_STEP_FIRST) = e.step_first;
        PI(SI_STEP_EVENT) = e.step_event;
        PI(SI_STEP_FORESEEN) = e.step_foreseen;
        PI(SI_RANDN_DONE) = e.randn_done;
        PI(SI_STEPS) = e.steps;
        PI(SI_STATUS) = e.status;
        PI(SI_N_DRAWS) = (int)e.n;
        PU(SU_ID) = e.id;
        PD(SD_DENSITY) = L.density;
        PD(SD_TI) = L.ti;
        PD(SD_WI) = L.wi;
        PD(SD_XI) = L.Xi;
        PD(SD_XF) = L.Xf;
        PD(SD_DEI) = L.dei;
        PD(SD_GRAMMAGE_MAX) = L.grammage_max;
        PD(SD_STEP_MAX_MEDIUM) = L.step_max_medium;
        PI(SI_MEDIUM) = L.medium;
        PI(SI_MATERIAL) = L.material;
        PI(SI_STRAIGHT) = L.straight;
        PI(SI_STEP_INDEX) = L.step_index;
        PI(SI_NEW_MEDIUM) = L.new_medium;
}

/* Append `slot` to a compact list with one atomic per warp. */
__device__ __forceinline__ void gp_append(int * count, int * list, int slot)
{
        cg::coalesced_group g = cg::coalesced_threads();
        int base = 0;
        if (g.thread_rank() == 0) base = atomicAdd(count, (int)g.size());
        base = g.shfl(base, 0);
        list[base + g.thread_rank()] = slot;
}

/* Finish an event: write its state and results back at its input index
 * and free the slot. */
__device__ __forceinline__ void gp_finish(const gp_pool & pool, int slot,
    const gp_config & cfg, const gp_io & io, gp_counters * cnt, gp_event & e,
    int event, int medium_out)
{
        gp_stepping_end(cfg, e);
        io.store((size_t)PU(SU_SRC), e, event, PI(SI_MEDIUM_IN), medium_out);
        PI(SI_PHASE) = GP_EMPTY;
        atomicSub(&cnt->active, 1);
}

/* Route a slot to its next phase. */
__device__ __forceinline__ void gp_route(const gp_pool & pool, int slot,
    const gp_config & cfg, const gp_io & io, gp_counters * cnt,
    int * del_list, int * ehs_list, int parity, int next, gp_event & e,
    gp_loop & L, int event)
{
        if (next == GP_NEXT_DONE) {
                gp_finish(pool, slot, cfg, io, cnt, e, event, L.medium);
                return;
        }
        gp_slot_store(pool, slot, e, L);
        PI(SI_PHASE) = next;
        if (next == GP_NEXT_DEL)
                gp_append(&cnt->n_del[parity], del_list, slot);
        else if (next == GP_NEXT_EHS)
                gp_append(&cnt->n_ehs[parity], ehs_list, slot);
}

/* Refill slot `slot` from the input queue. Events that end before their
 * first step are finished here and the next one is taken. Returns 1 if the
 * slot now holds an event to step (e, L loaded), 0 if the input is empty. */
static __device__ __forceinline__ int gp_refill(const gp_tables & T,
    const gp_config & cfg, const gpumas_geometry & g, const gp_io & io,
    size_t n, uint64_t first_event, const gp_pool & pool, int slot,
    gp_counters * cnt, gp_event & e, gp_loop & L)
{
        for (;;) {
                if (*(volatile unsigned long long *)&cnt->cursor >= n)
                        return 0;
                cg::coalesced_group w = cg::coalesced_threads();
                unsigned long long base = 0;
                if (w.thread_rank() == 0)
                        base = atomicAdd(&cnt->cursor,
                            (unsigned long long)w.size());
                base = w.shfl(base, 0);
                const unsigned long long idx = base + w.thread_rank();
                if (idx >= n) return 0;
                io.load((size_t)idx, e);
                gp_event_init(e, cfg.seed, first_event + idx);
                int medium_in, event = GPUMAS_EVENT_NONE;
                const int next = gp_transport_begin(
                    T, cfg, g, e, L, event, medium_in);
                if (next == GP_NEXT_DONE) {
                        io.store((size_t)idx, e, event, medium_in, L.medium);
                        continue;
                }
                PU(SU_SRC) = idx;
                PI(SI_MEDIUM_IN) = medium_in;
                atomicAdd(&cnt->active, 1);
                return 1;
        }
}

/* Continuous steps. The kernel is persistent: each lane takes slots from a
 * cursor over the pool (refilling empty ones from the input), steps its
 * slot until the step ends on an event or after max_inner steps, routes it
 * to the next phase and takes the next slot. All lanes thus execute the step
 * together until the pool is exhausted, whatever the number of steps of
 * each event. */
__global__ void __launch_bounds__(128, GP_POOL_MIN_BLOCKS) gp_pool_step(
    const gp_tables * __restrict__ Tp, const gpumas_geometry * __restrict__ gp,
    const gp_launch * __restrict__ X, const gp_pool pool, gp_counters * cnt,
    int * del_list, int * ehs_list, int parity)
{
        const gp_config & cfg = X->cfg;
        const gp_io & io = X->io;
        const size_t n = X->n;
        const uint64_t first_event = X->first_event;
        const int max_inner = X->max_inner;
        const gp_tables & T = *Tp;
        const gpumas_geometry & g = *gp;
        int * scursor = &cnt->step_next[parity];
        gp_event e;
        gp_loop L;
        int slot = -1, k = 0, exhausted = 0;
        for (long guard = 0; guard < (1L << 40); guard++) {
                while ((slot < 0) && !exhausted) {
                        cg::coalesced_group w = cg::coalesced_threads();
                        int base = 0;
                        if (w.thread_rank() == 0)
                                base = atomicAdd(scursor, (int)w.size());
                        base = w.shfl(base, 0);
                        const int j = base + (int)w.thread_rank();
                        if (j >= pool.P) {
                                exhausted = 1;
                                break;
                        }
                        if (j == 0) {
                                /* The other parity's lists and cursors were
                                 * consumed by the previous iteration's
                                 * kernels, which precede this one. */
                                cnt->n_del[parity ^ 1] = 0;
                                cnt->n_ehs[parity ^ 1] = 0;
                                cnt->n_polar[parity ^ 1] = 0;
                                cnt->polar_next[parity ^ 1] = 0;
                                cnt->step_next[parity ^ 1] = 0;
                        }
                        const int s_ = j;
                        {
                                const int slot = s_;
                                if (PI(SI_PHASE) == GP_EMPTY) {
                                        if (!gp_refill(T, cfg, g, io, n,
                                                first_event, pool, slot, cnt,
                                                e, L))
                                                continue;
                                } else {
                                        gp_slot_load(pool, slot, cfg, e, L);
                                }
                        }
                        slot = s_;
                        k = 0;
                }
                if (!__any_sync(0xFFFFFFFFu, slot >= 0)) break;
                if (slot >= 0) {
                        int event = GPUMAS_EVENT_NONE;
                        const int next =
                            gp_stepping_step(T, cfg, g, e, L, event);
                        k++;
                        if ((next != GP_NEXT_STEP) || (k >= max_inner)) {
                                gp_route(pool, slot, cfg, io, cnt, del_list,
                                    ehs_list, parity, next, e, L, event);
                                slot = -1;
                        }
                }
        }
}

/* DELs: energy loss and, except for photonuclear events, polar angle.
 * Photonuclear polar angles (a Brent maximisation of the DDCS followed by a
 * rejection sampling, pumas.c:11874-11950) cost far more than the others
 * and are deferred to the polar list, so that they run in full warps. */
__global__ void __launch_bounds__(128, GP_POOL_MIN_BLOCKS) gp_pool_del(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, const int * __restrict__ list,
    int * polar_list, int parity)
{
        const gp_config & cfg = X->cfg;
        const gp_io & io = X->io;
        const int count = cnt->n_del[parity];
        const gp_tables & T = *Tp;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count;
             j += gridDim.x * blockDim.x) {
                const int slot = list[j];
                gp_event e;
                gp_loop L;
                gp_slot_load(pool, slot, cfg, e, L);
                int event = GPUMAS_EVENT_NONE;
                gp_polar_job job;
                gp_do_del_energy(T, cfg, e, L.material, job);
                if (job.process == 2) {
                        gp_slot_store(pool, slot, e, L);
                        PD(SD_POLAR_KI) = job.ki;
                        PD(SD_POLAR_KF) = job.kf;
                        PI(SI_POLAR_PROCESS) = job.process;
                        PI(SI_POLAR_TARGET) = job.target;
                        PI(SI_PHASE) = GP_NEXT_DEL;
                        gp_append(&cnt->n_polar[parity], polar_list, slot);
                        continue;
                }
                gp_do_del_polar(T, e, job);
                const int next = gp_stepping_del_end(T, cfg, e, L, event);
                if (next == GP_NEXT_DONE) {
                        gp_finish(pool, slot, cfg, io, cnt, e, event,
                            L.medium);
                } else {
                        gp_slot_store(pool, slot, e, L);
                        PI(SI_PHASE) = GP_NEXT_STEP;
                }
        }
}

/* ------------------------------------------------------------------------ */
/* Photonuclear polar angles in lockstep.                                   */
/*                                                                          */
/* polar_photonuclear (pumas.c:11874-11950) maximises Q2 d2S/dqdQ2 over     */
/* ln Q2 with math_find_minimum (pumas.c:12105-12206; bisection, then       */
/* Brent, pumas.c:12233-12325), possibly twice, then samples Q2 by          */
/* rejection. Every step of it costs one evaluation of the DRSS DDCS, and   */
/* the number of steps differs from event to event. Here each lane runs     */
/* its own copy of that procedure as a state machine whose every iteration  */
/* needs exactly one DDCS evaluation, done by all lanes together; a lane    */
/* whose event is done takes the next event of the list. The arithmetic and */
/* the random draws of each event are those of the sequential procedure.    */
/* ------------------------------------------------------------------------ */
enum gp_pn_phase {
        PN_MIN_A, PN_MIN_C, PN_BISECT, PN_BRENT, PN_REJECT, PN_DONE
};

struct gp_pn {
        /* Event. */
        double ki, q, Q2min, lnQ2max, rQ2;
        int target;
        /* Search state (math_find_minimum and math_find_minimum_brent). */
        int phase, second, i, ib, max_b;
        double xa, xc, fa, fc, xb, fb, atol;
        double x, w, v, fx, fw, fv, d, e, tolb;
        double u;
        /* First search result and the maximum of the objective. */
        double xopt, fopt;
        /* Pending evaluation: Q2 and kind (0: objective, 1: rejection). */
        double Q2;
        double mu;
};

#define PN_TOL 1E-06
#define PN_MAX_ITER 100

/* Start a find_minimum search over [xa, xc]. */
static __device__ __forceinline__ void gp_pn_search(gp_pn & s, double xa,
    double xc, int second)
{
        s.xa = xa;
        s.xc = xc;
        s.second = second;
        s.phase = PN_MIN_A;
}

/* End of a search with (xopt, fopt, status): continue as in
 * polar_photonuclear. */
static __device__ __forceinline__ void gp_pn_searched(
    gp_pn & s, gp_event & e, double xo, double fo, int status)
{
        const double M = 0.5 * (GP_PROTON_MASS + GP_NEUTRON_MASS);
        if (!s.second) {
                s.xopt = xo;
                s.fopt = -fo;
                if (status == -2) {
                        s.mu = 0.;
                        s.phase = PN_DONE;
                        return;
                }
                const double x = exp(s.xopt) / (2 * s.q * M);
                const double lne = 0.1;
                if ((x <= 0.04) && (s.xopt + lne < s.lnQ2max)) {
                        gp_pn_search(s, s.xopt + lne, s.lnQ2max, 1);
                        return;
                }
        } else if (status >= 0) {
                const double f2 = -fo;
                if (f2 > s.fopt) {
                        s.xopt = xo;
                        s.fopt = f2;
                }
        }
        s.i = 0;
        s.phase = PN_REJECT;
}

/* Advance the state machine up to its next DDCS evaluation (s.Q2), or to
 * its end (PN_DONE). `f` is the objective value of the last requested
 * point, if any. */
static __device__ __forceinline__ void gp_pn_advance(const gp_tables & T,
    gp_pn & s, gp_event & e, int have_value, double value)
{
        const double EPS = 1E-15;
        const double GOLD = 0.3819660;
        for (int guard = 0; guard < 64; guard++) {
                switch (s.phase) {
                case PN_MIN_A:
                        if (!have_value) {
                                s.Q2 = exp(s.xa);
                                return;
                        }
                        s.fa = value;
                        have_value = 0;
                        s.phase = PN_MIN_C;
                        break;
                case PN_MIN_C:
                        if (!have_value) {
                                s.Q2 = exp(s.xc);
                                return;
                        }
                        s.fc = value;
                        have_value = 0;
                        s.atol = PN_TOL * fabs(s.xc - s.xa);
                        s.i = 0;
                        s.phase = PN_BISECT;
                        break;
                case PN_BISECT:
                        if (!have_value) {
                                if (s.i == PN_MAX_ITER) {
                                        if (s.fa < s.fb) {
                                                s.fb = s.fa;
                                                s.xb = s.xa;
                                        } else if (s.fc < s.fb) {
                                                s.fb = s.fc;
                                                s.xb = s.xc;
                                        }
                                        gp_pn_searched(s, e, s.xb, s.fb, -1);
                                        break;
                                }
                                s.xb = 0.5 * (s.xa + s.xc);
                                s.Q2 = exp(s.xb);
                                return;
                        }
                        s.fb = value;
                        have_value = 0;
                        if ((s.fb < s.fa) && (s.fb < s.fc)) {
                                /* Brent refinement, math_find_minimum_brent
                                 * with bracket (xa, xb) as in the reference. */
                                s.max_b = PN_MAX_ITER - s.i;
                                s.tolb = PN_TOL * fabs(s.xc - s.xa);
                                s.x = s.w = s.v = s.xb;
                                s.fw = s.fv = s.fx = s.fb;
                                s.d = s.e = 0.;
                                s.ib = 0;
                                s.phase = PN_BRENT;
                                break;
                        }
                        if (fabs(s.xc - s.xa) <= s.atol) {
                                gp_pn_searched(s, e, s.xb, s.fb, s.i);
                                break;
                        }
                        if (s.fb < s.fc) {
                                s.xc = s.xb;
                                s.fc = s.fb;
                        } else {
                                s.xa = s.xb;
                                s.fa = s.fb;
                        }
                        s.i++;
                        break;
                case PN_BRENT:
                        if (!have_value) {
                                if (s.ib >= s.max_b) {
                                        gp_pn_searched(s, e, s.x, s.fx, -2);
                                        break;
                                }
                                const double xm = 0.5 * (s.xa + s.xb);
                                const double tol1 = s.tolb * fabs(s.x) + EPS;
                                const double tol2 = 2 * tol1;
                                if (fabs(s.x - xm) <=
                                    (tol2 - 0.5 * (s.xb - s.xa))) {
                                        gp_pn_searched(s, e, s.x, s.fx,
                                            s.ib + s.i);
                                        break;
                                }
                                if (fabs(s.e) > tol1) {
                                        const double r = (s.x - s.w) *
                                            (s.fx - s.fv);
                                        double qq = (s.x - s.v) * (s.fx - s.fw);
                                        double p = (s.x - s.v) * qq -
                                            (s.x - s.w) * r;
                                        qq = 2. * (qq - r);
                                        if (qq > 0.) p = -p;
                                        qq = fabs(qq);
                                        const double etemp = s.e;
                                        s.e = s.d;
                                        if (fabs(p) >= fabs(0.5 * qq * etemp) ||
                                            (p <= qq * (s.xa - s.x)) ||
                                            (p >= qq * (s.xb - s.x))) {
                                                s.e = (s.x >= xm) ? s.xa - s.x :
                                                                    s.xb - s.x;
                                                s.d = GOLD * s.e;
                                        } else {
                                                s.d = p / qq;
                                                const double uu = s.x + s.d;
                                                if ((uu - s.xa < tol2) ||
                                                    (s.xb - uu < tol2))
                                                        s.d = ((xm - s.x) >= 0.0) ?
                                                            fabs(tol1) :
                                                            -fabs(tol1);
                                        }
                                } else {
                                        s.e = (s.x >= xm) ? s.xa - s.x :
                                                            s.xb - s.x;
                                        s.d = GOLD * s.e;
                                }
                                s.u = (fabs(s.d) >= tol1) ? s.x + s.d :
                                    s.x + ((s.d >= 0.0) ? fabs(tol1) :
                                                          -fabs(tol1));
                                s.Q2 = exp(s.u);
                                return;
                        }
                        {
                                const double fu = value;
                                const double uu = s.u;
                                have_value = 0;
                                if (fu <= s.fx) {
                                        if (uu >= s.x)
                                                s.xa = s.x;
                                        else
                                                s.xb = s.x;
                                        s.v = s.w, s.w = s.x, s.x = uu;
                                        s.fv = s.fw, s.fw = s.fx, s.fx = fu;
                                } else {
                                        if (uu < s.x)
                                                s.xa = uu;
                                        else
                                                s.xb = uu;
                                        if ((fu <= s.fw) || (s.w == s.x)) {
                                                s.v = s.w;
                                                s.w = uu;
                                                s.fv = s.fw;
                                                s.fw = fu;
                                        } else if ((fu <= s.fv) ||
                                            (s.v == s.x) || (s.v == s.w)) {
                                                s.v = uu;
                                                s.fv = fu;
                                        }
                                }
                                s.ib++;
                        }
                        break;
                case PN_REJECT:
                        if (!have_value) {
                                if (s.i == 100) {
                                        s.mu = 0.;
                                        s.phase = PN_DONE;
                                        return;
                                }
                                const double uu = gp_random(e);
                                s.Q2 = s.Q2min * exp(s.rQ2 * uu);
                                return;
                        }
                        if (gp_random(e) * s.fopt <= value) {
                                /* Accepted: polar parameter of Q2. */
                                const double ml = T.mass;
                                const double ki = s.ki, q = s.q;
                                const double E = ki + ml;
                                const double p = sqrt(ki * (ki + 2 * ml));
                                const double E1 = E - q;
                                const double eps = ml / E1;
                                const double p1 = E1 * sqrt((1. + eps) *
                                                         (1. - eps));
                                const double p2 = p * p1;
                                double tmp = GP_SUB(GP_ADD(p2, GP_MUL(ml, ml)),
                                    GP_MUL(E, E1));
                                if (fabs(tmp) <= 3 * GP_DBL_EPSILON * p2)
                                        tmp = 0.;
                                const double a_mu = 0.5 * tmp / p2;
                                const double b_mu = 0.25 / p2;
                                double mu = a_mu + b_mu * s.Q2;
                                if (mu < 0)
                                        mu = 0.;
                                else if (mu > 1.)
                                        mu = 1.;
                                s.mu = mu;
                                s.phase = PN_DONE;
                                return;
                        }
                        have_value = 0;
                        s.i++;
                        break;
                default:
                        return;
                }
        }
}

/* Set up the polar sampling of a photonuclear DEL (ki >= kf). Returns
 * with PN_DONE when no sampling is needed. */
static __device__ __forceinline__ void gp_pn_start(const gp_tables & T,
    gp_pn & s, gp_event & e, double ki, double kf, int target)
{
        const double M = 0.5 * (GP_PROTON_MASS + GP_NEUTRON_MASS);
        s.ki = ki;
        s.q = ki - kf;
        s.target = target;
        const double ml = T.mass;
        const double E = ki + ml;
        const double ml2 = ml * ml;
        const double q = s.q;
        const double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
        const double Q2max =
            2.0 * M * (q - GP_PION_MASS) - GP_PION_MASS * GP_PION_MASS;
        s.mu = 0.;
        if ((Q2max < Q2min) | (Q2min < 0)) {
                s.phase = PN_DONE;
                return;
        }
        s.Q2min = Q2min;
        const double lnQ2min = log(Q2min);
        s.lnQ2max = log(Q2max);
        s.rQ2 = s.lnQ2max - lnQ2min;
        gp_pn_search(s, lnQ2min, s.lnQ2max, 0);
        gp_pn_advance(T, s, e, 0, 0.);
}

/* The objective or rejection value at the pending point. */
static __device__ __forceinline__ double gp_pn_value(
    const gp_tables & T, const gp_pn & s)
{
        const gp_element & el = T.element[s.target];
        const double d2 = gp_photonuclear_d2(T, el, s.ki, s.q, s.Q2);
        return (s.phase == PN_REJECT) ? d2 * s.Q2 : -d2 * s.Q2;
}

/* Deferred photonuclear polar angles: lanes refill from the list. */
__global__ void __launch_bounds__(128, GP_POOL_MIN_BLOCKS) gp_pool_polar(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, const int * __restrict__ list,
    int parity)
{
        const gp_config & cfg = X->cfg;
        const gp_io & io = X->io;
        const int count = cnt->n_polar[parity];
        const gp_tables & T = *Tp;
        int * cursor = &cnt->polar_next[parity];
        gp_event e;
        gp_loop L;
        gp_pn s;
        int slot = -1;
        for (int guard = 0; guard < (1 << 30); guard++) {
                if (slot < 0) {
                        /* Take events until one needs a sampling. */
                        while (true) {
                                const int j = atomicAdd(cursor, 1);
                                if (j >= count) break;
                                slot = list[j];
                                gp_slot_load(pool, slot, cfg, e, L);
                                gp_pn_start(T, s, e, PD(SD_POLAR_KI),
                                    PD(SD_POLAR_KF), PI(SI_POLAR_TARGET));
                                if (s.phase != PN_DONE) break;
                                gp_rotate(e, s.mu);
                                int event = GPUMAS_EVENT_NONE;
                                const int next = gp_stepping_del_end(
                                    T, cfg, e, L, event);
                                if (next == GP_NEXT_DONE) {
                                        gp_finish(pool, slot, cfg, io, cnt, e,
                                            event, L.medium);
                                } else {
                                        gp_slot_store(pool, slot, e, L);
                                        PI(SI_PHASE) = GP_NEXT_STEP;
                                }
                                slot = -1;
                        }
                }
                if (!__any_sync(0xFFFFFFFFu, slot >= 0)) break;
                if (slot >= 0) {
                        const double value = gp_pn_value(T, s);
                        gp_pn_advance(T, s, e, 1, value);
                        if (s.phase == PN_DONE) {
                                gp_rotate(e, s.mu);
                                int event = GPUMAS_EVENT_NONE;
                                const int next = gp_stepping_del_end(
                                    T, cfg, e, L, event);
                                if (next == GP_NEXT_DONE) {
                                        gp_finish(pool, slot, cfg, io, cnt, e,
                                            event, L.medium);
                                } else {
                                        gp_slot_store(pool, slot, e, L);
                                        PI(SI_PHASE) = GP_NEXT_STEP;
                                }
                                slot = -1;
                        }
                }
        }
}

__global__ void __launch_bounds__(128, GP_POOL_MIN_BLOCKS) gp_pool_ehs(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, const int * __restrict__ list,
    int parity)
{
        const gp_config & cfg = X->cfg;
        const gp_io & io = X->io;
        const int count = cnt->n_ehs[parity];
        const gp_tables & T = *Tp;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count;
             j += gridDim.x * blockDim.x) {
                const int slot = list[j];
                gp_event e;
                gp_loop L;
                gp_slot_load(pool, slot, cfg, e, L);
                int event = GPUMAS_EVENT_NONE;
                const int next = gp_stepping_ehs(T, cfg, e, L, event);
                if (next == GP_NEXT_DONE) {
                        gp_finish(pool, slot, cfg, io, cnt, e, event,
                            L.medium);
                } else {
                        gp_slot_store(pool, slot, e, L);
                        PI(SI_PHASE) = GP_NEXT_STEP;
                }
        }
}

/* ------------------------------------------------------------------------ */
/* Host driver.                                                             */
/* ------------------------------------------------------------------------ */
extern "C" void gp_pool_free(struct gp_pool_state * ps)
{
        if (ps == NULL) return;
        if (ps->exec != NULL) cudaGraphExecDestroy(ps->exec);
        if (ps->graph != NULL) cudaGraphDestroy(ps->graph);
        if (ps->d_mem != NULL) cudaFree(ps->d_mem);
        if (ps->h_counters != NULL) cudaFreeHost(ps->h_counters);
        if (ps->h_launch != NULL) cudaFreeHost(ps->h_launch);
        free(ps);
}

static int gp_pool_alloc(gp_context * c, int P)
{
        gp_pool_state * ps = c->pool;
        if ((ps != NULL) && (ps->capacity == (size_t)P)) return 0;
        gp_pool_free(ps);
        c->pool = NULL;
        ps = (gp_pool_state *)calloc(1, sizeof(*ps));
        if (ps == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
        const size_t sd = (size_t)SD_N * P * sizeof(double);
        const size_t si = (size_t)SI_N * P * sizeof(int);
        const size_t su = (size_t)SU_N * P * sizeof(uint64_t);
        const size_t sl = (size_t)P * sizeof(int);
        const size_t total = sd + si + su + 6 * sl + 256 + sizeof(gp_launch);
        int rc = gp_check(cudaMalloc(&ps->d_mem, total));
        if (rc == 0)
                rc = gp_check(cudaMallocHost(
                    (void **)&ps->h_counters, sizeof(gp_counters)));
        if (rc == 0)
                rc = gp_check(cudaMallocHost(
                    (void **)&ps->h_launch, sizeof(gp_launch)));
        if (rc != 0) {
                gp_pool_free(ps);
                return rc;
        }
        char * p = (char *)ps->d_mem;
        ps->pool.d = (double *)p;
        ps->pool.u = (uint64_t *)(p + sd);
        ps->pool.i = (int *)(p + sd + su);
        ps->del_list[0] = (int *)(p + sd + su + si);
        ps->del_list[1] = ps->del_list[0] + P;
        ps->ehs_list[0] = ps->del_list[1] + P;
        ps->ehs_list[1] = ps->ehs_list[0] + P;
        ps->polar_list[0] = ps->ehs_list[1] + P;
        ps->polar_list[1] = ps->polar_list[0] + P;
        ps->d_counters = (gp_counters *)(ps->polar_list[1] + P);
        ps->d_launch = (gp_launch *)((char *)ps->d_counters + 256);
        ps->pool.P = P;
        ps->capacity = P;
        {
                /* One wave of persistent step blocks. */
                int device = 0, sms = 0, per_sm = 0;
                cudaGetDevice(&device);
                cudaDeviceGetAttribute(
                    &sms, cudaDevAttrMultiProcessorCount, device);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, gp_pool_step, 128, 0);
                ps->step_grid = (unsigned int)(sms * (per_sm > 0 ? per_sm : 1));
        }
        c->pool = ps;
        return 0;
}

static void gp_iteration(gp_context * c, int parity, int block,
    cudaStream_t s)
{
        gp_pool_state * ps = c->pool;
        const int P = ps->pool.P;
        const unsigned int grid = (P + block - 1) / block;
        const unsigned int grid_step =
            (ps->step_grid > 0) && (ps->step_grid < grid) ? ps->step_grid :
                                                             grid;
        gp_pool_step<<<grid_step, block, 0, s>>>(c->d_tables, c->d_geometry,
            ps->d_launch, ps->pool, ps->d_counters, ps->del_list[parity],
            ps->ehs_list[parity], parity);
        const unsigned int grid2 = (grid + 3) / 4;
        gp_pool_del<<<grid2, block, 0, s>>>(c->d_tables, ps->d_launch,
            ps->pool, ps->d_counters, ps->del_list[parity],
            ps->polar_list[parity], parity);
        gp_pool_polar<<<grid2, block, 0, s>>>(c->d_tables, ps->d_launch,
            ps->pool, ps->d_counters, ps->polar_list[parity], parity);
        gp_pool_ehs<<<grid2, block, 0, s>>>(c->d_tables, ps->d_launch,
            ps->pool, ps->d_counters, ps->ehs_list[parity], parity);
}

/* Transport n events of `io` with the slot pool. Returns the number of
 * kernel launches in *launches. */
extern "C" int gp_pool_transport(gp_context * c, const gp_config * cfg_,
    const gp_io * io_, size_t n, uint64_t first, cudaStream_t s,
    const gp_tuning * tuning, int * launches)
{
        const gp_config cfg = *cfg_;
        const gp_io io = *io_;
        int P = tuning->pool_slots;
        if ((size_t)P > n) P = (int)((n + 127) / 128 * 128);
        if (P < 128) P = 128;
        int rc = gp_pool_alloc(c, P);
        if (rc != 0) return rc;
        gp_pool_state * ps = c->pool;
        const int block = 128;
        const int batch = (tuning->batch > 0) ? tuning->batch : 16;
        const int inner = (tuning->max_inner > 0) ? tuning->max_inner : 1;

        rc = gp_check(cudaMemsetAsync(ps->pool.i + (size_t)SI_PHASE * P, 0,
            (size_t)P * sizeof(int), s));
        if (rc == 0)
                rc = gp_check(cudaMemsetAsync(
                    ps->d_counters, 0, sizeof(gp_counters), s));
        if (rc != 0) return rc;

        /* Launch parameters of this call. */
        ps->h_launch->cfg = cfg;
        ps->h_launch->io = io;
        ps->h_launch->n = n;
        ps->h_launch->first_event = first;
        ps->h_launch->max_inner = inner;
        rc = gp_check(cudaMemcpyAsync(ps->d_launch, ps->h_launch,
            sizeof(gp_launch), cudaMemcpyHostToDevice, s));
        if (rc != 0) return rc;

        /* A batch of iterations as a CUDA graph (an even number, for the
         * list parity), rebuilt only when the pool or the context changes. */
        const int iters = 2 * ((batch + 1) / 2);
        const int same = (ps->exec != NULL) && (ps->graph_batch == iters) &&
            (ps->graph_tables == c->d_tables) &&
            (ps->graph_geometry == c->d_geometry);
        if (!same) {
                if (ps->exec != NULL) cudaGraphExecDestroy(ps->exec);
                if (ps->graph != NULL) cudaGraphDestroy(ps->graph);
                ps->exec = NULL;
                ps->graph = NULL;
                cudaStream_t cap;
                rc = gp_check(cudaStreamCreateWithFlags(
                    &cap, cudaStreamNonBlocking));
                if (rc != 0) return rc;
                rc = gp_check(cudaStreamBeginCapture(
                    cap, cudaStreamCaptureModeThreadLocal));
                if (rc == 0) {
                        for (int k = 0; k < iters; k++)
                                gp_iteration(c, k & 1, block, cap);
                        rc = gp_check(cudaStreamEndCapture(cap, &ps->graph));
                }
                if (rc == 0)
                        rc = gp_check(cudaGraphInstantiate(
                            &ps->exec, ps->graph, 0));
                cudaStreamDestroy(cap);
                if (rc != 0) return rc;
                ps->graph_batch = iters;
                ps->graph_tables = c->d_tables;
                ps->graph_geometry = c->d_geometry;
        }
        int n_launch = 0;
        for (long it = 0;; it++) {
                rc = gp_check(cudaGraphLaunch(ps->exec, s));
                if (rc != 0) return rc;
                n_launch += 4 * iters;
                rc = gp_check(cudaMemcpyAsync(ps->h_counters, ps->d_counters,
                    sizeof(gp_counters), cudaMemcpyDeviceToHost, s));
                if (rc == 0) rc = gp_check(cudaStreamSynchronize(s));
                if (rc != 0) return rc;
                if ((ps->h_counters->cursor >= n) &&
                    (ps->h_counters->active == 0))
                        break;
                if (it > (1L << 40)) return GPUMAS_RETURN_INTERNAL_ERROR;
        }
        if (launches != NULL) *launches = n_launch;
        return 0;
}

/* ------------------------------------------------------------------------ */
/* Allocation free transport.                                               */
/*                                                                          */
/* Some callers cannot allocate device memory while they transport: a host  */
/* program whose allocator owns all of the GPU memory and hands out fixed   */
/* arenas, a plugin embedded in a framework that forbids allocation on its  */
/* hot path, or code that must not pay (or fail on) a cudaMalloc in the     */
/* middle of a run. For them the slot pool of the pool engine also exists   */
/* as one static device array, reserved when the library is loaded on a     */
/* device and kept until the process exits.                                 */
/* ------------------------------------------------------------------------ */

/* Largest pool of the allocation free entry point, in event slots
 * (GPUMAS_STATIC_SLOTS of gpumas.h). */
#define GP_STATIC_SLOTS GPUMAS_STATIC_SLOTS

/* Bytes of the static pool: slot fields, the DEL / EHS lists of both
 * parities, the counters and the launch descriptor. */
#define GP_STATIC_BYTES                                                       \
        ((size_t)GP_STATIC_SLOTS *                                            \
                (SD_N * sizeof(double) + SU_N * sizeof(uint64_t) +            \
                    SI_N * sizeof(int) + 6 * sizeof(int)) +                   \
            512 + sizeof(gp_launch))

static __device__ __align__(256) unsigned char gp_static_pool[GP_STATIC_BYTES];

/* Device address of gp_static_pool on each device, found once per device
 * with that device current (a host side use of the symbol itself is not a
 * device address). */
#define GP_STATIC_DEVICES 64
static void * gp_static_address[GP_STATIC_DEVICES];

static int gp_static_setup(int device, void ** address)
{
        if ((device < 0) || (device >= GP_STATIC_DEVICES))
                return GPUMAS_RETURN_DEVICE_ERROR;
        if (gp_static_address[device] == NULL) {
                void * ptr = NULL;
                if (cudaGetSymbolAddress(&ptr, gp_static_pool) != cudaSuccess)
                        return GPUMAS_RETURN_DEVICE_ERROR;
                gp_static_address[device] = ptr;
        }
        *address = gp_static_address[device];
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_config_check(const struct gpumas_context * context,
    const struct gpumas_physics * physics, gp_config * cfg);

extern "C" int gpumas_context_transport_device_static(
    struct gpumas_context * context, size_t n,
    const struct gpumas_soa * events, uint64_t first_event, int pool_slots,
    void * stream)
{
        if ((context == NULL) || (events == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        if (pool_slots == 0) pool_slots = GP_STATIC_SLOTS;
        if ((pool_slots < 128) || (pool_slots > GP_STATIC_SLOTS) ||
            (pool_slots % 128 != 0))
                return GPUMAS_RETURN_VALUE_ERROR;
        gp_context * c = (gp_context *)context;
        if (!c->has_geometry) return GPUMAS_RETURN_MEDIUM_ERROR;
        gp_config cfg;
        int rc = gp_config_check(context, c->physics, &cfg);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        if (n == 0) return GPUMAS_RETURN_SUCCESS;

        int device = 0;
        if (cudaGetDevice(&device) != cudaSuccess)
                return GPUMAS_RETURN_DEVICE_ERROR;
        void * base = NULL;
        rc = gp_static_setup(device, &base);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;

        /* Carve the static array: the layout of the pool engine for P
         * slots, followed by the counters and the launch descriptor. */
        const int P = pool_slots;
        char * p = (char *)base;
        gp_pool pool;
        pool.d = (double *)p;
        p += (size_t)SD_N * P * sizeof(double);
        pool.u = (uint64_t *)p;
        p += (size_t)SU_N * P * sizeof(uint64_t);
        pool.i = (int *)p;
        p += (size_t)SI_N * P * sizeof(int);
        int * lists = (int *)p;
        p += (size_t)6 * P * sizeof(int);
        p = (char *)(((size_t)p + 255) & ~(size_t)255);
        gp_counters * counters = (gp_counters *)p;
        gp_launch * launch = (gp_launch *)(p + 256);
        pool.P = P;

        cudaStream_t s = (cudaStream_t)stream;
        /* The array keeps the previous call's contents: empty every slot
         * and zero the counters and list lengths. */
        rc = gp_check(cudaMemsetAsync(pool.i + (size_t)SI_PHASE * P, 0,
            (size_t)P * sizeof(int), s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemsetAsync(counters, 0,
                    sizeof(gp_counters), s));
        gp_launch h;
        memset(&h, 0, sizeof(h));
        h.cfg = cfg;
        memset(&h.io, 0, sizeof(h.io));
        h.io.soa.a = *events;
        h.n = n;
        h.first_event = first_event;
        h.max_inner = (c->tuning.max_inner > 0) ? c->tuning.max_inner : 1;
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpyAsync(launch, &h, sizeof(h),
                    cudaMemcpyHostToDevice, s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaStreamSynchronize(s));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;

        const int block = 128;
        const unsigned int grid = (P + block - 1) / block;
        const unsigned int grid2 = (grid + 3) / 4;
        unsigned int grid_step = grid;
        {
                int sms = 0, per_sm = 0;
                cudaDeviceGetAttribute(
                    &sms, cudaDevAttrMultiProcessorCount, device);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    &per_sm, gp_pool_step, block, 0);
                const unsigned int wave =
                    (unsigned int)(sms * (per_sm > 0 ? per_sm : 1));
                if (wave < grid_step) grid_step = wave;
        }
        const int batch = 16;
        for (long it = 0;; it++) {
                for (int k = 0; k < batch; k++) {
                        const int parity = k & 1;
                        int * del_list = lists + (size_t)parity * P;
                        int * ehs_list = lists + (size_t)(2 + parity) * P;
                        int * polar_list = lists + (size_t)(4 + parity) * P;
                        gp_pool_step<<<grid_step, block, 0, s>>>(
                            c->d_tables, c->d_geometry, launch, pool,
                            counters, del_list, ehs_list, parity);
                        gp_pool_del<<<grid2, block, 0, s>>>(c->d_tables,
                            launch, pool, counters, del_list, polar_list,
                            parity);
                        gp_pool_polar<<<grid2, block, 0, s>>>(c->d_tables,
                            launch, pool, counters, polar_list, parity);
                        gp_pool_ehs<<<grid2, block, 0, s>>>(c->d_tables,
                            launch, pool, counters, ehs_list, parity);
                }
                rc = gp_check(cudaGetLastError());
                gp_counters hc;
                if (rc == GPUMAS_RETURN_SUCCESS)
                        rc = gp_check(cudaMemcpyAsync(&hc, counters,
                            sizeof(hc), cudaMemcpyDeviceToHost, s));
                if (rc == GPUMAS_RETURN_SUCCESS)
                        rc = gp_check(cudaStreamSynchronize(s));
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                if ((hc.cursor >= n) && (hc.active == 0)) break;
                if (it > (1L << 40)) return GPUMAS_RETURN_INTERNAL_ERROR;
        }
        return GPUMAS_RETURN_SUCCESS;
}

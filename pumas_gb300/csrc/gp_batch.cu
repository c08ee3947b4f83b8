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
 * arrays) and advances all of them one iteration at a time with one kernel
 * per step kind:
 *
 *   0. gp_pool_drain: clears the consumed lists and, once the queue is
 *      empty and few slots remain active, runs their events to the end in
 *      one launch (otherwise it returns at once).
 *   1. gp_pool_fill: slot turnover. Events that ended in the last step
 *      kernel are written back to the caller's arrays at their input index;
 *      empty slots are refilled from the input (a device work queue: an
 *      atomic cursor over the events of every job).
 *   2. gp_pool_step: every slot in the step phase makes its continuous
 *      step(s). Slots whose step ended on a DEL or an EHS are appended to
 *      the DEL or EHS list with warp aggregated atomics (a ballot and prefix
 *      count per warp), so that the lists are compact.
 *   3. gp_pool_del: one thread per listed DEL, full warps; photonuclear
 *      polar angles are deferred to
 *   4. gp_pool_polar: Brent search and rejection in lockstep, with refill,
 *      on a second graph stream beside the next kernels;
 *   5. gp_pool_ehs: one thread per listed EHS, full warps.
 *
 * Each kernel is built twice (template <int LOC>): without the code of the
 * media's local properties, and with it for jobs whose geometry has them.
 * Per event results are identical to the one thread per event kernel: the
 * random stream of an event depends only on (seed, event id), and an
 * event's draws are consumed in the same order whichever slot, warp or
 * kernel executes them.
 *
 * The host runs the iterations in batches captured in a CUDA graph and reads
 * the counters (input cursor, active slots, completed jobs) after each
 * batch to stop or to report completions.
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
/* The step kernel runs as one persistent wave: 4 blocks of 128 threads per
 * SM, i.e. at most 128 registers per thread. */
#ifndef GP_STEP_MIN_BLOCKS
#define GP_STEP_MIN_BLOCKS 4
#endif

/* Field layout of a slot: doubles, ints and 64 bit integers, each as an
 * array of P values. */
enum gp_slot_double {
        SD_CHARGE, SD_ENERGY, SD_DISTANCE, SD_GRAMMAGE, SD_TIME, SD_WEIGHT,
        SD_POS0, SD_POS1, SD_POS2, SD_DIR0, SD_DIR1, SD_DIR2,
        SD_STEP_X_LIMIT, SD_STEP_INVLB1, SD_RANDN_NEXT, SD_LIFETIME, SD_RNEXT,
        SD_DENSITY, SD_TI, SD_WI, SD_XI, SD_XF, SD_DEI, SD_GRAMMAGE_MAX,
        SD_STEP_MAX_MEDIUM, SD_POLAR_KI, SD_POLAR_KF, SD_LOC_MAG0,
        SD_LOC_MAG1, SD_LOC_MAG2, SD_LOC_DENSITY, SD_LOC_STEP_MAX, SD_N
};
enum gp_slot_int {
        SI_DECAYED, SI_STEP_FIRST, SI_STEP_EVENT, SI_STEP_FORESEEN,
        SI_RANDN_DONE, SI_STEPS, SI_STATUS, SI_MEDIUM, SI_MATERIAL,
        SI_STRAIGHT, SI_STEP_INDEX, SI_NEW_MEDIUM, SI_PHASE, SI_MEDIUM_IN,
        SI_N_DRAWS, SI_POLAR_PROCESS, SI_POLAR_TARGET, SI_JOB, SI_EVENT_END,
        SI_LOC_MAGNETIZED, SI_N
};
enum gp_slot_u64 { SU_ID, SU_SRC, SU_N };

#define GP_EMPTY 0
/* A slot whose event ended in the step kernel (GP_NEXT_DONE): its state
 * and end event wait in the slot for the fill kernel, which writes them back
 * to the job's output and frees the slot. */
/* Slots whose photonuclear polar angle was sampled beside the next
 * iteration (the polar kernel runs on its own graph stream into the next
 * iteration): back in the step phase (GP_POLAR_STEP) or emptied
 * (GP_POLAR_EMPTY), tagged with the parity p of the iteration that listed
 * them. The kernels of parity p, two iterations later and after the polar
 * kernel has joined, take them as GP_NEXT_STEP and GP_EMPTY; those of the
 * other parity, which can run while the polar kernel writes them, leave
 * them alone, as they leave the slots still listed (GP_NEXT_DEL). */
#define GP_POLAR_STEP(p) (5 + (p))
#define GP_POLAR_EMPTY(p) (7 + (p))

struct gp_pool {
        double * d;
        int * i;
        uint64_t * u;
        int P;
};

struct gp_counters {
        unsigned long long cursor;
        /* Slot visits routed so far (continuous step phases ended, and
         * events run to their end by the drain): a batch of iterations that
         * leaves it and the cursor unchanged while events remain is a
         * stall, which the host loops turn into an error. */
        unsigned long long progress;
        int active;
        int n_done;
        int n_del[2];
        int n_ehs[2];
        int n_polar[2];
        int polar_next[2];
        int step_next[2];
        int drain_next[2];
};

/* A job: events of one context (settings, geometry, random seed), read from
 * and written back to `io` at their index in the job. The job owns queue
 * positions [begin, begin + n) of the engine's event queue; event k of the
 * job uses the random stream of event id first_event + k. */
struct gp_job {
        gp_config cfg;
        const gpumas_geometry * geometry;
        gp_io io;
        unsigned long long begin;
        unsigned long long n;
        uint64_t first_event;
};

/* Per call launch parameters, read by the kernels from device memory so
 * that one instantiated graph serves every call: the job table (sorted by
 * queue position), per job counts of finished events, the list of jobs
 * completed so far and the end of the queue. */
struct gp_launch {
        const gp_job * jobs;
        unsigned long long * job_done;
        int * done_list;
        int n_jobs;
        int max_inner;
        unsigned long long total;
        /* Drain threshold: once the queue is exhausted and at most this many
         * slots are active, the step kernel runs each remaining event to its
         * end, DELs and EHSs included (0: never). */
        int tail_slots;
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

/* Local properties of the current medium (struct gp_loc) of a slot whose
 * job's geometry has locals (struct gpumas_locals): loaded into `loc`,
 * whose address is returned, or NULL for the other jobs. The kernels are
 * built twice: with LOC = 0 (no job with locals in the pool, the locals
 * code compiled out) and LOC = 1. */
template <int LOC>
__device__ __forceinline__ gp_loc * gp_loc_load(const gp_pool & pool,
    int slot, const gpumas_geometry * g, gp_loc & loc)
{
        if (!LOC || (g->locals == NULL)) return NULL;
        loc.g = g;
        loc.magnet[0] = PD(SD_LOC_MAG0);
        loc.magnet[1] = PD(SD_LOC_MAG1);
        loc.magnet[2] = PD(SD_LOC_MAG2);
        loc.density = PD(SD_LOC_DENSITY);
        loc.step_max = PD(SD_LOC_STEP_MAX);
        loc.magnetized = PI(SI_LOC_MAGNETIZED);
        return &loc;
}

__device__ __forceinline__ void gp_loc_store(const gp_pool & pool, int slot,
    const gp_loc * loc)
{
        if (loc == NULL) return;
        PD(SD_LOC_MAG0) = loc->magnet[0];
        PD(SD_LOC_MAG1) = loc->magnet[1];
        PD(SD_LOC_MAG2) = loc->magnet[2];
        PD(SD_LOC_DENSITY) = loc->density;
        PD(SD_LOC_STEP_MAX) = loc->step_max;
        PI(SI_LOC_MAGNETIZED) = loc->magnetized;
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

/* Count a finished event of job `job`; the event that completes the job
 * appends it to the list of completed jobs. */
__device__ __forceinline__ void gp_job_event_done(const gp_launch * X,
    gp_counters * cnt, int job)
{
        const unsigned long long k = atomicAdd(&X->job_done[job], 1ull) + 1;
        if (k == X->jobs[job].n) {
                const int pos = atomicAdd(&cnt->n_done, 1);
                X->done_list[pos] = job;
        }
}

/* Finish an event: write its state and results back at its index in its
 * job and free the slot (phase `empty`: GP_EMPTY, or GP_POLAR_EMPTY from
 * the polar kernel). */
__device__ __forceinline__ void gp_finish(const gp_pool & pool, int slot,
    const gp_launch * X, const gp_job & J, gp_counters * cnt, gp_event & e,
    int event, int medium_out, int empty = GP_EMPTY)
{
        gp_stepping_end(J.cfg, e);
        const int job = PI(SI_JOB);
        J.io.store((size_t)PU(SU_SRC), e, event, PI(SI_MEDIUM_IN),
            medium_out);
        PI(SI_PHASE) = empty;
        atomicSub(&cnt->active, 1);
        gp_job_event_done(X, cnt, job);
}

/* Count one unit of progress per calling lane, with one atomic per warp. */
__device__ __forceinline__ void gp_progress(gp_counters * cnt)
{
        cg::coalesced_group g = cg::coalesced_threads();
        if (g.thread_rank() == 0)
                atomicAdd(&cnt->progress, (unsigned long long)g.size());
}

/* Route a slot to its next phase; an ended event waits in its slot for the
 * fill kernel (GP_NEXT_DONE). */
__device__ __forceinline__ void gp_route(const gp_pool & pool, int slot,
    const gp_launch * X, const gp_job & J, gp_counters * cnt,
    int * del_list, int * ehs_list, int parity, int next, gp_event & e,
    gp_loop & L, int event)
{
        gp_progress(cnt);
        gp_slot_store(pool, slot, e, L);
        if (next == GP_NEXT_DONE) PI(SI_EVENT_END) = event;
        PI(SI_PHASE) = next;
        if (next == GP_NEXT_DEL)
                gp_append(&cnt->n_del[parity], del_list, slot);
        else if (next == GP_NEXT_EHS)
                gp_append(&cnt->n_ehs[parity], ehs_list, slot);
}

/* Job owning queue position idx: the last job whose first position is not
 * above idx (the table is sorted by position and positions between two
 * jobs are never handed out, see gp_engine_append). */
__device__ __forceinline__ int gp_job_of(const gp_launch * X,
    unsigned long long idx)
{
        int lo = 0, hi = X->n_jobs;
        while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (X->jobs[mid].begin <= idx)
                        lo = mid;
                else
                        hi = mid;
        }
        return lo;
}

/* Refill slot `slot` from the event queue. Events that end before their
 * first step are finished here and the next one is taken. Returns 1 if the
 * slot now holds an event to step (e, L loaded, *job set), 0 if the queue
 * is empty. */
template <int LOC>
static __device__ __forceinline__ int gp_refill(const gp_tables & T,
    const gp_launch * X, const gp_pool & pool, int slot, gp_counters * cnt,
    gp_event & e, gp_loop & L, int & job, gp_loc & loc, gp_loc *& lp)
{
        const unsigned long long total = X->total;
        for (;;) {
                if (*(volatile unsigned long long *)&cnt->cursor >= total)
                        return 0;
                cg::coalesced_group w = cg::coalesced_threads();
                unsigned long long base = 0;
                if (w.thread_rank() == 0)
                        base = atomicAdd(&cnt->cursor,
                            (unsigned long long)w.size());
                base = w.shfl(base, 0);
                const unsigned long long idx = base + w.thread_rank();
                if (idx >= total) return 0;
                job = gp_job_of(X, idx);
                const gp_job & J = X->jobs[job];
                const unsigned long long k = idx - J.begin;
                J.io.begin((size_t)k, J.cfg, J.first_event + k, e);
                int medium_in, event = GPUMAS_EVENT_NONE;
                lp = (LOC && (J.geometry->locals != NULL)) ? &loc : NULL;
                const int next = gp_transport_begin(
                    T, J.cfg, *J.geometry, e, L, event, medium_in, NULL, lp);
                if (next == GP_NEXT_DONE) {
                        J.io.store((size_t)k, e, event, medium_in, L.medium);
                        gp_job_event_done(X, cnt, job);
                        continue;
                }
                PU(SU_SRC) = k;
                PI(SI_MEDIUM_IN) = medium_in;
                PI(SI_JOB) = job;
                atomicAdd(&cnt->active, 1);
                return 1;
        }
}

/* First kernel of a pool iteration. Block 0 clears the other parity's DEL
 * and EHS lists and cursors, which the previous iteration's kernels (before
 * this one in stream order) have consumed, and this parity's polar list,
 * consumed by the polar kernel of two iterations before (joined before this
 * one).
 *
 * It also drains the pool: once no event is left in the queue and at most
 * tail_slots slots are active, regrouping by step kind would leave most
 * lanes idle for hundreds of short iterations. Each lane then takes active
 * slots and carries their events to the end, DELs and EHSs included (the
 * one thread per event scheme); an event's operations and draws are the
 * same either way. Otherwise the kernel returns at once. At the start of
 * an iteration an active slot is in the continuous step phase, ended
 * (GP_NEXT_DONE) or with the polar kernel of the previous iteration. */
template <int LOC>
__global__ void __launch_bounds__(128, 1) gp_pool_drain(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, int parity)
{
        if ((blockIdx.x == 0) && (threadIdx.x == 0)) {
                cnt->n_del[parity ^ 1] = 0;
                cnt->n_ehs[parity ^ 1] = 0;
                cnt->step_next[parity ^ 1] = 0;
                cnt->drain_next[parity ^ 1] = 0;
                cnt->n_polar[parity] = 0;
                cnt->polar_next[parity] = 0;
        }
        const int tail = (X->tail_slots > 0) && (cnt->cursor >= X->total) &&
            (cnt->active <= X->tail_slots);
        if (!tail) return;
        const gp_tables & T = *Tp;
        int * dcursor = &cnt->drain_next[parity];
        /* Each pass takes a new slot index: at most P + 1 passes. */
        for (long guard = 0; guard <= pool.P; guard++) {
                cg::coalesced_group w = cg::coalesced_threads();
                int base = 0;
                if (w.thread_rank() == 0)
                        base = atomicAdd(dcursor, (int)w.size());
                base = w.shfl(base, 0);
                const int slot = base + (int)w.thread_rank();
                if (slot >= pool.P) return;
                const int phase = PI(SI_PHASE);
                if ((phase != GP_NEXT_STEP) &&
                    (phase != GP_POLAR_STEP(parity)))
                        continue;
                const gp_job & J = X->jobs[PI(SI_JOB)];
                gp_event e;
                gp_loop L;
                gp_loc loc;
                gp_slot_load(pool, slot, J.cfg, e, L);
                gp_loc * lp = gp_loc_load<LOC>(pool, slot, J.geometry, loc);
                int event = GPUMAS_EVENT_NONE;
                int next = GP_NEXT_STEP;
                /* An event ends within GP_MAX_STEPS steps, each followed by
                 * at most one DEL and one EHS. */
                for (long s_ = 0; next != GP_NEXT_DONE; s_++) {
                        if (s_ > 3L * GP_MAX_STEPS) {
                                e.status = GPUMAS_RETURN_INTERNAL_ERROR;
                                break;
                        }
                        if (next == GP_NEXT_STEP)
                                next = gp_stepping_step(T, J.cfg,
                                    *J.geometry, e, L, event, NULL, lp);
                        else if (next == GP_NEXT_DEL)
                                next = gp_stepping_del(
                                    T, J.cfg, e, L, event, NULL, lp);
                        else
                                next = gp_stepping_ehs(
                                    T, J.cfg, e, L, event, lp);
                }
                gp_progress(cnt);
                gp_finish(pool, slot, X, J, cnt, e, event, L.medium);
        }
}

/* Slot turnover, one thread per slot: an event that ended in the previous
 * step kernel (GP_NEXT_DONE) is written back to its job's output and its
 * slot freed; an empty slot takes the next event of the queue
 * (gp_refill: events that end before their first step are written back at
 * once and the next one taken), which enters the step phase. */
template <int LOC>
__global__ void __launch_bounds__(128, 1) gp_pool_fill(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, int parity)
{
        const int slot = blockIdx.x * blockDim.x + threadIdx.x;
        if (slot >= pool.P) return;
        const gp_tables & T = *Tp;
        gp_event e;
        gp_loop L;
        int phase = PI(SI_PHASE);
        if (phase == GP_NEXT_DONE) {
                const gp_job & J = X->jobs[PI(SI_JOB)];
                gp_slot_load(pool, slot, J.cfg, e, L);
                gp_finish(pool, slot, X, J, cnt, e, PI(SI_EVENT_END),
                    L.medium);
                phase = GP_EMPTY;
        }
        if ((phase != GP_EMPTY) && (phase != GP_POLAR_EMPTY(parity))) return;
        int job;
        gp_loc loc, * lp = NULL;
        if (!gp_refill<LOC>(T, X, pool, slot, cnt, e, L, job, loc, lp))
                return;
        gp_slot_store(pool, slot, e, L);
        gp_loc_store(pool, slot, lp);
        PI(SI_PHASE) = GP_NEXT_STEP;
}

/* Continuous steps. The kernel is persistent: each lane takes slots from a
 * cursor over the pool, steps the slots in the step phase until the step
 * ends on an event or after max_inner steps, routes them to the next phase
 * and takes the next slot. All lanes thus execute the step together until
 * the pool is exhausted, whatever the number of steps of each event. Slots
 * are emptied and refilled by the fill kernel, which keeps the input and
 * output code out of this one. */
template <int LOC>
__global__ void __launch_bounds__(128, GP_STEP_MIN_BLOCKS) gp_pool_step(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, int * del_list, int * ehs_list,
    int parity)
{
        const gp_tables & T = *Tp;
        const int max_inner = X->max_inner;
        int * scursor = &cnt->step_next[parity];
        gp_event e;
        gp_loop L;
        gp_loc loc, * lp = NULL;
        const gp_job * J = X->jobs;
        int slot = -1, k = 0, exhausted = 0;
        /* Every pass steps each lane that holds a slot; a lane takes at
         * most P slots (distinct cursor positions), each for at most
         * max_inner steps. */
        const long passes = (long)pool.P * max_inner + 2;
        for (long guard = 0; guard < passes; guard++) {
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
                        {
                                const int slot = j;
                                const int phase = PI(SI_PHASE);
                                if ((phase != GP_NEXT_STEP) &&
                                    (phase != GP_POLAR_STEP(parity)))
                                        continue;
                                J = X->jobs + PI(SI_JOB);
                                gp_slot_load(pool, slot, J->cfg, e, L);
                                lp = gp_loc_load<LOC>(
                                    pool, slot, J->geometry, loc);
                        }
                        slot = j;
                        k = 0;
                }
                if (!__any_sync(0xFFFFFFFFu, slot >= 0)) break;
                if (slot >= 0) {
                        int event = GPUMAS_EVENT_NONE;
                        const int next = gp_stepping_step(T, J->cfg,
                            *J->geometry, e, L, event, NULL, lp);
                        k++;
                        if ((next != GP_NEXT_STEP) || (k >= max_inner)) {
                                gp_loc_store(pool, slot, lp);
                                gp_route(pool, slot, X, *J, cnt, del_list,
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
template <int LOC>
__global__ void __launch_bounds__(128, GP_POOL_MIN_BLOCKS) gp_pool_del(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, const int * __restrict__ list,
    int * polar_list, int parity)
{
        const int count = cnt->n_del[parity];
        const gp_tables & T = *Tp;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count;
             j += gridDim.x * blockDim.x) {
                const int slot = list[j];
                const gp_job & J = X->jobs[PI(SI_JOB)];
                const gp_config & cfg = J.cfg;
                gp_event e;
                gp_loop L;
                gp_slot_load(pool, slot, cfg, e, L);
                int event = GPUMAS_EVENT_NONE;
                gp_polar_job job;
                gp_stepping_weight(T, cfg, e, L);
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
                gp_loc loc;
                gp_loc * lp = gp_loc_load<LOC>(pool, slot, J.geometry, loc);
                const int next =
                    gp_stepping_del_end(T, cfg, e, L, event, lp);
                if (next == GP_NEXT_DONE) {
                        gp_finish(pool, slot, X, J, cnt, e, event, L.medium);
                } else {
                        gp_slot_store(pool, slot, e, L);
                        gp_loc_store(pool, slot, lp);
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
                const double x = gp_exp(s.xopt) / (2 * s.q * M);
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
                                s.Q2 = gp_exp(s.xa);
                                return;
                        }
                        s.fa = value;
                        have_value = 0;
                        s.phase = PN_MIN_C;
                        break;
                case PN_MIN_C:
                        if (!have_value) {
                                s.Q2 = gp_exp(s.xc);
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
                                s.Q2 = gp_exp(s.xb);
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
                                s.Q2 = gp_exp(s.u);
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
                                s.Q2 = s.Q2min * gp_exp(s.rQ2 * uu);
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
        const double lnQ2min = gp_log(Q2min);
        s.lnQ2max = gp_log(Q2max);
        s.rQ2 = s.lnQ2max - lnQ2min;
        gp_pn_search(s, lnQ2min, s.lnQ2max, 0);
        gp_pn_advance(T, s, e, 0, 0.);
}

/* The objective or rejection value at the pending point. */
static __device__ __forceinline__ double gp_pn_value(
    const gp_tables & T, const gp_pn & s)
{
        const gp_element & el = T.element[s.target];
        const double d2 = gp_photonuclear_ddcs(T, el, s.ki, s.q, s.Q2);
        return (s.phase == PN_REJECT) ? d2 * s.Q2 : -d2 * s.Q2;
}

/* Deferred photonuclear polar angles: lanes refill from the list. With
 * `side`, the kernel runs beside the next iteration and marks the slots it
 * releases with this iteration's parity (GP_POLAR_STEP, GP_POLAR_EMPTY). */
template <int LOC>
__global__ void __launch_bounds__(128, GP_POOL_MIN_BLOCKS) gp_pool_polar(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, const int * __restrict__ list,
    int parity, int side)
{
        const int count = cnt->n_polar[parity];
        const int step = side ? GP_POLAR_STEP(parity) : GP_NEXT_STEP;
        const int empty = side ? GP_POLAR_EMPTY(parity) : GP_EMPTY;
        const gp_tables & T = *Tp;
        int * cursor = &cnt->polar_next[parity];
        gp_event e;
        gp_loop L;
        gp_pn s;
        const gp_job * J = X->jobs;
        int slot = -1;
        /* A lane takes at most count events, each needing at most two
         * searches of 202 evaluations and 100 rejection trials. */
        const long passes = 1024L * (count + 1);
        for (long guard = 0; guard < passes; guard++) {
                if (slot < 0) {
                        /* Take events until one needs a sampling. */
                        while (true) {
                                const int j = atomicAdd(cursor, 1);
                                if (j >= count) break;
                                slot = list[j];
                                J = X->jobs + PI(SI_JOB);
                                gp_slot_load(pool, slot, J->cfg, e, L);
                                gp_pn_start(T, s, e, PD(SD_POLAR_KI),
                                    PD(SD_POLAR_KF), PI(SI_POLAR_TARGET));
                                if (s.phase != PN_DONE) break;
                                gp_rotate(e, s.mu);
                                int event = GPUMAS_EVENT_NONE;
                                gp_loc loc;
                                gp_loc * lp = gp_loc_load<LOC>(
                                    pool, slot, J->geometry, loc);
                                const int next = gp_stepping_del_end(
                                    T, J->cfg, e, L, event, lp);
                                if (next == GP_NEXT_DONE) {
                                        gp_finish(pool, slot, X, *J, cnt, e,
                                            event, L.medium, empty);
                                } else {
                                        gp_slot_store(pool, slot, e, L);
                                        gp_loc_store(pool, slot, lp);
                                        PI(SI_PHASE) = step;
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
                                gp_loc loc;
                                gp_loc * lp = gp_loc_load<LOC>(
                                    pool, slot, J->geometry, loc);
                                const int next = gp_stepping_del_end(
                                    T, J->cfg, e, L, event, lp);
                                if (next == GP_NEXT_DONE) {
                                        gp_finish(pool, slot, X, *J, cnt, e,
                                            event, L.medium, empty);
                                } else {
                                        gp_slot_store(pool, slot, e, L);
                                        gp_loc_store(pool, slot, lp);
                                        PI(SI_PHASE) = step;
                                }
                                slot = -1;
                        }
                }
        }
}

template <int LOC>
__global__ void __launch_bounds__(128, GP_POOL_MIN_BLOCKS) gp_pool_ehs(
    const gp_tables * __restrict__ Tp, const gp_launch * __restrict__ X,
    const gp_pool pool, gp_counters * cnt, const int * __restrict__ list,
    int parity)
{
        const int count = cnt->n_ehs[parity];
        const gp_tables & T = *Tp;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < count;
             j += gridDim.x * blockDim.x) {
                const int slot = list[j];
                const gp_job & J = X->jobs[PI(SI_JOB)];
                const gp_config & cfg = J.cfg;
                gp_event e;
                gp_loop L;
                gp_slot_load(pool, slot, cfg, e, L);
                gp_loc loc;
                gp_loc * lp = gp_loc_load<LOC>(pool, slot, J.geometry, loc);
                int event = GPUMAS_EVENT_NONE;
                const int next = gp_stepping_ehs(T, cfg, e, L, event, lp);
                if (next == GP_NEXT_DONE) {
                        gp_finish(pool, slot, X, J, cnt, e, event, L.medium);
                } else {
                        gp_slot_store(pool, slot, e, L);
                        gp_loc_store(pool, slot, lp);
                        PI(SI_PHASE) = GP_NEXT_STEP;
                }
        }
}

/* ------------------------------------------------------------------------ */
/* Pool layout and iterations (host side).                                  */
/* ------------------------------------------------------------------------ */

/* Round a byte count up to 256. */
static inline size_t gp_align256(size_t n) { return (n + 255) & ~(size_t)255; }

/* Bytes of a pool of P slots: slot fields, the six work lists (DEL, EHS and
 * photonuclear polar, two parities each), the counters and the launch
 * descriptor, each 256 byte aligned. */
static size_t gp_pool_bytes(int P)
{
        return gp_align256((size_t)SD_N * P * sizeof(double)) +
            gp_align256((size_t)SU_N * P * sizeof(uint64_t)) +
            gp_align256((size_t)SI_N * P * sizeof(int)) +
            gp_align256((size_t)6 * P * sizeof(int)) +
            gp_align256(sizeof(gp_counters)) + gp_align256(sizeof(gp_launch));
}

/* Device side view of a pool laid out over gp_pool_bytes(P) bytes. */
struct gp_pool_view {
        gp_pool pool;
        int * lists[6];
        gp_counters * counters;
        gp_launch * launch;
};

static void gp_pool_carve(char * base, int P, gp_pool_view * v)
{
        char * p = base;
        v->pool.P = P;
        v->pool.d = (double *)p;
        p += gp_align256((size_t)SD_N * P * sizeof(double));
        v->pool.u = (uint64_t *)p;
        p += gp_align256((size_t)SU_N * P * sizeof(uint64_t));
        v->pool.i = (int *)p;
        p += gp_align256((size_t)SI_N * P * sizeof(int));
        for (int k = 0; k < 6; k++) v->lists[k] = (int *)p + (size_t)k * P;
        p += gp_align256((size_t)6 * P * sizeof(int));
        v->counters = (gp_counters *)p;
        p += gp_align256(sizeof(gp_counters));
        v->launch = (gp_launch *)p;
}

/* One wave of persistent step blocks on the current device. */
static unsigned int gp_step_wave(int P, int block)
{
        int device = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &per_sm, gp_pool_step<0>, block, 0);
        const unsigned int wave =
            (unsigned int)(sms * (per_sm > 0 ? per_sm : 1));
        const unsigned int grid = (P + block - 1) / block;
        return (wave < grid) ? wave : grid;
}

/* Launch pool iteration k (list parity k & 1): list reset and drain, slot
 * turnover, continuous steps, DELs, hard elastic scatters and photonuclear
 * polar angles. Lists 0-1 are the DEL lists, 2-3 the EHS lists and 4-5 the
 * polar lists of both parities.
 *
 * With fork == NULL every kernel runs on s, one after the other. With a
 * fork, the polar kernel runs on a second stream from the end of the DEL
 * kernel on into the next iteration: each of its lanes carries one event's
 * chain of up to hundreds of DDCS evaluations, so it keeps few warps busy
 * for about a millisecond, which the EHS kernel and the next iteration's
 * step kernel now fill. Its slots (a few per thousand of the pool) sit out
 * the next step kernel; iteration k + 2 waits for it before it starts. */
struct gp_fork {
        cudaStream_t s2;
        cudaEvent_t del_done, polar_done[2];
};

template <int LOC>
static void gp_iteration(const gp_tables * d_tables, const gp_pool_view & v,
    unsigned int grid_step, int k, cudaStream_t s,
    const gp_fork * fork = NULL)
{
        const int block = 128;
        const int parity = k & 1;
        const int side = (fork != NULL);
        const unsigned int grid = (v.pool.P + block - 1) / block;
        const unsigned int grid2 = (grid + 3) / 4;
        int * del_list = v.lists[parity];
        int * ehs_list = v.lists[2 + parity];
        int * polar_list = v.lists[4 + parity];
        if (side && (k >= 2))
                cudaStreamWaitEvent(s, fork->polar_done[parity], 0);
        gp_pool_drain<LOC><<<grid_step, block, 0, s>>>(d_tables, v.launch,
            v.pool, v.counters, parity);
        gp_pool_fill<LOC><<<grid, block, 0, s>>>(d_tables, v.launch,
            v.pool, v.counters, parity);
        gp_pool_step<LOC><<<grid_step, block, 0, s>>>(d_tables, v.launch,
            v.pool, v.counters, del_list, ehs_list, parity);
        gp_pool_del<LOC><<<grid2, block, 0, s>>>(d_tables, v.launch,
            v.pool, v.counters, del_list, polar_list, parity);
        cudaStream_t sp = s;
        if (side) {
                cudaEventRecord(fork->del_done, s);
                cudaStreamWaitEvent(fork->s2, fork->del_done, 0);
                sp = fork->s2;
        }
        gp_pool_polar<LOC><<<grid2, block, 0, sp>>>(d_tables, v.launch,
            v.pool, v.counters, polar_list, parity, side);
        if (side) cudaEventRecord(fork->polar_done[parity], sp);
        gp_pool_ehs<LOC><<<grid2, block, 0, s>>>(d_tables, v.launch,
            v.pool, v.counters, ehs_list, parity);
}

/* Kernels per pool iteration, and the slot turnover that closes a batch of
 * iterations: the events that ended in its last step kernel are written
 * back before the host reads the counters. */
#define GP_KERNELS_PER_ITERATION 6

template <int LOC>
static void gp_batch_end(const gp_tables * d_tables, const gp_pool_view & v,
    cudaStream_t s, const gp_fork * fork = NULL)
{
        if (fork != NULL) {
                cudaStreamWaitEvent(s, fork->polar_done[0], 0);
                cudaStreamWaitEvent(s, fork->polar_done[1], 0);
        }
        const unsigned int grid = (v.pool.P + 127) / 128;
        gp_pool_fill<LOC><<<grid, 128, 0, s>>>(d_tables, v.launch, v.pool,
            v.counters, 0);
}

/* ------------------------------------------------------------------------ */
/* Engine: job table, state budget and graph batches.                       */
/* ------------------------------------------------------------------------ */

/* First fit allocator of the state budget (host side bookkeeping of one
 * device allocation), in units of 256 bytes. */
struct gp_arena {
        char * base;
        size_t size;
        size_t used;
        /* Free blocks (offset, size), sorted by offset. */
        size_t * off;
        size_t * len;
        int n, cap;
};

static int gp_arena_alloc(gp_arena * a, size_t size, size_t * offset)
{
        size = gp_align256(size);
        for (int k = 0; k < a->n; k++) {
                if (a->len[k] >= size) {
                        *offset = a->off[k];
                        a->off[k] += size;
                        a->len[k] -= size;
                        if (a->len[k] == 0) {
                                memmove(a->off + k, a->off + k + 1,
                                    (a->n - k - 1) * sizeof(size_t));
                                memmove(a->len + k, a->len + k + 1,
                                    (a->n - k - 1) * sizeof(size_t));
                                a->n--;
                        }
                        a->used += size;
                        return 1;
                }
        }
        return 0;
}

static int gp_arena_free(gp_arena * a, size_t offset, size_t size)
{
        size = gp_align256(size);
        int k = 0;
        while ((k < a->n) && (a->off[k] < offset)) k++;
        const int merge_prev = (k > 0) && (a->off[k - 1] + a->len[k - 1] ==
                                              offset);
        const int merge_next = (k < a->n) && (offset + size == a->off[k]);
        if (merge_prev && merge_next) {
                a->len[k - 1] += size + a->len[k];
                memmove(a->off + k, a->off + k + 1,
                    (a->n - k - 1) * sizeof(size_t));
                memmove(a->len + k, a->len + k + 1,
                    (a->n - k - 1) * sizeof(size_t));
                a->n--;
        } else if (merge_prev) {
                a->len[k - 1] += size;
        } else if (merge_next) {
                a->off[k] = offset;
                a->len[k] += size;
        } else {
                if (a->n == a->cap) {
                        const int cap = 2 * a->cap + 16;
                        size_t * off = (size_t *)realloc(
                            a->off, cap * sizeof(size_t));
                        if (off == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
                        a->off = off;
                        size_t * len = (size_t *)realloc(
                            a->len, cap * sizeof(size_t));
                        if (len == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
                        a->len = len;
                        a->cap = cap;
                }
                memmove(a->off + k + 1, a->off + k,
                    (a->n - k) * sizeof(size_t));
                memmove(a->len + k + 1, a->len + k,
                    (a->n - k) * sizeof(size_t));
                a->off[k] = offset;
                a->len[k] = size;
                a->n++;
        }
        a->used -= size;
        return GPUMAS_RETURN_SUCCESS;
}

/* Host side record of a job in flight. */
struct gp_job_host {
        int ticket;
        /* Jobs submitted from host memory: their records in the budget. */
        gpumas_state * states;
        gpumas_result * results;
        size_t offset, bytes;
        int in_arena;
};

struct gpumas_engine {
        const struct gpumas_physics * physics;
        gp_tables * d_tables;  /* owned unless borrowed from a context */
        int own_tables;
        gp_tuning tuning;
        cudaStream_t stream;
        int own_stream;
        /* Pool. */
        void * d_pool;
        int P;
        gp_pool_view view;
        unsigned int grid_step;
        /* Batch graphs of the kernels built without (0) and with (1) the
         * media's local properties; the second serves once a job with
         * locals joined the table, until the table is emptied. */
        cudaGraph_t graph[2];
        cudaGraphExec_t exec[2];
        int graph_iters[2];
        int locals;
        /* Jobs: device table, completion counts and list. */
        int capacity;
        gp_job * d_jobs;
        unsigned long long * d_job_done;
        int * d_done_list;
        gp_job * h_jobs;
        gp_job_host * h_info;
        int n_jobs;      /* jobs in the table */
        int n_uploaded;  /* jobs of the table already on the device */
        int n_reported;  /* entries of the completion list already read */
        int ticket0;     /* ticket of table entry 0 */
        int inflight;    /* jobs of the table not yet seen completed */
        unsigned long long total;  /* end of the event queue */
        int busy;        /* events queued or in slots */
        /* Tickets completed and not yet reported. */
        int * fifo;
        int fifo_head, fifo_n, fifo_cap;
        /* Pinned mirrors. */
        gp_counters * h_counters;
        gp_launch * h_launch;
        int * h_done;
        /* State budget. */
        gp_arena arena;
        /* Statistics. */
        cudaEvent_t t0, t1;
        struct gpumas_engine_stats stats;
        /* Progress seen after the last batch (stall detection). */
        unsigned long long seen_cursor, seen_progress;
};

/* Whether the counters moved since the last batch; records them. */
static int gp_moved(unsigned long long * cursor, unsigned long long * progress,
    const gp_counters & c)
{
        const int moved = (c.cursor != *cursor) || (c.progress != *progress);
        *cursor = c.cursor;
        *progress = c.progress;
        return moved;
}

static int gp_fifo_push(gpumas_engine * g, int ticket)
{
        if (g->fifo_n == g->fifo_cap) {
                const int cap = 2 * g->fifo_cap + 64;
                int * f = (int *)malloc(cap * sizeof(int));
                if (f == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
                for (int k = 0; k < g->fifo_n; k++)
                        f[k] = g->fifo[(g->fifo_head + k) % g->fifo_cap];
                free(g->fifo);
                g->fifo = f;
                g->fifo_head = 0;
                g->fifo_cap = cap;
        }
        g->fifo[(g->fifo_head + g->fifo_n) % g->fifo_cap] = ticket;
        g->fifo_n++;
        return GPUMAS_RETURN_SUCCESS;
}

/* (Re)allocate the pool for P slots; the graph is rebuilt. */
static int gp_engine_pool(gpumas_engine * g, int P)
{
        if ((g->d_pool != NULL) && (g->P == P)) return GPUMAS_RETURN_SUCCESS;
        for (int q = 0; q < 2; q++) {
                if (g->exec[q] != NULL) cudaGraphExecDestroy(g->exec[q]);
                if (g->graph[q] != NULL) cudaGraphDestroy(g->graph[q]);
                g->exec[q] = NULL;
                g->graph[q] = NULL;
        }
        if (g->d_pool != NULL) cudaFree(g->d_pool);
        g->d_pool = NULL;
        g->P = 0;
        int rc = gp_check(cudaMalloc(&g->d_pool, gp_pool_bytes(P)));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        g->P = P;
        gp_pool_carve((char *)g->d_pool, P, &g->view);
        if (g->h_counters != NULL) memset(g->h_counters, 0,
            sizeof(gp_counters));
        g->seen_cursor = g->seen_progress = 0;
        g->grid_step = gp_step_wave(P, 128);
        rc = gp_check(cudaMemsetAsync(g->view.pool.i + (size_t)SI_PHASE * P,
            0, (size_t)P * sizeof(int), g->stream));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemsetAsync(g->view.counters, 0,
                    sizeof(gp_counters), g->stream));
        return rc;
}

/* Capture `iters` iterations (an even number, for the list parity) as a
 * CUDA graph of the kernels without (loc = 0) or with the locals, once per
 * pool. */
static int gp_engine_graph(gpumas_engine * g, int loc)
{
        const int batch = (g->tuning.batch > 0) ? g->tuning.batch : 16;
        const int iters = 2 * ((batch + 1) / 2);
        if ((g->exec[loc] != NULL) && (g->graph_iters[loc] == iters))
                return GPUMAS_RETURN_SUCCESS;
        if (g->exec[loc] != NULL) cudaGraphExecDestroy(g->exec[loc]);
        if (g->graph[loc] != NULL) cudaGraphDestroy(g->graph[loc]);
        g->exec[loc] = NULL;
        g->graph[loc] = NULL;
        cudaStream_t cap;
        int rc = gp_check(cudaStreamCreateWithFlags(
            &cap, cudaStreamNonBlocking));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        gp_fork fork;
        memset(&fork, 0, sizeof(fork));
        cudaEvent_t * events[3] = { &fork.del_done, &fork.polar_done[0],
                &fork.polar_done[1] };
        rc = gp_check(cudaStreamCreateWithFlags(
            &fork.s2, cudaStreamNonBlocking));
        for (int q = 0; (q < 3) && (rc == GPUMAS_RETURN_SUCCESS); q++)
                rc = gp_check(cudaEventCreateWithFlags(
                    events[q], cudaEventDisableTiming));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaStreamBeginCapture(
                    cap, cudaStreamCaptureModeThreadLocal));
        if (rc == GPUMAS_RETURN_SUCCESS) {
                for (int k = 0; k < iters; k++) {
                        if (loc)
                                gp_iteration<1>(g->d_tables, g->view,
                                    g->grid_step, k, cap, &fork);
                        else
                                gp_iteration<0>(g->d_tables, g->view,
                                    g->grid_step, k, cap, &fork);
                }
                if (loc)
                        gp_batch_end<1>(g->d_tables, g->view, cap, &fork);
                else
                        gp_batch_end<0>(g->d_tables, g->view, cap, &fork);
                rc = gp_check(cudaStreamEndCapture(cap, &g->graph[loc]));
        }
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaGraphInstantiate(
                    &g->exec[loc], g->graph[loc], 0));
        for (int q = 0; q < 3; q++)
                if (*events[q] != NULL) cudaEventDestroy(*events[q]);
        if (fork.s2 != NULL) cudaStreamDestroy(fork.s2);
        cudaStreamDestroy(cap);
        if (rc == GPUMAS_RETURN_SUCCESS) g->graph_iters[loc] = iters;
        return rc;
}

static void gp_engine_free(gpumas_engine * g)
{
        for (int q = 0; q < 2; q++) {
                if (g->exec[q] != NULL) cudaGraphExecDestroy(g->exec[q]);
                if (g->graph[q] != NULL) cudaGraphDestroy(g->graph[q]);
        }
        if (g->d_pool != NULL) cudaFree(g->d_pool);
        if (g->d_jobs != NULL) cudaFree(g->d_jobs);
        if (g->own_tables && (g->d_tables != NULL)) cudaFree(g->d_tables);
        if (g->arena.base != NULL) cudaFree(g->arena.base);
        if (g->h_counters != NULL) cudaFreeHost(g->h_counters);
        if (g->h_launch != NULL) cudaFreeHost(g->h_launch);
        if (g->h_done != NULL) cudaFreeHost(g->h_done);
        if (g->own_stream && (g->stream != NULL))
                cudaStreamDestroy(g->stream);
        if (g->t0 != NULL) cudaEventDestroy(g->t0);
        if (g->t1 != NULL) cudaEventDestroy(g->t1);
        free(g->h_jobs);
        free(g->h_info);
        free(g->fifo);
        free(g->arena.off);
        free(g->arena.len);
        free(g);
}

/* Create an engine. `d_tables` may borrow an existing device copy of the
 * tables (the context path); `stream` may be NULL for an own stream. */
static int gp_engine_new(gpumas_engine ** out,
    const struct gpumas_physics * physics, gp_tables * d_tables,
    const gp_tuning * tuning, int max_jobs, size_t budget)
{
        *out = NULL;
        gpumas_engine * g = (gpumas_engine *)calloc(1, sizeof(*g));
        if (g == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
        g->physics = physics;
        g->tuning = *tuning;
        g->capacity = max_jobs;
        int rc = gp_check(cudaStreamCreateWithFlags(
            &g->stream, cudaStreamNonBlocking));
        g->own_stream = 1;
        if ((rc == GPUMAS_RETURN_SUCCESS) && (d_tables == NULL)) {
                gp_tables tables;
                gp_physics_tables(physics, &tables);
                rc = gp_check(cudaMalloc(&g->d_tables, sizeof(gp_tables)));
                g->own_tables = 1;
                if (rc == GPUMAS_RETURN_SUCCESS)
                        rc = gp_check(cudaMemcpy(g->d_tables, &tables,
                            sizeof(gp_tables), cudaMemcpyHostToDevice));
        } else {
                g->d_tables = d_tables;
        }
        /* Job table, completion counts and list in one allocation. */
        const size_t o_done = gp_align256((size_t)max_jobs * sizeof(gp_job));
        const size_t o_list = o_done + gp_align256(
            (size_t)max_jobs * sizeof(unsigned long long));
        const size_t jbytes = o_list + (size_t)max_jobs * sizeof(int);
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMalloc((void **)&g->d_jobs, jbytes));
        if (rc == GPUMAS_RETURN_SUCCESS) {
                g->d_job_done = (unsigned long long *)((char *)g->d_jobs +
                    o_done);
                g->d_done_list = (int *)((char *)g->d_jobs + o_list);
                g->h_jobs = (gp_job *)calloc(max_jobs, sizeof(gp_job));
                g->h_info = (gp_job_host *)calloc(
                    max_jobs, sizeof(gp_job_host));
                if ((g->h_jobs == NULL) || (g->h_info == NULL))
                        rc = GPUMAS_RETURN_MEMORY_ERROR;
        }
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMallocHost(
                    (void **)&g->h_counters, sizeof(gp_counters)));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMallocHost(
                    (void **)&g->h_launch, sizeof(gp_launch)));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMallocHost(
                    (void **)&g->h_done, (size_t)max_jobs * sizeof(int)));
        if ((rc == GPUMAS_RETURN_SUCCESS) && (budget > 0)) {
                budget = budget & ~(size_t)255;
                rc = gp_check(cudaMalloc((void **)&g->arena.base, budget));
                if (rc == GPUMAS_RETURN_SUCCESS) {
                        g->arena.size = budget;
                        g->arena.cap = 16;
                        g->arena.off = (size_t *)malloc(16 * sizeof(size_t));
                        g->arena.len = (size_t *)malloc(16 * sizeof(size_t));
                        if ((g->arena.off == NULL) || (g->arena.len == NULL))
                                rc = GPUMAS_RETURN_MEMORY_ERROR;
                        else {
                                g->arena.off[0] = 0;
                                g->arena.len[0] = budget;
                                g->arena.n = 1;
                        }
                }
        }
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaEventCreate(&g->t0));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaEventCreate(&g->t1));
        if (rc == GPUMAS_RETURN_SUCCESS) {
                const int P = (tuning->pool_slots > 0) ? tuning->pool_slots :
                                                         1048576;
                rc = gp_engine_pool(g, (P + 127) / 128 * 128);
        }
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaStreamSynchronize(g->stream));
        if (rc != GPUMAS_RETURN_SUCCESS) {
                gp_engine_free(g);
                return rc;
        }
        *out = g;
        return GPUMAS_RETURN_SUCCESS;
}

/* Start a new job table when nothing is in flight (queue positions,
 * completion counts and list restart at 0). */
static int gp_engine_restart(gpumas_engine * g)
{
        if ((g->inflight > 0) || g->busy || (g->n_jobs == 0))
                return GPUMAS_RETURN_SUCCESS;
        g->ticket0 += g->n_jobs;
        g->n_jobs = 0;
        g->locals = 0;
        g->n_uploaded = 0;
        g->n_reported = 0;
        g->total = 0;
        g->seen_cursor = g->seen_progress = 0;
        memset(g->h_counters, 0, sizeof(gp_counters));
        return gp_check(cudaMemsetAsync(
            g->view.counters, 0, sizeof(gp_counters), g->stream));
}

/* Append a job to the table. Queue positions handed out before (and
 * burned by lanes that found the queue empty) are skipped: the job starts
 * at the larger of the queue end and the cursor read after the last batch,
 * so that no lane can ever be given a position between two jobs. */
static int gp_engine_append(gpumas_engine * g, const gp_config & cfg,
    const gpumas_geometry * geometry, const gp_io & io, size_t n,
    uint64_t first_event, const gp_job_host & info, int * ticket,
    int locals = 0)
{
        if (locals) g->locals = 1;
        gp_job & J = g->h_jobs[g->n_jobs];
        memset(&J, 0, sizeof(J));
        J.cfg = cfg;
        J.geometry = geometry;
        J.io = io;
        unsigned long long begin = g->total;
        if (g->h_counters->cursor > begin) begin = g->h_counters->cursor;
        J.begin = begin;
        J.n = n;
        J.first_event = first_event;
        g->total = begin + n;
        g->h_info[g->n_jobs] = info;
        g->h_info[g->n_jobs].ticket = g->ticket0 + g->n_jobs;
        *ticket = g->ticket0 + g->n_jobs;
        g->n_jobs++;
        g->stats.events += (long long)n;
        if (n == 0) {
                /* Never seen by the device: completed now. */
                return gp_fifo_push(g, *ticket);
        }
        g->inflight++;
        g->busy = 1;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_config_check(const struct gpumas_context * context,
    const struct gpumas_physics * physics, gp_config * cfg);

/* Checks and settings of a job's context. */
static int gp_engine_context(gpumas_engine * g,
    const struct gpumas_context * context, gp_config * cfg,
    const gpumas_geometry ** geometry, int * locals)
{
        if (context == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        const gp_context * c = (const gp_context *)context;
        if (c->physics != g->physics) return GPUMAS_RETURN_PHYSICS_ERROR;
        if (!c->has_geometry) return GPUMAS_RETURN_MEDIUM_ERROR;
        const int rc = gp_config_check(context, c->physics, cfg);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        *geometry = c->d_geometry;
        *locals = c->has_locals;
        return GPUMAS_RETURN_SUCCESS;
}

/* One graph batch on the engine's stream, then the completions. */
static int gp_engine_batch(gpumas_engine * g)
{
        cudaStream_t s = g->stream;
        int rc = GPUMAS_RETURN_SUCCESS;
        const int launched = g->busy;
        if (g->n_uploaded < g->n_jobs) {
                const int k0 = g->n_uploaded, k = g->n_jobs - g->n_uploaded;
                rc = gp_check(cudaMemcpyAsync(g->d_jobs + k0, g->h_jobs + k0,
                    (size_t)k * sizeof(gp_job), cudaMemcpyHostToDevice, s));
                if (rc == GPUMAS_RETURN_SUCCESS)
                        rc = gp_check(cudaMemsetAsync(g->d_job_done + k0, 0,
                            (size_t)k * sizeof(unsigned long long), s));
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                g->n_uploaded = g->n_jobs;
        }
        if (g->busy) {
                gp_launch * h = g->h_launch;
                h->jobs = g->d_jobs;
                h->job_done = g->d_job_done;
                h->done_list = g->d_done_list;
                h->n_jobs = g->n_jobs;
                h->max_inner = (g->tuning.max_inner > 0) ?
                    g->tuning.max_inner : 8;
                h->total = g->total;
                h->tail_slots = (g->tuning.tail > 0) ? g->tuning.tail :
                    (g->tuning.tail < 0) ? (int)(g->grid_step * 128) : 0;
                rc = gp_check(cudaMemcpyAsync(g->view.launch, h,
                    sizeof(gp_launch), cudaMemcpyHostToDevice, s));
                const int loc = g->locals;
                if (rc == GPUMAS_RETURN_SUCCESS) rc = gp_engine_graph(g, loc);
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                cudaEventRecord(g->t0, s);
                rc = gp_check(cudaGraphLaunch(g->exec[loc], s));
                cudaEventRecord(g->t1, s);
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                g->stats.launches +=
                    GP_KERNELS_PER_ITERATION * g->graph_iters[loc] + 1;
                g->stats.batches++;
        }
        rc = gp_check(cudaMemcpyAsync(g->h_counters, g->view.counters,
            sizeof(gp_counters), cudaMemcpyDeviceToHost, s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaStreamSynchronize(s));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        if (g->busy) {
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, g->t0, g->t1) == cudaSuccess)
                        g->stats.kernel_ms += ms;
        }
        g->busy = !((g->h_counters->cursor >= g->total) &&
            (g->h_counters->active == 0));
        /* A batch that neither took an event from the queue nor moved one
         * while events remain is a stall (no kernel makes progress): fail
         * instead of looping. */
        if (!gp_moved(&g->seen_cursor, &g->seen_progress, *g->h_counters) &&
            launched && g->busy)
                return GPUMAS_RETURN_INTERNAL_ERROR;

        /* Jobs completed during the batch, in completion order. */
        const int nd = g->h_counters->n_done;
        if (nd > g->n_reported) {
                const int k0 = g->n_reported, k = nd - g->n_reported;
                rc = gp_check(cudaMemcpyAsync(g->h_done + k0,
                    g->d_done_list + k0, (size_t)k * sizeof(int),
                    cudaMemcpyDeviceToHost, s));
                if (rc == GPUMAS_RETURN_SUCCESS)
                        rc = gp_check(cudaStreamSynchronize(s));
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                int copies = 0;
                for (int q = k0; q < nd; q++) {
                        const int j = g->h_done[q];
                        const gp_job_host & info = g->h_info[j];
                        if (!info.in_arena) continue;
                        const gp_job & J = g->h_jobs[j];
                        rc = gp_check(cudaMemcpyAsync(info.states,
                            J.io.aos.states, J.n * sizeof(gpumas_state),
                            cudaMemcpyDeviceToHost, s));
                        if ((rc == GPUMAS_RETURN_SUCCESS) &&
                            (info.results != NULL))
                                rc = gp_check(cudaMemcpyAsync(info.results,
                                    J.io.aos.results,
                                    J.n * sizeof(gpumas_result),
                                    cudaMemcpyDeviceToHost, s));
                        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                        copies++;
                }
                if (copies > 0) {
                        rc = gp_check(cudaStreamSynchronize(s));
                        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                }
                for (int q = k0; q < nd; q++) {
                        const int j = g->h_done[q];
                        gp_job_host & info = g->h_info[j];
                        if (info.in_arena) {
                                rc = gp_arena_free(
                                    &g->arena, info.offset, info.bytes);
                                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                                info.in_arena = 0;
                        }
                        rc = gp_fifo_push(g, info.ticket);
                        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                        g->inflight--;
                }
                g->n_reported = nd;
        }
        return gp_engine_restart(g);
}

extern "C" void gpumas_engine_destroy(struct gpumas_engine ** engine)
{
        if ((engine == NULL) || (*engine == NULL)) return;
        gpumas_engine * g = *engine;
        if (g->stream != NULL) cudaStreamSynchronize(g->stream);
        gp_engine_free(g);
        *engine = NULL;
}

extern "C" int gp_api_engine_create(struct gpumas_engine ** engine,
    const struct gpumas_physics * physics,
    const struct gpumas_tuning * tuning, int max_jobs, size_t state_budget)
{
        if (engine == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        *engine = NULL;
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        if (max_jobs < 0) return GPUMAS_RETURN_VALUE_ERROR;
        gp_tuning t;
        t.engine = 2;
        t.pool_slots = 1048576;
        t.max_inner = 8;
        t.batch = 16;
        t.tail = 0;
        if (tuning != NULL) {
                if ((tuning->pool_slots < 0) || (tuning->max_inner < 0) ||
                    (tuning->batch < 0))
                        return GPUMAS_RETURN_VALUE_ERROR;
                if (tuning->pool_slots > 0) t.pool_slots = tuning->pool_slots;
                if (tuning->max_inner > 0) t.max_inner = tuning->max_inner;
                if (tuning->batch > 0) t.batch = tuning->batch;
                t.tail = tuning->tail;
        }
        if (t.pool_slots < 128) t.pool_slots = 128;
        return gp_engine_new(engine, physics, NULL, &t,
            (max_jobs > 0) ? max_jobs : 65536, state_budget);
}

/* Room for one more job in the table. */
static int gp_engine_room(gpumas_engine * g)
{
        if (g->n_jobs < g->capacity) return GPUMAS_RETURN_SUCCESS;
        const int rc = gp_engine_restart(g);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        return (g->n_jobs < g->capacity) ? GPUMAS_RETURN_SUCCESS :
                                           GPUMAS_RETURN_MEMORY_ERROR;
}

extern "C" int gp_api_engine_submit(struct gpumas_engine * engine,
    const struct gpumas_job * job, int * ticket)
{
        if ((engine == NULL) || (job == NULL) || (ticket == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        gpumas_engine * g = engine;
        gp_config cfg;
        const gpumas_geometry * geometry;
        int locals;
        int rc = gp_engine_context(g, job->context, &cfg, &geometry, &locals);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        if (job->n > 0) {
                const gpumas_soa & a = job->events;
                if ((a.charge == NULL) || (a.energy == NULL) ||
                    (a.distance == NULL) || (a.grammage == NULL) ||
                    (a.time == NULL) || (a.weight == NULL) ||
                    (a.position[0] == NULL) || (a.position[1] == NULL) ||
                    (a.position[2] == NULL) || (a.direction[0] == NULL) ||
                    (a.direction[1] == NULL) || (a.direction[2] == NULL) ||
                    (a.decayed == NULL) || (cfg.carry && (a.result == NULL)))
                        return GPUMAS_RETURN_VALUE_ERROR;
        }
        rc = gp_engine_room(g);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        gp_io io;
        memset(&io, 0, sizeof(io));
        io.soa.a = job->events;
        gp_job_host info;
        memset(&info, 0, sizeof(info));
        return gp_engine_append(g, cfg, geometry, io, job->n,
            job->first_event, info, ticket, locals);
}

extern "C" int gp_api_engine_submit_host(struct gpumas_engine * engine,
    const struct gpumas_context * context, size_t n,
    struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event, int * ticket)
{
        if ((engine == NULL) || (ticket == NULL) ||
            ((n > 0) && (states == NULL)))
                return GPUMAS_RETURN_VALUE_ERROR;
        gpumas_engine * g = engine;
        gp_config cfg;
        const gpumas_geometry * geometry;
        int locals;
        int rc = gp_engine_context(g, context, &cfg, &geometry, &locals);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        if (cfg.carry && (n > 0) && (results == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        rc = gp_engine_room(g);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        gp_job_host info;
        memset(&info, 0, sizeof(info));
        gp_io io;
        memset(&io, 0, sizeof(io));
        if (n > 0) {
                const size_t bs = gp_align256(n * sizeof(gpumas_state));
                const size_t bytes = bs + n * sizeof(gpumas_result);
                size_t offset;
                if ((g->arena.base == NULL) ||
                    !gp_arena_alloc(&g->arena, bytes, &offset))
                        return GPUMAS_RETURN_MEMORY_ERROR;
                io.aos.states = (gpumas_state *)(g->arena.base + offset);
                io.aos.results = (gpumas_result *)(g->arena.base + offset +
                    bs);
                rc = gp_check(cudaMemcpyAsync(io.aos.states, states,
                    n * sizeof(gpumas_state), cudaMemcpyHostToDevice,
                    g->stream));
                if ((rc == GPUMAS_RETURN_SUCCESS) && cfg.carry)
                        rc = gp_check(cudaMemcpyAsync(io.aos.results, results,
                            n * sizeof(gpumas_result), cudaMemcpyHostToDevice,
                            g->stream));
                if (rc != GPUMAS_RETURN_SUCCESS) {
                        gp_arena_free(&g->arena, offset, bytes);
                        return rc;
                }
                info.states = states;
                info.results = results;
                info.offset = offset;
                info.bytes = bytes;
                info.in_arena = 1;
        }
        return gp_engine_append(g, cfg, geometry, io, n, first_event, info,
            ticket, locals);
}

extern "C" int gp_api_engine_step(struct gpumas_engine * engine,
    int max_done, int * done, int * n_done, int * pending)
{
        if ((engine == NULL) || ((max_done > 0) && (done == NULL)))
                return GPUMAS_RETURN_VALUE_ERROR;
        gpumas_engine * g = engine;
        int rc = GPUMAS_RETURN_SUCCESS;
        if (g->busy || (g->n_uploaded < g->n_jobs)) rc = gp_engine_batch(g);
        int k = 0;
        while ((rc == GPUMAS_RETURN_SUCCESS) && (k < max_done) &&
            (g->fifo_n > 0)) {
                done[k++] = g->fifo[g->fifo_head];
                g->fifo_head = (g->fifo_head + 1) % g->fifo_cap;
                g->fifo_n--;
        }
        if (n_done != NULL) *n_done = k;
        if (pending != NULL) *pending = g->inflight + g->fifo_n;
        return rc;
}

extern "C" int gp_api_engine_run(struct gpumas_engine * engine,
    size_t n_jobs, const struct gpumas_job * jobs)
{
        if ((engine == NULL) || ((n_jobs > 0) && (jobs == NULL)))
                return GPUMAS_RETURN_VALUE_ERROR;
        gpumas_engine * g = engine;
        for (size_t k = 0; k < n_jobs; k++) {
                int ticket;
                int rc = gp_api_engine_submit(g, jobs + k, &ticket);
                if (rc == GPUMAS_RETURN_MEMORY_ERROR) {
                        /* Table full: drain it, then go on. */
                        while ((rc == GPUMAS_RETURN_MEMORY_ERROR) &&
                            (g->inflight > 0)) {
                                rc = gp_engine_batch(g);
                                if (rc == GPUMAS_RETURN_SUCCESS)
                                        rc = gp_api_engine_submit(
                                            g, jobs + k, &ticket);
                        }
                }
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        }
        while (g->inflight > 0 || g->busy) {
                /* Ends: every batch moves an event or fails (stall). */
                const int rc = gp_engine_batch(g);
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        }
        /* Completions of a run are not reported as tickets. */
        g->fifo_n = 0;
        g->fifo_head = 0;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_engine_stats(const struct gpumas_engine * engine,
    struct gpumas_engine_stats * stats)
{
        if ((engine == NULL) || (stats == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        *stats = engine->stats;
        stats->budget_used = engine->arena.used;
        return GPUMAS_RETURN_SUCCESS;
}

/* ------------------------------------------------------------------------ */
/* Context path: one job through the context's own engine.                  */
/* ------------------------------------------------------------------------ */
extern "C" void gp_pool_free(struct gpumas_engine * g)
{
        if (g != NULL) gp_engine_free(g);
}

/* Transport n events of `io` with the slot pool, on stream s. Returns the
 * number of kernel launches in *launches. */
extern "C" int gp_pool_transport(gp_context * c, const gp_config * cfg,
    const gp_io * io, size_t n, uint64_t first, cudaStream_t s,
    const gp_tuning * tuning, int * launches)
{
        int P = tuning->pool_slots;
        if ((size_t)P > n) P = (int)((n + 127) / 128 * 128);
        if (P < 128) P = 128;
        int rc;
        if (c->pool == NULL) {
                gp_tuning t = *tuning;
                t.pool_slots = P;
                rc = gp_engine_new(&c->pool, c->physics, c->d_tables, &t, 1,
                    0);
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        }
        gpumas_engine * g = c->pool;
        g->tuning = *tuning;
        /* Work of this call on the caller's stream. */
        cudaStream_t own = g->stream;
        g->stream = s;
        rc = gp_engine_pool(g, P);
        const long long l0 = g->stats.launches;
        int ticket = 0;
        if (rc == GPUMAS_RETURN_SUCCESS) rc = gp_engine_room(g);
        if (rc == GPUMAS_RETURN_SUCCESS) {
                gp_job_host info;
                memset(&info, 0, sizeof(info));
                rc = gp_engine_append(g, *cfg, c->d_geometry, *io, n, first,
                    info, &ticket, c->has_locals);
        }
        /* Ends: every batch moves an event or fails (stall). */
        while ((rc == GPUMAS_RETURN_SUCCESS) && (g->inflight > 0 || g->busy))
                rc = gp_engine_batch(g);
        g->fifo_n = 0;
        g->fifo_head = 0;
        g->stream = own;
        if (launches != NULL) *launches = (int)(g->stats.launches - l0);
        if (rc != GPUMAS_RETURN_SUCCESS) {
                /* Start afresh at the next call. */
                cudaStreamSynchronize(s);
                gp_engine_free(g);
                c->pool = NULL;
        }
        return rc;
}

/* ------------------------------------------------------------------------ */
/* Allocation free transport.                                               */
/*                                                                          */
/* Some callers cannot allocate device memory while they transport: a host  */
/* program whose allocator owns all of the GPU memory and hands out fixed   */
/* arenas, a plugin embedded in a framework that forbids allocation on its  */
/* hot path, or code that must not pay (or fail on) a cudaMalloc in the     */
/* middle of a run. For them the slot pool of the pool engine also exists   */
/* as one static device array. The CUDA runtime loads the library's device  */
/* code on a device lazily, at its first use there, and reserves the array  */
/* then: gp_static_reserve does that when a physics is loaded onto the      */
/* device (gpumas_physics_load / _upload), where the caller allocates       */
/* anyway, so that the transport calls themselves allocate nothing. The     */
/* array is kept until the process exits.                                   */
/* ------------------------------------------------------------------------ */

/* Largest pool of the allocation free entry point, in event slots
 * (GPUMAS_STATIC_SLOTS of gpumas.h). */
#define GP_STATIC_SLOTS GPUMAS_STATIC_SLOTS

/* Bytes of the static pool: the layout of gp_pool_bytes for the largest
 * pool, then one job record, its completion count and completion list. */
#define GP_A256(n) ((((size_t)(n)) + 255) & ~(size_t)255)
#define GP_STATIC_POOL_BYTES                                                  \
        (GP_A256((size_t)SD_N * GP_STATIC_SLOTS * sizeof(double)) +           \
            GP_A256((size_t)SU_N * GP_STATIC_SLOTS * sizeof(uint64_t)) +      \
            GP_A256((size_t)SI_N * GP_STATIC_SLOTS * sizeof(int)) +           \
            GP_A256((size_t)6 * GP_STATIC_SLOTS * sizeof(int)) +              \
            GP_A256(sizeof(gp_counters)) + GP_A256(sizeof(gp_launch)))
#define GP_STATIC_BYTES (GP_STATIC_POOL_BYTES + GP_A256(sizeof(gp_job)) + 256)

static __device__ __align__(256) unsigned char gp_static_pool[GP_STATIC_BYTES];

/* Device address of gp_static_pool on the current device (a host side use
 * of the symbol itself is not a device address). The lookup loads this
 * file's device code on the current device if it is not loaded yet, which
 * reserves the array there. It is made at every call: once the code is
 * loaded it is a table lookup of the runtime, safe from several host
 * threads, and it stays right after a device reset. */
static int gp_static_setup(void ** address)
{
        void * ptr = NULL;
        if (cudaGetSymbolAddress(&ptr, gp_static_pool) != cudaSuccess)
                return GPUMAS_RETURN_DEVICE_ERROR;
        *address = ptr;
        return GPUMAS_RETURN_SUCCESS;
}

/* Reserve the static array on the current device (at physics load). */
extern "C" int gp_static_reserve(void)
{
        void * ptr = NULL;
        return gp_static_setup(&ptr);
}

extern "C" int gp_api_context_transport_device_static(
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
        if (cfg.carry && (events->result == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;

        void * base = NULL;
        rc = gp_static_setup(&base);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;

        /* Carve the static array: the pool of P slots, then the job. No more
         * slots than events, as in gp_pool_transport. */
        int P = pool_slots;
        if ((size_t)P > n) P = (int)((n + 127) / 128 * 128);
        gp_pool_view v;
        gp_pool_carve((char *)base, P, &v);
        gp_job * job = (gp_job *)((char *)base + GP_STATIC_POOL_BYTES);
        unsigned long long * job_done = (unsigned long long *)(
            (char *)job + GP_A256(sizeof(gp_job)));
        int * done_list = (int *)(job_done + 1);

        cudaStream_t s = (cudaStream_t)stream;
        /* The array keeps the previous call's contents: empty every slot
         * and zero the counters and the completion count. */
        rc = gp_check(cudaMemsetAsync(v.pool.i + (size_t)SI_PHASE * P, 0,
            (size_t)P * sizeof(int), s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemsetAsync(v.counters, 0,
                    sizeof(gp_counters), s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemsetAsync(job_done, 0,
                    sizeof(unsigned long long), s));
        gp_job hj;
        memset(&hj, 0, sizeof(hj));
        hj.cfg = cfg;
        hj.geometry = c->d_geometry;
        hj.io.soa.a = *events;
        hj.begin = 0;
        hj.n = n;
        hj.first_event = first_event;
        gp_launch h;
        memset(&h, 0, sizeof(h));
        h.jobs = job;
        h.job_done = job_done;
        h.done_list = done_list;
        h.n_jobs = 1;
        const unsigned int grid_step = gp_step_wave(P, 128);
        h.max_inner = (c->tuning.max_inner > 0) ? c->tuning.max_inner : 8;
        h.total = n;
        h.tail_slots = (c->tuning.tail > 0) ? c->tuning.tail :
            (c->tuning.tail < 0) ? (int)(grid_step * 128) : 0;
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpyAsync(job, &hj, sizeof(hj),
                    cudaMemcpyHostToDevice, s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpyAsync(v.launch, &h, sizeof(h),
                    cudaMemcpyHostToDevice, s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaStreamSynchronize(s));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;

        const int batch = 16;
        unsigned long long seen_cursor = 0, seen_progress = 0;
        for (;;) {
                for (int k = 0; k < batch; k++) {
                        if (c->has_locals)
                                gp_iteration<1>(c->d_tables, v, grid_step, k,
                                    s);
                        else
                                gp_iteration<0>(c->d_tables, v, grid_step, k,
                                    s);
                }
                if (c->has_locals)
                        gp_batch_end<1>(c->d_tables, v, s);
                else
                        gp_batch_end<0>(c->d_tables, v, s);
                rc = gp_check(cudaGetLastError());
                gp_counters hc;
                if (rc == GPUMAS_RETURN_SUCCESS)
                        rc = gp_check(cudaMemcpyAsync(&hc, v.counters,
                            sizeof(hc), cudaMemcpyDeviceToHost, s));
                if (rc == GPUMAS_RETURN_SUCCESS)
                        rc = gp_check(cudaStreamSynchronize(s));
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                if ((hc.cursor >= n) && (hc.active == 0)) break;
                /* A batch that neither took an event from the queue nor
                 * moved one is a stall: fail instead of looping. */
                if (!gp_moved(&seen_cursor, &seen_progress, hc))
                        return GPUMAS_RETURN_INTERNAL_ERROR;
        }
        return GPUMAS_RETURN_SUCCESS;
}

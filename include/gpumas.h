/*
 * gpumas.h -- C ABI of the GB300 muon transport engine (libgpumas.so).
 *
 * This library runs the hot path of the reference library PUMAS 1.2.3,
 * `pumas_context_transport` (pumas.h:1046-1048), on an NVIDIA GB300 GPU for
 * whole batches of events: forward and backward Monte Carlo with CSDA, mixed
 * or straggled energy loss, discrete energy losses (bremsstrahlung, pair
 * production, photonuclear, delta rays), mixed Coulomb multiple scattering,
 * decay weighting or randomisation and geometry stepping.
 *
 * The API mirrors pumas.h: the physics tables are the reference's own
 * (produced by `pumas_physics_create` and serialised by
 * `pumas_physics_dump`), contexts carry the same mode / event / limit /
 * accuracy settings, and states use the layout of `struct pumas_state`. What
 * differs is what a GPU needs instead of host callbacks:
 *   - the medium callback is replaced by a geometry descriptor
 *     (gpumas_geometry.h);
 *   - the random callback is replaced by a Philox-4x32-10 stream keyed by
 *     (seed, event id), see `gpumas_context.seed`;
 *   - the transport call takes arrays of events.
 *
 * All functions return an `enum pumas_return` value (pumas.h:143-196) as an
 * int. The library never exits the process; there is no CPU fallback, and
 * every transport entry point returns PUMAS_RETURN_PHYSICS_ERROR-like codes
 * (GPUMAS_RETURN_DEVICE_ERROR) if no CUDA device is usable.
 */
#ifndef GPUMAS_H
#define GPUMAS_H

#include <stddef.h>
#include <stdint.h>

#include "gpumas_geometry.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes: same values as enum pumas_return (pumas.h:143-196). */
#define GPUMAS_RETURN_SUCCESS 0
#define GPUMAS_RETURN_ACCURACY_ERROR 1
#define GPUMAS_RETURN_END_OF_FILE 2
#define GPUMAS_RETURN_DECAY_ERROR 3
#define GPUMAS_RETURN_DENSITY_ERROR 4
#define GPUMAS_RETURN_DIRECTION_ERROR 5
#define GPUMAS_RETURN_INCOMPLETE_FILE 6
#define GPUMAS_RETURN_INDEX_ERROR 7
#define GPUMAS_RETURN_PHYSICS_ERROR 8
#define GPUMAS_RETURN_INTERNAL_ERROR 9
#define GPUMAS_RETURN_IO_ERROR 10
#define GPUMAS_RETURN_FORMAT_ERROR 11
#define GPUMAS_RETURN_MEDIUM_ERROR 12
#define GPUMAS_RETURN_MEMORY_ERROR 13
#define GPUMAS_RETURN_MODEL_ERROR 14
#define GPUMAS_RETURN_MISSING_LIMIT 15
#define GPUMAS_RETURN_MISSING_RANDOM 16
#define GPUMAS_RETURN_PATH_ERROR 17
#define GPUMAS_RETURN_RAISE_ERROR 18
#define GPUMAS_RETURN_TOO_LONG 19
#define GPUMAS_RETURN_UNDEFINED_MDF 20
#define GPUMAS_RETURN_UNKNOWN_ELEMENT 21
#define GPUMAS_RETURN_UNKNOWN_MATERIAL 22
#define GPUMAS_RETURN_UNKNOWN_PARTICLE 23
#define GPUMAS_RETURN_VALUE_ERROR 24
/* Codes beyond the reference's: a CUDA call failed. */
#define GPUMAS_RETURN_DEVICE_ERROR 64

/* Modes and events: same values as enum pumas_mode and pumas_event. */
#define GPUMAS_MODE_DISABLED -1
#define GPUMAS_MODE_CSDA 0
#define GPUMAS_MODE_MIXED 1
#define GPUMAS_MODE_STRAGGLED 2
#define GPUMAS_MODE_WEIGHTED 0
#define GPUMAS_MODE_RANDOMISED 1
#define GPUMAS_MODE_FORWARD 0
#define GPUMAS_MODE_BACKWARD 1

/* Particles: same values as enum pumas_particle. */
#define GPUMAS_PARTICLE_MUON 0
#define GPUMAS_PARTICLE_TAU 1

#define GPUMAS_EVENT_NONE 0
#define GPUMAS_EVENT_LIMIT_ENERGY 1
#define GPUMAS_EVENT_LIMIT_DISTANCE 2
#define GPUMAS_EVENT_LIMIT_GRAMMAGE 4
#define GPUMAS_EVENT_LIMIT_TIME 8
#define GPUMAS_EVENT_LIMIT 15
#define GPUMAS_EVENT_MEDIUM 16
#define GPUMAS_EVENT_VERTEX_BREMSSTRAHLUNG 32
#define GPUMAS_EVENT_VERTEX_PAIR_CREATION 64
#define GPUMAS_EVENT_VERTEX_PHOTONUCLEAR 128
#define GPUMAS_EVENT_VERTEX_DELTA_RAY 256
#define GPUMAS_EVENT_VERTEX_DEL 480
#define GPUMAS_EVENT_VERTEX_COULOMB 512
#define GPUMAS_EVENT_VERTEX_DECAY 1024
#define GPUMAS_EVENT_VERTEX 2016
#define GPUMAS_EVENT_WEIGHT 2048

/** A Monte Carlo state: same layout as struct pumas_state
 * (pumas.h:289-309), so that arrays of either type can be passed. */
struct gpumas_state {
        double charge;
        double energy;
        double distance;
        double grammage;
        double time;
        double weight;
        double position[3];
        double direction[3];
        int decayed;
};

/** Per event outputs besides the state. */
struct gpumas_result {
        /** The transport end event (pumas_context_transport `event`). */
        int event;
        /** Start and end medium indices in the geometry (`media[2]`),
         * -1 for no medium. */
        int medium_in;
        int medium_out;
        /** The per event return code (pumas_context_transport's return). */
        int status;
        /** Number of geometric step proposals (medium callback calls with a
         * step argument, pumas.c:3182, 5281). */
        int steps;
        /** Box-Muller cache of the event's normal deviates at the end of
         * the call (step_randn, pumas.c:7016-7029): 1 when `randn_next`
         * holds the second deviate of a pair, else 0. */
        int randn_done;
        /** Position of the event's random stream at the end of the call:
         * the number of draws consumed since its first call. */
        uint64_t draws;
        /** The cached deviate, meaningful when randn_done is 1. */
        double randn_next;
};

/** Structure of arrays view of events in device memory. Every pointer
 * holds `n` values; `result` may be NULL. */
struct gpumas_soa {
        double * charge;
        double * energy;
        double * distance;
        double * grammage;
        double * time;
        double * weight;
        double * position[3];
        double * direction[3];
        int * decayed;
        struct gpumas_result * result;
};

/* ------------------------------------------------------------------------ */
/* Physics.                                                                 */
/* ------------------------------------------------------------------------ */

/** Device image of the physics tables. */
struct gpumas_physics;

/**
 * Load physics tables from the bytes of a `pumas_physics_dump` stream
 * (pumas.c:2167-2196; replaces pumas_physics_load, pumas.h:980-981) and
 * upload them to the current CUDA device. The dump must come from an LP64
 * little-endian host (tag 13), for muons or taus, with any of the
 * reference's DCS models (bremsstrahlung SSR, KKP or ABB; pair production
 * SSR or KKP; photonuclear DRSS, BBKS or BM); otherwise
 * GPUMAS_RETURN_FORMAT_ERROR or GPUMAS_RETURN_MODEL_ERROR (an unknown
 * model name) is returned.
 */
int gpumas_physics_load(
    struct gpumas_physics ** physics, const void * dump, size_t size);

/**
 * Upload a live `struct pumas_physics` (returned by the reference's
 * pumas_physics_create or pumas_physics_load, pumas.h:898-981) of this
 * process. Same checks as gpumas_physics_load.
 */
int gpumas_physics_upload(
    struct gpumas_physics ** physics, const void * pumas_physics);

/**
 * Tabulate on the device the per element DEL tables of a physics, from its
 * own elements, energy grid, cutoff and DCS models, as the reference's
 * pumas_physics_create does (pumas.c:10704-10737, 11358-11438,
 * 11629-11735): the restricted cross sections CSn (180 point Gauss-Legendre
 * integrals of the DCS in ln q, the analytic one for ionisation) and their
 * PCHIP slopes over the energy grid, for the 4 DEL processes, n_elements x
 * n_energies each, in the reference's layout [process][element][row]; the
 * single precision DCS interpolation tables of the 3 radiative processes,
 * [process][element][row][n_table_dcs][2] (logarithm of the DCS and slope
 * in ln(q / K)); and the exponents of their envelopes, [process][element]
 * [row]. All arrays are in host memory. `ms`, if not NULL, receives the
 * device time in ms. The tables a physics was loaded with can be compared
 * with these: they come from the same definitions.
 */
int gpumas_physics_tabulate(const struct gpumas_physics * physics,
    double * csn, double * csn_dk, float * dcs, float * alpha, float * ms);

/** Release the device image (pumas_physics_destroy, pumas.h:924). */
void gpumas_physics_destroy(struct gpumas_physics ** physics);

/** Index of a material from its name (pumas_physics_material_index,
 * pumas.h:1772-1773). */
int gpumas_physics_material_index(const struct gpumas_physics * physics,
    const char * name, int * index);

/** Number of materials and elements, the cutoff and the particle mass. */
int gpumas_physics_info(const struct gpumas_physics * physics,
    int * n_materials, int * n_elements, double * cutoff, double * mass);

/** Transported particle (GPUMAS_PARTICLE_MUON or GPUMAS_PARTICLE_TAU), its
 * proper lifetime c tau in m and its mass in GeV/c^2. Replaces
 * `pumas_physics_particle` (pumas.h:1106-1108). The particle, and the DCS
 * models, come from the physics dump. */
int gpumas_physics_particle(const struct gpumas_physics * physics,
    int * particle, double * lifetime, double * mass);

/* ------------------------------------------------------------------------ */
/* Contexts.                                                                */
/* ------------------------------------------------------------------------ */

/** Mode flags (struct pumas_context_mode, pumas.h:554-579). */
struct gpumas_context_mode {
        int energy_loss;
        int decay;
        int direction;
        int scattering;
};

/** External limits (struct pumas_context_limit, pumas.h:582-594). */
struct gpumas_context_limit {
        double energy;
        double distance;
        double grammage;
        double time;
};

/**
 * A simulation context. The public fields have the meaning and defaults of
 * struct pumas_context (pumas.h:636-672; defaults pumas.c:2592-2612):
 * STRAGGLED energy loss, MIXED scattering, FORWARD, WEIGHTED decay,
 * no stop event, null limits and an accuracy of 1E-02.
 */
struct gpumas_context {
        struct gpumas_context_mode mode;
        int event;
        struct gpumas_context_limit limit;
        double accuracy;
        /** Key of the Philox random stream (replaces `random`). */
        uint64_t seed;
        /** A pointer to user memory of `extra_memory` bytes, or NULL. */
        void * user_data;
};

/** Create a context (pumas_context_create, pumas.h:1214-1216). */
int gpumas_context_create(struct gpumas_context ** context,
    const struct gpumas_physics * physics, int extra_memory);

/** Destroy a context and its device buffers (pumas_context_destroy, pumas.h:1326). */
void gpumas_context_destroy(struct gpumas_context ** context);

/** Set the key of the context's random stream
 * (pumas_context_random_seed_set, pumas.h:1240-1241). With a NULL seed the
 * key is drawn from the OS random stream (/dev/urandom), whose failure
 * returns GPUMAS_RETURN_PATH_ERROR. A new context has the key 0. */
int gpumas_context_random_seed_set(
    struct gpumas_context * context, const uint64_t * seed);

/** Get the key of the context's random stream
 * (pumas_context_random_seed_get, pumas.h:1265-1266). */
int gpumas_context_random_seed_get(
    const struct gpumas_context * context, uint64_t * seed);

/** The physics of a context (pumas_context_physics_get, pumas.h:1337). */
const struct gpumas_physics * gpumas_context_physics_get(
    const struct gpumas_context * context);

/** Minimum kinetic transfer of DELs, relative (pumas_physics_cutoff,
 * pumas.h:993), and elastic ratio (pumas_physics_elastic_ratio,
 * pumas.h:1005); 0 for a NULL physics. */
double gpumas_physics_cutoff(const struct gpumas_physics * physics);
double gpumas_physics_elastic_ratio(const struct gpumas_physics * physics);

/**
 * Set the geometry (replaces the `medium` callback). The descriptor and its
 * arrays are copied to the device; media materials are checked against the
 * physics.
 */
int gpumas_context_geometry_set(
    struct gpumas_context * context, const struct gpumas_geometry * geometry);

/**
 * Transport n events held in host memory (the batched form of
 * pumas_context_transport, pumas.h:1046-1048). States are updated in place;
 * `results` (n entries, may be NULL) receives the per event end event,
 * media, return code and counters. Event k uses the random stream of event
 * id `first_event + k`. The return value is GPUMAS_RETURN_SUCCESS if the
 * configuration is valid and every event succeeded, the first failing
 * event's code otherwise (context level checks mirror pumas.c:3120-3177).
 */
int gpumas_context_transport(struct gpumas_context * context, size_t n,
    struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event);

/**
 * Transport n events held in device memory as a structure of arrays, on a
 * CUDA stream (cudaStream_t, or NULL for the default stream). Asynchronous:
 * only the configuration is checked before returning.
 */
int gpumas_context_transport_device(struct gpumas_context * context,
    size_t n, const struct gpumas_soa * events, uint64_t first_event,
    void * stream);

/** A recorded frame (struct pumas_frame, pumas.h:378-395): the state, the
 * medium index in the geometry (-1 for none) and the event flags, with the
 * reference's PUMAS_EVENT_START (4096) and PUMAS_EVENT_STOP (8192). */
struct gpumas_frame {
        struct gpumas_state state;
        int medium;
        int event;
};

#define GPUMAS_EVENT_START 4096
#define GPUMAS_EVENT_STOP 8192

/**
 * A device frame recorder (struct pumas_recorder, pumas.h:432-458). Event k
 * of a transport call writes its frames to frames[k * max_frames ...] and
 * the number of frames the reference's recorder would hold to length[k];
 * frames beyond max_frames are not written (length still counts them). As
 * in the reference, `period` = 1 records every step, n every n-th step and
 * a period <= 0 only the start, the stop, the DELs and the medium changes
 * (pumas.c:5227-5231, 5296-5374, 5464-5467, 5507-5510, 4793-4798,
 * 4944-4946). Both arrays are in device memory.
 */
struct gpumas_recorder {
        int period;
        int max_frames;
        struct gpumas_frame * frames;
        int * length;
};

/**
 * Record the next transport calls of this context (the `recorder` field of
 * pumas_context, pumas.h:636-672), or stop recording with NULL. A
 * recording context runs the one thread per event engine; the transported
 * states are the same as without recording.
 */
int gpumas_context_recorder_set(struct gpumas_context * context,
    const struct gpumas_recorder * recorder);

/**
 * Engine parameters of a context. `engine` selects the execution scheme:
 * 0 automatic, 1 one GPU thread per event for the whole transport call,
 * 2 the slot pool, where events are refilled into `pool_slots` resident
 * slots and stepped by kernels regrouped by step kind (continuous step,
 * DEL, hard elastic scatter), with `max_inner` continuous steps per slot and
 * iteration and `batch` iterations per captured CUDA graph. With `tail`
 * > 0, once every event is in a slot and at most `tail` slots are active,
 * the remaining events run to their end in one launch (negative: one slot
 * per resident thread; 0, the default: never). Results do not depend on
 * these parameters. Zero fields keep the current value.
 */
struct gpumas_tuning {
        int engine;
        int pool_slots;
        int max_inner;
        int batch;
        int tail;
};

int gpumas_context_tuning_set(
    struct gpumas_context * context, const struct gpumas_tuning * tuning);
int gpumas_context_tuning_get(
    const struct gpumas_context * context, struct gpumas_tuning * tuning);

/**
 * Failure detection of the rejection samplings. The reference's rejection
 * loops have no bound (pumas.c:5839, 6115, 6126, 6241, 6918, 6973, 11208);
 * on the device each of them stops after `max_trials` trials and the event
 * ends with GPUMAS_RETURN_INTERNAL_ERROR in its result, the other events of
 * the call going on unchanged. A new context has 100 000 trials; 0 restores
 * that default, negative values return GPUMAS_RETURN_VALUE_ERROR. No
 * counterpart in the reference.
 */
int gpumas_context_trials_set(struct gpumas_context * context,
    int max_trials);
int gpumas_context_trials_get(const struct gpumas_context * context,
    int * max_trials);

/**
 * Events transported over several calls. A reference context keeps its
 * random engine and its Box-Muller cache from one pumas_context_transport
 * call to the next (struct simulation_context, pumas.c:426-477; reset only
 * at creation, pumas.c:2607-2609), so that an event transported in several
 * calls -- switching energy loss and scattering modes at an energy
 * threshold, as in examples/pumas/geometry.c:269-312 -- continues its
 * random sequence. Here each event's random stream is keyed by (seed, event
 * id). With `carry` set to 1, every transport call starts each event where
 * its gpumas_result entry says -- stream position `draws`, Box-Muller cache
 * `randn_done` and `randn_next`, all zero before the first call -- and
 * leaves the end values there for the next call; the results array is then
 * required (GPUMAS_RETURN_VALUE_ERROR without it). With 0, the default,
 * each call starts every event's stream afresh, as a new reference context
 * per event would. Results of an event over a chain of calls do not depend
 * on the engine or on what runs beside it.
 */
int gpumas_context_carry_set(struct gpumas_context * context, int carry);
int gpumas_context_carry_get(
    const struct gpumas_context * context, int * carry);

/**
 * Allocation free form of gpumas_context_transport_device. It has no
 * counterpart in the reference: it exists for callers that cannot allocate
 * device memory while they transport (a host whose allocator owns the GPU
 * memory, a plugin whose framework forbids allocation on its hot path).
 *
 * The slot pool lives in one static device array of the library, sized for
 * GPUMAS_STATIC_SLOTS slots (about 13 MB), which every GPU that loads the
 * library holds until the process exits. `pool_slots` must be a multiple of
 * 128 in [128, GPUMAS_STATIC_SLOTS], or 0 for the maximum; other values
 * return GPUMAS_RETURN_VALUE_ERROR. The call makes no cudaMalloc or
 * cudaFree; events, of any number n, stream through the slots as in the
 * pool engine and give the same results.
 *
 * The array is reserved on a device when a physics is loaded there
 * (gpumas_physics_load or gpumas_physics_upload, with that device current:
 * the CUDA runtime loads the library's device code, and with it the array,
 * at its first use on a device). Transport calls on that device then only
 * look up the array's address. Every call shares the array and clears it
 * at its start, so calls that overlap on the GPU (other streams or threads)
 * race and must be serialised by the caller. The call waits for `stream`
 * (cudaStreamSynchronize) between its batches of iterations, so it must not
 * be made while `stream` is being captured into a CUDA graph. Slots beyond
 * the number of events are not used; the engine parameters of the context
 * (gpumas_context_tuning_set: max_inner, tail) apply as in the pool engine.
 */
#define GPUMAS_STATIC_SLOTS 32768
int gpumas_context_transport_device_static(struct gpumas_context * context,
    size_t n, const struct gpumas_soa * events, uint64_t first_event,
    int pool_slots, void * stream);

/* ------------------------------------------------------------------------ */
/* Batched jobs and continuous batching.                                    */
/* ------------------------------------------------------------------------ */

/*
 * The reference transports one event per call; a program with many
 * independent transport jobs (different geometries, modes, limits, seeds
 * and event counts) calls pumas_context_transport in nested loops over jobs
 * and events (e.g. examples/pumas/geometry.c:229-313 for one job). An
 * engine runs all of them in one resident slot pool: the events of every
 * submitted job share one device event queue, each slot steps the event of
 * whatever job it took, and a slot freed by a finished event takes the next
 * queued event, of any job. Jobs can be submitted while others run
 * (continuous batching): their events join the queue and fill slots as
 * they free up. Results do not depend on what else runs: event k of a job
 * always uses the random stream (context seed, first_event + k).
 */

/** A job whose events are in device memory (structure of arrays). The
 * context supplies the settings, the geometry and the seed; it must use the
 * engine's physics and outlive the job, with its geometry unchanged. */
struct gpumas_job {
        const struct gpumas_context * context;
        size_t n;
        struct gpumas_soa events;
        uint64_t first_event;
};

/** A persistent transport engine. */
struct gpumas_engine;

/**
 * Create an engine for `physics` with the pool parameters of `tuning` (NULL
 * or zero fields for defaults: 1 048 576 slots, 8 steps per slot visit, 16
 * iterations per graph), room for `max_jobs` jobs in flight (0: 65 536) and
 * a device budget of `state_budget` bytes for the events of jobs submitted
 * from host memory (0: none). Allocates all of its device memory here.
 */
int gpumas_engine_create(struct gpumas_engine ** engine,
    const struct gpumas_physics * physics,
    const struct gpumas_tuning * tuning, int max_jobs, size_t state_budget);

/** Wait for the engine's work and release it. */
void gpumas_engine_destroy(struct gpumas_engine ** engine);

/**
 * Queue a job whose events are in device memory. Returns its ticket in
 * *ticket. The job starts running at the next gpumas_engine_step. Returns
 * GPUMAS_RETURN_MEMORY_ERROR if `max_jobs` jobs are already in flight,
 * other codes for an invalid context (the checks of pumas.c:3120-3177).
 */
int gpumas_engine_submit(struct gpumas_engine * engine,
    const struct gpumas_job * job, int * ticket);

/**
 * Queue a job whose events are `pumas_state` records in host memory. The
 * events are copied into the engine's state budget (144 bytes per event)
 * and back into `states` (and `results`, if not NULL) when the job
 * completes, before its ticket is reported. Returns
 * GPUMAS_RETURN_MEMORY_ERROR, with no side effect, when the budget has no
 * room for the job now (submit it again after some jobs completed).
 */
int gpumas_engine_submit_host(struct gpumas_engine * engine,
    const struct gpumas_context * context, size_t n,
    struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event, int * ticket);

/**
 * Run one batch of pool iterations (one CUDA graph launch) and wait for it.
 * Tickets of jobs completed since the last call are written to `done` (at
 * most `max_done`; the rest are reported by the next calls), their number
 * to *n_done and the number of submitted jobs not yet reported to
 * *pending. Does nothing on the device when no event is queued or running.
 */
int gpumas_engine_step(struct gpumas_engine * engine, int max_done,
    int * done, int * n_done, int * pending);

/** Submit `n_jobs` device jobs and step until all of them completed (the
 * batched form: one pool, one event queue, CUDA graph batches). */
int gpumas_engine_run(struct gpumas_engine * engine, size_t n_jobs,
    const struct gpumas_job * jobs);

/** Cumulated statistics: kernel launches and device time of the engine's
 * graph batches since the engine was created. */
struct gpumas_engine_stats {
        long long launches;
        long long batches;
        double kernel_ms;
        long long events;
        size_t budget_used;
};
int gpumas_engine_stats(const struct gpumas_engine * engine,
    struct gpumas_engine_stats * stats);

/** Engine statistics of the last transport call on this context. */
struct gpumas_stats {
        /** Kernel launches of the call. */
        int launches;
        /** Total device time of the transport kernels, in ms. */
        double kernel_ms;
};
int gpumas_context_stats(
    const struct gpumas_context * context, struct gpumas_stats * stats);

/* ------------------------------------------------------------------------ */
/* Errors.                                                                  */
/* ------------------------------------------------------------------------ */

/** A library function, as given to an error handler (pumas_function_t,
 * pumas.h:519). */
typedef void gpumas_function_t(void);

/** An error handler (pumas_handler_cb, pumas.h:532-533): the return code,
 * the library function that returned it and a message. */
typedef void gpumas_handler_cb(
    int rc, gpumas_function_t * caller, const char * message);

/**
 * Set or clear the error handler (pumas_error_handler_set, pumas.h:1133).
 * Every function of this header that returns a code other than
 * GPUMAS_RETURN_SUCCESS calls the handler, if one is set, with that code,
 * then returns the code. Unlike the reference, whose default handler
 * prints the error and exits the process (pumas.c:871-889), this library
 * has no handler until one is set and never exits. The handler is shared
 * by all threads; setting it is not thread safe.
 */
void gpumas_error_handler_set(gpumas_handler_cb * handler);

/** The current error handler, NULL if none (pumas_error_handler_get,
 * pumas.h:1144). */
gpumas_handler_cb * gpumas_error_handler_get(void);

/**
 * Catch errors (pumas_error_catch, pumas.h:1163): with a non-zero `enable`,
 * the following errors do not call the handler; the first one is recorded
 * until gpumas_error_raise. With 0, catching stops without raising.
 */
void gpumas_error_catch(int enable);

/**
 * Raise a caught error (pumas_error_raise, pumas.h:1184): returns the code
 * of the first error caught since gpumas_error_catch, or
 * GPUMAS_RETURN_SUCCESS, and calls the handler with it if one is set.
 * Catching stops. Without a previous gpumas_error_catch, returns (and
 * reports) GPUMAS_RETURN_RAISE_ERROR.
 */
int gpumas_error_raise(void);

/** The name of a library function given to an error handler, or NULL
 * (pumas_error_function, pumas.h:1120). */
const char * gpumas_error_function(gpumas_function_t * function);

/* ------------------------------------------------------------------------ */
/* Diagnostics.                                                             */
/* ------------------------------------------------------------------------ */

/** Measured FP64 fused multiply-add throughput of the current device, in
 * TFLOP/s (2 flops per DFMA), from a register-resident microbenchmark. It
 * is the denominator of the engine's FP64 roofline. */
int gpumas_bench_dfma(double * tflops);

/** Evaluate the engine's double precision logarithm (fn = 0) or
 * exponential (fn = 1) on the device for n arguments (for checking; they
 * replace the CUDA library functions in the transport, see gp_math.cuh).
 * fn = 2 evaluates the single precision screen of thinned candidates,
 * gp_neglog_beyond(u, p, q, r), for n quadruples x[4 i] .. x[4 i + 3]:
 * y[i] is 1 when it rules the candidate out, else 0. fn = 3 and fn = 4
 * evaluate the single precision logarithm and exponential of the DCS
 * interpolation (gp_libmf.cuh: the build host C library's logf and expf on
 * the DCS domains) at (float)x[i]. */
int gpumas_math_eval(int fn, size_t n, const double * x, double * y);

/* ------------------------------------------------------------------------ */
/* Random stream.                                                           */
/* ------------------------------------------------------------------------ */

/** Fill `out` with draws first .. first + n - 1 of the stream of
 * (seed, domain, event), computed on the device (for checking). */
int gpumas_random_fill(uint64_t seed, uint32_t domain, uint64_t event,
    uint64_t first, size_t n, double * out);

#ifdef __cplusplus
}
#endif
#endif /* GPUMAS_H */

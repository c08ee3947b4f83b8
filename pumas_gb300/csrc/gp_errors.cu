/*
 * gp_errors.cu -- error reporting of the C ABI: the error handler, catch and
 * raise of the reference (pumas_error_handler_set, pumas_error_catch,
 * pumas_error_raise, pumas_error_function; pumas.h:1110-1184,
 * pumas.c:2210-2326), without an exit.
 *
 * Every int returning entry point of gpumas.h is defined here as a call of
 * its implementation (gp_api_*, in gp_physics.cu, gp_transport.cu and
 * gp_batch.cu) whose code goes through gp_report: a code other than
 * GPUMAS_RETURN_SUCCESS calls the installed handler, or is recorded while
 * errors are caught, and is returned unchanged. Implementations call each
 * other directly, so that one failing call reports once.
 */
#include <stdio.h>

#include "gpumas.h"

/* The error handling state: shared by all threads, as the reference's. */
static gpumas_handler_cb * gp_handler = NULL;
static int gp_catch = 0;
static int gp_caught_code = GPUMAS_RETURN_SUCCESS;
static gpumas_function_t * gp_caught_function = NULL;

/* Name of a return code (enum pumas_return, pumas.h:143-196). */
static const char * gp_code_name(int rc)
{
        static const char * names[] = { "SUCCESS", "ACCURACY_ERROR",
                "END_OF_FILE", "DECAY_ERROR", "DENSITY_ERROR",
                "DIRECTION_ERROR", "INCOMPLETE_FILE", "INDEX_ERROR",
                "PHYSICS_ERROR", "INTERNAL_ERROR", "IO_ERROR", "FORMAT_ERROR",
                "MEDIUM_ERROR", "MEMORY_ERROR", "MODEL_ERROR",
                "MISSING_LIMIT", "MISSING_RANDOM", "PATH_ERROR",
                "RAISE_ERROR", "TOO_LONG", "UNDEFINED_MDF",
                "UNKNOWN_ELEMENT", "UNKNOWN_MATERIAL", "UNKNOWN_PARTICLE",
                "VALUE_ERROR" };
        if ((rc >= 0) && (rc < (int)(sizeof(names) / sizeof(*names))))
                return names[rc];
        if (rc == GPUMAS_RETURN_DEVICE_ERROR) return "DEVICE_ERROR";
        return "UNKNOWN";
}

/* Report a code of `caller`: handler or catch, then the code itself. */
static int gp_report(int rc, gpumas_function_t * caller)
{
        if (rc == GPUMAS_RETURN_SUCCESS) return rc;
        if (gp_catch) {
                if (gp_caught_code == GPUMAS_RETURN_SUCCESS) {
                        gp_caught_code = rc;
                        gp_caught_function = caller;
                }
                return rc;
        }
        if (gp_handler != NULL) {
                char message[160];
                snprintf(message, sizeof(message), "%s returned "
                    "GPUMAS_RETURN_%s (%d)", gpumas_error_function(caller),
                    gp_code_name(rc), rc);
                gp_handler(rc, caller, message);
        }
        return rc;
}

extern "C" void gpumas_error_handler_set(gpumas_handler_cb * handler)
{
        gp_handler = handler;
}

extern "C" gpumas_handler_cb * gpumas_error_handler_get(void)
{
        return gp_handler;
}

extern "C" void gpumas_error_catch(int enable)
{
        gp_catch = (enable != 0);
        if (gp_catch) {
                gp_caught_code = GPUMAS_RETURN_SUCCESS;
                gp_caught_function = NULL;
        }
}

extern "C" int gpumas_error_raise(void)
{
        if (!gp_catch)
                return gp_report(GPUMAS_RETURN_RAISE_ERROR,
                    (gpumas_function_t *)&gpumas_error_raise);
        gp_catch = 0;
        return gp_report(gp_caught_code, gp_caught_function);
}

/* Implementations (gp_physics.cu, gp_transport.cu, gp_batch.cu). */
extern "C" {
int gp_api_physics_load(struct gpumas_physics ** physics, const void * dump,
    size_t size);
int gp_api_physics_upload(struct gpumas_physics ** physics,
    const void * pumas_physics);
int gp_api_physics_material_index(const struct gpumas_physics * physics,
    const char * name, int * index);
int gp_api_physics_info(const struct gpumas_physics * physics,
    int * n_materials, int * n_elements, double * cutoff, double * mass);
int gp_api_physics_tabulate(const struct gpumas_physics * physics,
    double * csn, double * csn_dk, float * dcs, float * alpha, float * ms);
int gp_api_physics_particle(const struct gpumas_physics * physics,
    int * particle, double * lifetime, double * mass);
int gp_api_context_create(struct gpumas_context ** context,
    const struct gpumas_physics * physics, int extra_memory);
int gp_api_context_random_seed_set(struct gpumas_context * context,
    const uint64_t * seed);
int gp_api_context_random_seed_get(const struct gpumas_context * context,
    uint64_t * seed);
int gp_api_context_geometry_set(struct gpumas_context * context,
    const struct gpumas_geometry * geometry);
int gp_api_context_transport(struct gpumas_context * context, size_t n,
    struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event);
int gp_api_context_transport_device(struct gpumas_context * context, size_t n,
    const struct gpumas_soa * events, uint64_t first_event, void * stream);
int gp_api_context_recorder_set(struct gpumas_context * context,
    const struct gpumas_recorder * recorder);
int gp_api_context_tuning_set(struct gpumas_context * context,
    const struct gpumas_tuning * tuning);
int gp_api_context_tuning_get(const struct gpumas_context * context,
    struct gpumas_tuning * tuning);
int gp_api_context_trials_set(struct gpumas_context * context, int max_trials);
int gp_api_context_trials_get(const struct gpumas_context * context,
    int * max_trials);
int gp_api_context_carry_set(struct gpumas_context * context, int carry);
int gp_api_context_carry_get(const struct gpumas_context * context,
    int * carry);
int gp_api_context_transport_device_static(struct gpumas_context * context,
    size_t n, const struct gpumas_soa * events, uint64_t first_event,
    int pool_slots, void * stream);
int gp_api_engine_create(struct gpumas_engine ** engine,
    const struct gpumas_physics * physics, const struct gpumas_tuning * tuning,
    int max_jobs, size_t state_budget);
int gp_api_engine_submit(struct gpumas_engine * engine,
    const struct gpumas_job * job, int * ticket);
int gp_api_engine_submit_host(struct gpumas_engine * engine,
    const struct gpumas_context * context, size_t n,
    struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event, int * ticket);
int gp_api_engine_step(struct gpumas_engine * engine, int max_done, int * done,
    int * n_done, int * pending);
int gp_api_engine_run(struct gpumas_engine * engine, size_t n_jobs,
    const struct gpumas_job * jobs);
int gp_api_engine_stats(const struct gpumas_engine * engine,
    struct gpumas_engine_stats * stats);
int gp_api_context_stats(const struct gpumas_context * context,
    struct gpumas_stats * stats);
int gp_api_bench_dfma(double * tflops);
int gp_api_math_eval(int fn, size_t n, const double * x, double * y);
int gp_api_random_fill(uint64_t seed, uint32_t domain, uint64_t event,
    uint64_t first, size_t n, double * out);
}

extern "C" const char * gpumas_error_function(gpumas_function_t * function)
{
#define GP_NAME(f)                                                            \
        if (function == (gpumas_function_t *)&f) return #f;
        GP_NAME(gpumas_error_raise)
        GP_NAME(gpumas_physics_load)
        GP_NAME(gpumas_physics_upload)
        GP_NAME(gpumas_physics_material_index)
        GP_NAME(gpumas_physics_info)
        GP_NAME(gpumas_physics_particle)
        GP_NAME(gpumas_physics_tabulate)
        GP_NAME(gpumas_context_create)
        GP_NAME(gpumas_context_random_seed_set)
        GP_NAME(gpumas_context_random_seed_get)
        GP_NAME(gpumas_context_geometry_set)
        GP_NAME(gpumas_context_transport)
        GP_NAME(gpumas_context_transport_device)
        GP_NAME(gpumas_context_recorder_set)
        GP_NAME(gpumas_context_tuning_set)
        GP_NAME(gpumas_context_tuning_get)
        GP_NAME(gpumas_context_trials_set)
        GP_NAME(gpumas_context_trials_get)
        GP_NAME(gpumas_context_carry_set)
        GP_NAME(gpumas_context_carry_get)
        GP_NAME(gpumas_context_transport_device_static)
        GP_NAME(gpumas_engine_create)
        GP_NAME(gpumas_engine_submit)
        GP_NAME(gpumas_engine_submit_host)
        GP_NAME(gpumas_engine_step)
        GP_NAME(gpumas_engine_run)
        GP_NAME(gpumas_engine_stats)
        GP_NAME(gpumas_context_stats)
        GP_NAME(gpumas_bench_dfma)
        GP_NAME(gpumas_math_eval)
        GP_NAME(gpumas_random_fill)
#undef GP_NAME
        return NULL;
}

extern "C" int gpumas_physics_load(struct gpumas_physics ** physics,
    const void * dump, size_t size)
{
        return gp_report(gp_api_physics_load(physics, dump, size),
            (gpumas_function_t *)&gpumas_physics_load);
}

extern "C" int gpumas_physics_upload(struct gpumas_physics ** physics,
    const void * pumas_physics)
{
        return gp_report(gp_api_physics_upload(physics, pumas_physics),
            (gpumas_function_t *)&gpumas_physics_upload);
}

extern "C" int gpumas_physics_material_index(
    const struct gpumas_physics * physics, const char * name, int * index)
{
        return gp_report(gp_api_physics_material_index(physics, name, index),
            (gpumas_function_t *)&gpumas_physics_material_index);
}

extern "C" int gpumas_physics_info(const struct gpumas_physics * physics,
    int * n_materials, int * n_elements, double * cutoff, double * mass)
{
        return gp_report(gp_api_physics_info(
            physics, n_materials, n_elements, cutoff, mass),
            (gpumas_function_t *)&gpumas_physics_info);
}

extern "C" int gpumas_physics_particle(const struct gpumas_physics * physics,
    int * particle, double * lifetime, double * mass)
{
        return gp_report(gp_api_physics_particle(
            physics, particle, lifetime, mass),
            (gpumas_function_t *)&gpumas_physics_particle);
}

extern "C" int gpumas_context_create(struct gpumas_context ** context,
    const struct gpumas_physics * physics, int extra_memory)
{
        return gp_report(gp_api_context_create(context, physics, extra_memory),
            (gpumas_function_t *)&gpumas_context_create);
}

extern "C" int gpumas_context_random_seed_set(struct gpumas_context * context,
    const uint64_t * seed)
{
        return gp_report(gp_api_context_random_seed_set(context, seed),
            (gpumas_function_t *)&gpumas_context_random_seed_set);
}

extern "C" int gpumas_context_random_seed_get(
    const struct gpumas_context * context, uint64_t * seed)
{
        return gp_report(gp_api_context_random_seed_get(context, seed),
            (gpumas_function_t *)&gpumas_context_random_seed_get);
}

extern "C" int gpumas_context_geometry_set(struct gpumas_context * context,
    const struct gpumas_geometry * geometry)
{
        return gp_report(gp_api_context_geometry_set(context, geometry),
            (gpumas_function_t *)&gpumas_context_geometry_set);
}

extern "C" int gpumas_context_transport(struct gpumas_context * context,
    size_t n, struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event)
{
        return gp_report(gp_api_context_transport(
            context, n, states, results, first_event),
            (gpumas_function_t *)&gpumas_context_transport);
}

extern "C" int gpumas_context_transport_device(struct gpumas_context * context,
    size_t n, const struct gpumas_soa * events, uint64_t first_event,
    void * stream)
{
        return gp_report(gp_api_context_transport_device(
            context, n, events, first_event, stream),
            (gpumas_function_t *)&gpumas_context_transport_device);
}

extern "C" int gpumas_context_recorder_set(struct gpumas_context * context,
    const struct gpumas_recorder * recorder)
{
        return gp_report(gp_api_context_recorder_set(context, recorder),
            (gpumas_function_t *)&gpumas_context_recorder_set);
}

extern "C" int gpumas_context_tuning_set(struct gpumas_context * context,
    const struct gpumas_tuning * tuning)
{
        return gp_report(gp_api_context_tuning_set(context, tuning),
            (gpumas_function_t *)&gpumas_context_tuning_set);
}

extern "C" int gpumas_context_tuning_get(const struct gpumas_context * context,
    struct gpumas_tuning * tuning)
{
        return gp_report(gp_api_context_tuning_get(context, tuning),
            (gpumas_function_t *)&gpumas_context_tuning_get);
}

extern "C" int gpumas_context_trials_set(struct gpumas_context * context,
    int max_trials)
{
        return gp_report(gp_api_context_trials_set(context, max_trials),
            (gpumas_function_t *)&gpumas_context_trials_set);
}

extern "C" int gpumas_context_trials_get(const struct gpumas_context * context,
    int * max_trials)
{
        return gp_report(gp_api_context_trials_get(context, max_trials),
            (gpumas_function_t *)&gpumas_context_trials_get);
}

extern "C" int gpumas_context_carry_set(struct gpumas_context * context,
    int carry)
{
        return gp_report(gp_api_context_carry_set(context, carry),
            (gpumas_function_t *)&gpumas_context_carry_set);
}

extern "C" int gpumas_context_carry_get(const struct gpumas_context * context,
    int * carry)
{
        return gp_report(gp_api_context_carry_get(context, carry),
            (gpumas_function_t *)&gpumas_context_carry_get);
}

extern "C" int gpumas_context_transport_device_static(
    struct gpumas_context * context, size_t n,
    const struct gpumas_soa * events, uint64_t first_event, int pool_slots,
    void * stream)
{
        return gp_report(gp_api_context_transport_device_static(
            context, n, events, first_event, pool_slots, stream),
            (gpumas_function_t *)&gpumas_context_transport_device_static);
}

extern "C" int gpumas_engine_create(struct gpumas_engine ** engine,
    const struct gpumas_physics * physics, const struct gpumas_tuning * tuning,
    int max_jobs, size_t state_budget)
{
        return gp_report(gp_api_engine_create(
            engine, physics, tuning, max_jobs, state_budget),
            (gpumas_function_t *)&gpumas_engine_create);
}

extern "C" int gpumas_engine_submit(struct gpumas_engine * engine,
    const struct gpumas_job * job, int * ticket)
{
        return gp_report(gp_api_engine_submit(engine, job, ticket),
            (gpumas_function_t *)&gpumas_engine_submit);
}

extern "C" int gpumas_engine_submit_host(struct gpumas_engine * engine,
    const struct gpumas_context * context, size_t n,
    struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event, int * ticket)
{
        return gp_report(gp_api_engine_submit_host(
            engine, context, n, states, results, first_event, ticket),
            (gpumas_function_t *)&gpumas_engine_submit_host);
}

extern "C" int gpumas_engine_step(struct gpumas_engine * engine, int max_done,
    int * done, int * n_done, int * pending)
{
        return gp_report(gp_api_engine_step(
            engine, max_done, done, n_done, pending),
            (gpumas_function_t *)&gpumas_engine_step);
}

extern "C" int gpumas_engine_run(struct gpumas_engine * engine, size_t n_jobs,
    const struct gpumas_job * jobs)
{
        return gp_report(gp_api_engine_run(engine, n_jobs, jobs),
            (gpumas_function_t *)&gpumas_engine_run);
}

extern "C" int gpumas_engine_stats(const struct gpumas_engine * engine,
    struct gpumas_engine_stats * stats)
{
        return gp_report(gp_api_engine_stats(engine, stats),
            (gpumas_function_t *)&gpumas_engine_stats);
}

extern "C" int gpumas_context_stats(const struct gpumas_context * context,
    struct gpumas_stats * stats)
{
        return gp_report(gp_api_context_stats(context, stats),
            (gpumas_function_t *)&gpumas_context_stats);
}

extern "C" int gpumas_bench_dfma(double * tflops)
{
        return gp_report(gp_api_bench_dfma(tflops),
            (gpumas_function_t *)&gpumas_bench_dfma);
}

extern "C" int gpumas_math_eval(int fn, size_t n, const double * x, double * y)
{
        return gp_report(gp_api_math_eval(fn, n, x, y),
            (gpumas_function_t *)&gpumas_math_eval);
}

extern "C" int gpumas_random_fill(uint64_t seed, uint32_t domain,
    uint64_t event, uint64_t first, size_t n, double * out)
{
        return gp_report(gp_api_random_fill(seed, domain, event, first, n, out),
            (gpumas_function_t *)&gpumas_random_fill);
}

extern "C" int gpumas_physics_tabulate(const struct gpumas_physics * physics,
    double * csn, double * csn_dk, float * dcs, float * alpha, float * ms)
{
        return gp_report(gp_api_physics_tabulate(physics, csn, csn_dk, dcs,
                             alpha, ms),
            (gpumas_function_t *)&gpumas_physics_tabulate);
}

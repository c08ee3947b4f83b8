/*
 * gp_io.cuh -- event input / output of the transport kernels: an array of
 * pumas_state records (with per event results) or a structure of arrays.
 */
#ifndef GP_IO_CUH
#define GP_IO_CUH

#include "gp_device.cuh"

/* ------------------------------------------------------------------------ */
/* Event I/O: array of pumas_state structures or structure of arrays.       */
/* ------------------------------------------------------------------------ */
/* Per event results, with the random state that a following call of a
 * carrying context continues. */
__device__ __forceinline__ void gp_result_store(gpumas_result & out,
    const gp_event & e, int event, int m_in, int m_out)
{
        gpumas_result r;
        r.event = event;
        r.medium_in = m_in;
        r.medium_out = m_out;
        r.status = e.status;
        r.steps = e.steps;
        r.randn_done = e.randn_done;
        r.draws = e.n;
        r.randn_next = e.randn_next;
        out = r;
}

struct gp_io_aos {
        gpumas_state * states;
        gpumas_result * results;
        __device__ void load(size_t i, gp_event & e) const
        {
                const gpumas_state & s = states[i];
                e.charge = s.charge;
                e.energy = s.energy;
                e.distance = s.distance;
                e.grammage = s.grammage;
                e.time = s.time;
                e.weight = s.weight;
                for (int k = 0; k < 3; k++) {
                        e.pos[k] = s.position[k];
                        e.dir[k] = s.direction[k];
                }
                e.decayed = s.decayed;
        }
        __device__ void store(size_t i, const gp_event & e, int event,
            int m_in, int m_out) const
        {
                gpumas_state & s = states[i];
                s.charge = e.charge;
                s.energy = e.energy;
                s.distance = e.distance;
                s.grammage = e.grammage;
                s.time = e.time;
                s.weight = e.weight;
                for (int k = 0; k < 3; k++) {
                        s.position[k] = e.pos[k];
                        s.direction[k] = e.dir[k];
                }
                s.decayed = e.decayed;
                if (results != NULL) gp_result_store(results[i], e, event,
                    m_in, m_out);
        }
        __device__ void load_carry(size_t i, gp_event & e) const
        {
                const gpumas_result & r = results[i];
                gp_event_carry(e, r.draws, r.randn_done, r.randn_next);
        }
};

struct gp_io_soa {
        gpumas_soa a;
        __device__ void load(size_t i, gp_event & e) const
        {
                e.charge = a.charge[i];
                e.energy = a.energy[i];
                e.distance = a.distance[i];
                e.grammage = a.grammage[i];
                e.time = a.time[i];
                e.weight = a.weight[i];
                for (int k = 0; k < 3; k++) {
                        e.pos[k] = a.position[k][i];
                        e.dir[k] = a.direction[k][i];
                }
                e.decayed = a.decayed[i];
        }
        __device__ void store(size_t i, const gp_event & e, int event,
            int m_in, int m_out) const
        {
                a.charge[i] = e.charge;
                a.energy[i] = e.energy;
                a.distance[i] = e.distance;
                a.grammage[i] = e.grammage;
                a.time[i] = e.time;
                a.weight[i] = e.weight;
                for (int k = 0; k < 3; k++) {
                        a.position[k][i] = e.pos[k];
                        a.direction[k][i] = e.dir[k];
                }
                a.decayed[i] = e.decayed;
                if (a.result != NULL) gp_result_store(a.result[i], e, event,
                    m_in, m_out);
        }
        __device__ void load_carry(size_t i, gp_event & e) const
        {
                const gpumas_result & r = a.result[i];
                gp_event_carry(e, r.draws, r.randn_done, r.randn_next);
        }
};


/* Event I/O of a launch: AoS (pumas_state array) when `aos.states` is set,
 * SoA otherwise. */
struct gp_io {
        gp_io_aos aos;
        gp_io_soa soa;
        __device__ void load(size_t i, gp_event & e) const
        {
                if (aos.states != NULL)
                        aos.load(i, e);
                else
                        soa.load(i, e);
        }
        __device__ void store(size_t i, const gp_event & e, int event,
            int m_in, int m_out) const
        {
                if (aos.states != NULL)
                        aos.store(i, e, event, m_in, m_out);
                else
                        soa.store(i, e, event, m_in, m_out);
        }
        /* Start event i's stream where its previous call left it. */
        __device__ void load_carry(size_t i, gp_event & e) const
        {
                if (aos.states != NULL)
                        aos.load_carry(i, e);
                else
                        soa.load_carry(i, e);
        }
        /* An event's setup for a call: state, stream and, when the config
         * carries, the random state of its previous call. */
        __device__ void begin(size_t i, const gp_config & cfg, uint64_t id,
            gp_event & e) const
        {
                load(i, e);
                gp_event_init(e, cfg.seed, id);
                if (cfg.carry) load_carry(i, e);
        }
};

#endif

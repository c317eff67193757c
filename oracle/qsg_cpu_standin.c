/*
 * qsg_cpu_standin.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU stand-in for the handful of libqsg tracking calls the reference-side
 * adapter makes (oracle/dropin_adapter.hh: qsgAttach / qsgCycleTracking),
 * answered by the C oracle (qs_oracle.c), so that the adapter can drive the
 * reference's own main loop on a machine without a GPU
 * (oracle/dropin_cycle.cc, `make -C oracle dropin_cycle`).  It checks the
 * adapter's glue -- vaults in, census out, tallies into the reference's
 * Tallies -- not the library: the GPU tests show the library's tracking is
 * the oracle's.  Never linked into libqsg.so or loaded from Python.
 *
 * Differences from the library, none of which the adapter relies on: the
 * problem passed to qsg_create is kept by pointer (the library copies it to
 * the device), options other than none are ignored, and only the calls below
 * exist.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "qs_oracle.h"

struct QsgHandle {
    const QsgProblem* problem;
    OracleParticle* in;
    uint64_t n_in;
    OracleParticle* census;
    uint64_t n_census;
    uint64_t balance[QSG_BAL_COUNT];
    double* flux;
    double* cell_tally;   /* NULL unless qsg_set_exponential_tally turned it on */
};

static char g_error[512];

static int fail(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof g_error, fmt, ap);
    va_end(ap);
    return code;
}

static size_t flux_size(const QsgHandle* h)
{
    return (size_t)h->problem->num_cells * (size_t)h->problem->num_groups;
}

int qsg_last_error(char* buf, size_t len)
{
    if (buf && len) snprintf(buf, len, "%s", g_error);
    return QSG_OK;
}

int qsg_create(const QsgProblem* problem, const QsgOptions* options, QsgHandle** out)
{
    (void)options;
    if (!problem || !out) return fail(QSG_ERR_INVALID, "qsg_create: null argument");
    QsgHandle* h = (QsgHandle*)calloc(1, sizeof *h);
    if (!h) return fail(QSG_ERR_CAPACITY, "qsg_create: out of host memory");
    h->problem = problem;
    h->flux = (double*)calloc(flux_size(h) ? flux_size(h) : 1, sizeof(double));
    if (!h->flux) { free(h); return fail(QSG_ERR_CAPACITY, "qsg_create: out of host memory"); }
    *out = h;
    return QSG_OK;
}

int qsg_destroy(QsgHandle* h)
{
    if (h) { free(h->in); free(h->census); free(h->flux); free(h->cell_tally); free(h); }
    return QSG_OK;
}

int qsg_set_particles(QsgHandle* h, const QsgParticleSoA* s, uint64_t n)
{
    if (!h || (n && !s)) return fail(QSG_ERR_INVALID, "qsg_set_particles: null argument");
    OracleParticle* p = (OracleParticle*)realloc(h->in, (n ? n : 1) * sizeof *p);
    if (!p) return fail(QSG_ERR_CAPACITY, "qsg_set_particles: out of host memory");
    h->in = p;
    for (uint64_t k = 0; k < n; ++k) {
        OracleParticle r = {s->x[k], s->y[k], s->z[k], s->vx[k], s->vy[k], s->vz[k], s->kinetic_energy[k],
                            s->weight[k], s->time_to_census[k], s->age[k], s->num_mean_free_paths[k],
                            s->num_segments[k], s->random_number_seed[k], s->identifier[k], s->last_event[k],
                            s->num_collisions[k], s->breed[k], s->species[k], s->domain[k], s->cell[k]};
        p[k] = r;
    }
    h->n_in = n;
    h->n_census = 0;
    return QSG_OK;
}

/* The processing particles tracked to census, fission products included;
 * counters and flux accumulate until qsg_reset_tallies. */
int qsg_track_cycle_sync(QsgHandle* h)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_track_cycle_sync: null handle");
    const size_t nf = flux_size(h);
    double* flux = (double*)malloc((nf ? nf : 1) * sizeof(double));
    if (!flux) return fail(QSG_ERR_CAPACITY, "qsg_track_cycle_sync: out of host memory");
    uint64_t cap = 4 * h->n_in + 1024;
    for (;;) {
        OracleParticle* census = (OracleParticle*)malloc(cap * sizeof *census);
        if (!census) { free(flux); return fail(QSG_ERR_CAPACITY, "qsg_track_cycle_sync: out of host memory"); }
        uint64_t bal[QSG_BAL_COUNT] = {0}, n_census = 0;
        memset(flux, 0, (nf ? nf : 1) * sizeof(double));
        const size_t nc = h->cell_tally ? (size_t)h->problem->num_cells : 0;
        double* cell = nc ? (double*)calloc(nc, sizeof(double)) : NULL;
        if (nc && !cell) { free(census); free(flux); return fail(QSG_ERR_CAPACITY, "out of host memory"); }
        const int rc = oracle_track_cell_tally(h->problem, h->in, h->n_in, census, cap, &n_census, bal, flux, cell, 8);
        for (size_t k = 0; k < nc && rc == 0; ++k) h->cell_tally[k] += cell[k];
        free(cell);
        if (rc == -3) {   /* fission grew the census past its room: again, with room for all of it */
            free(census);
            cap = n_census + 16;
            continue;
        }
        if (rc != 0) { free(census); free(flux); return fail(QSG_ERR_DEVICE, "oracle_track returned %d", rc); }
        free(h->census);
        h->census = census;
        h->n_census = n_census;
        h->n_in = 0;
        for (int k = 0; k < QSG_BAL_COUNT; ++k) h->balance[k] += bal[k];
        for (size_t k = 0; k < nf; ++k) h->flux[k] += flux[k];
        free(flux);
        return QSG_OK;
    }
}

int qsg_sizes(QsgHandle* h, uint64_t* processing, uint64_t* processed)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_sizes: null handle");
    if (processing) *processing = h->n_in;
    if (processed) *processed = h->n_census;
    return QSG_OK;
}

int qsg_get_census(QsgHandle* h, QsgParticleSoA* s, uint64_t cap, uint64_t* n_out)
{
    if (!h || !s || !n_out) return fail(QSG_ERR_INVALID, "qsg_get_census: null argument");
    const uint64_t n = h->n_census < cap ? h->n_census : cap;
    for (uint64_t k = 0; k < n; ++k) {
        const OracleParticle* r = &h->census[k];
        s->x[k] = r->x; s->y[k] = r->y; s->z[k] = r->z;
        s->vx[k] = r->vx; s->vy[k] = r->vy; s->vz[k] = r->vz;
        s->kinetic_energy[k] = r->kinetic_energy; s->weight[k] = r->weight;
        s->time_to_census[k] = r->time_to_census; s->age[k] = r->age;
        s->num_mean_free_paths[k] = r->num_mean_free_paths; s->num_segments[k] = r->num_segments;
        s->random_number_seed[k] = r->random_number_seed; s->identifier[k] = r->identifier;
        s->last_event[k] = r->last_event; s->num_collisions[k] = r->num_collisions; s->breed[k] = r->breed;
        s->species[k] = r->species; s->domain[k] = r->domain; s->cell[k] = r->cell;
    }
    *n_out = n;
    return h->n_census > cap ? fail(QSG_ERR_CAPACITY, "qsg_get_census: %llu census particles, room for %llu",
                                    (unsigned long long)h->n_census, (unsigned long long)cap)
                             : QSG_OK;
}

int qsg_read_tallies(QsgHandle* h, uint64_t* balance, double* flux)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_read_tallies: null handle");
    if (balance) memcpy(balance, h->balance, sizeof h->balance);
    if (flux) memcpy(flux, h->flux, flux_size(h) * sizeof(double));
    return QSG_OK;
}

int qsg_reset_tallies(QsgHandle* h)
{
    if (!h) return fail(QSG_ERR_INVALID, "qsg_reset_tallies: null handle");
    memset(h->balance, 0, sizeof h->balance);
    memset(h->flux, 0, flux_size(h) * sizeof(double));
    if (h->cell_tally) memset(h->cell_tally, 0, (size_t)h->problem->num_cells * sizeof(double));
    return QSG_OK;
}

/* The -DEXPONENTIAL_TALLY build's draw and cell tally (oracle_track_cell_tally). */
int qsg_set_exponential_tally(QsgHandle* h, int32_t enabled)
{
    if (!h || (enabled != 0 && enabled != 1)) return fail(QSG_ERR_INVALID, "qsg_set_exponential_tally: bad argument");
    free(h->cell_tally);
    h->cell_tally = enabled ? (double*)calloc((size_t)h->problem->num_cells + 1, sizeof(double)) : NULL;
    return enabled && !h->cell_tally ? fail(QSG_ERR_CAPACITY, "out of host memory") : QSG_OK;
}

int qsg_read_cell_tally(QsgHandle* h, double* cell_tally)
{
    if (!h || !cell_tally) return fail(QSG_ERR_INVALID, "qsg_read_cell_tally: null argument");
    if (!h->cell_tally) return fail(QSG_ERR_INVALID, "qsg_read_cell_tally: the exponential tally is off");
    memcpy(cell_tally, h->cell_tally, (size_t)h->problem->num_cells * sizeof(double));
    return QSG_OK;
}

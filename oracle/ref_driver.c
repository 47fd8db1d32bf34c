/* ref_driver.c -- thin C driver over the reference's own tracking code.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file against
 * the reference's header-only hot path (sixtracklib/common/track/track.h,
 * the be_* maps, the CObjects managed-buffer helpers) into
 * oracle/_ref/libstref.so.  It exposes the same signatures as oracle.h with
 * a "ref_" prefix so tests can run both on identical inputs.  Nothing here
 * is part of the product; the reference sources stay where they lie.
 */
#include "sixtracklib/common/definitions.h"
#include "sixtracklib/common/track/track.h"
#include "sixtracklib/common/be_beamfields/gauss_fields.h"
#include "sixtracklib/common/be_beamfields/faddeeva_cern.h"
#include "sixtracklib/common/buffer/managed_buffer_remap.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct {
    unsigned char *mem;
    NS(Object) const *begin;
    NS(Object) const *end;
    NS(ParticlesGenericAddr) *mon_out; /* one per patched monitor */
} ref_lattice;

static void fill_generic(NS(ParticlesGenericAddr) *g, void *cols, int64_t n)
{
    uint64_t const base = (uint64_t)(uintptr_t)cols;
    uint64_t const stride = (uint64_t)n * 8u;
    g->num_particles = n;
    g->q0_addr = base + 0 * stride;
    g->mass0_addr = base + 1 * stride;
    g->beta0_addr = base + 2 * stride;
    g->gamma0_addr = base + 3 * stride;
    g->p0c_addr = base + 4 * stride;
    g->s_addr = base + 5 * stride;
    g->x_addr = base + 6 * stride;
    g->y_addr = base + 7 * stride;
    g->px_addr = base + 8 * stride;
    g->py_addr = base + 9 * stride;
    g->zeta_addr = base + 10 * stride;
    g->psigma_addr = base + 11 * stride;
    g->delta_addr = base + 12 * stride;
    g->rpp_addr = base + 13 * stride;
    g->rvv_addr = base + 14 * stride;
    g->chi_addr = base + 15 * stride;
    g->charge_ratio_addr = base + 16 * stride;
    g->particle_id_addr = base + 17 * stride;
    g->at_element_id_addr = base + 18 * stride;
    g->at_turn_addr = base + 19 * stride;
    g->state_addr = base + 20 * stride;
}

static int open_lattice(ref_lattice *L, const uint8_t *img,
                        const orc_monitor_outputs *mon)
{
    uint64_t const size = ((const uint64_t *)img)[1];
    L->mem = (unsigned char *)aligned_alloc(64, (size + 63) & ~(uint64_t)63);
    if (!L->mem) return -1;
    memcpy(L->mem, img, size);
    uint64_t const old_base = ((const uint64_t *)img)[0];
    if (NS(ManagedBuffer_remap)(L->mem, 8u) != 0) return -1;
    L->begin = NS(ManagedBuffer_get_const_objects_index_begin)(L->mem, 8u);
    L->end = NS(ManagedBuffer_get_const_objects_index_end)(L->mem, 8u);
    /* the interpolated space-charge element holds a plain address (no
     * dataptr; the reference's TrackJob assigns it): when it points into
     * this image, move it with the image, as the caller would */
    uint64_t const new_base = (uint64_t)(uintptr_t)L->mem;
    for (NS(Object) const *it = L->begin; it != L->end; ++it) {
        if (NS(Object_get_type_id)(it) == NS(OBJECT_TYPE_TRICUB)) {
            /* TriCub's data_addr likewise */
            NS(TriCub) *tc = (NS(TriCub) *)(uintptr_t)NS(Object_get_begin_addr)(it);
            if (tc->data_addr >= old_base && tc->data_addr < old_base + size)
                tc->data_addr = tc->data_addr - old_base + new_base;
            continue;
        }
        if (NS(Object_get_type_id)(it) != NS(OBJECT_TYPE_SC_INTERPOLATED_PROF)) continue;
        NS(SCInterpolatedProfile) *sc =
            (NS(SCInterpolatedProfile) *)(uintptr_t)NS(Object_get_begin_addr)(it);
        if (sc->interpol_data_addr >= old_base && sc->interpol_data_addr < old_base + size)
            sc->interpol_data_addr = sc->interpol_data_addr - old_base + new_base;
    }
    L->mon_out = NULL;
    if (mon && mon->num > 0) {
        L->mon_out = (NS(ParticlesGenericAddr) *)calloc(
            (size_t)mon->num, sizeof(NS(ParticlesGenericAddr)));
        int64_t k = 0;
        for (NS(Object) const *it = L->begin; it != L->end; ++it) {
            if (NS(Object_get_type_id)(it) != NS(OBJECT_TYPE_BEAM_MONITOR))
                continue;
            NS(BeamMonitor) *m =
                (NS(BeamMonitor) *)(uintptr_t)NS(Object_get_begin_addr)(it);
            if (m->out_address == 0) continue;
            if (k < mon->num) {
                fill_generic(&L->mon_out[k], mon->cols[k], mon->caps[k]);
                m->out_address = (uint64_t)(uintptr_t)&L->mon_out[k];
            }
            ++k;
        }
    }
    return 0;
}

static void close_lattice(ref_lattice *L)
{
    free(L->mem);
    free(L->mon_out);
}

static void make_particles(NS(Particles) *p, void *cols, int64_t n)
{
    double *d = (double *)cols;
    int64_t *k = (int64_t *)cols;
    p->num_particles = n;
    p->q0 = d + 0 * n;
    p->mass0 = d + 1 * n;
    p->beta0 = d + 2 * n;
    p->gamma0 = d + 3 * n;
    p->p0c = d + 4 * n;
    p->s = d + 5 * n;
    p->x = d + 6 * n;
    p->y = d + 7 * n;
    p->px = d + 8 * n;
    p->py = d + 9 * n;
    p->zeta = d + 10 * n;
    p->psigma = d + 11 * n;
    p->delta = d + 12 * n;
    p->rpp = d + 13 * n;
    p->rvv = d + 14 * n;
    p->chi = d + 15 * n;
    p->charge_ratio = d + 16 * n;
    p->particle_id = k + 17 * n;
    p->at_element_id = k + 18 * n;
    p->at_turn = k + 19 * n;
    p->state = k + 20 * n;
}

int32_t ref_track_until(const uint8_t *lattice, void *cols, int64_t n,
                        int64_t i0, int64_t i1, int64_t until_turn,
                        const orc_monitor_outputs *mon)
{
    ref_lattice L;
    NS(Particles) p;
    int32_t st = 0;
    if (open_lattice(&L, lattice, mon) != 0) return -1;
    make_particles(&p, cols, n);
#ifdef STG_REF_OMP
#pragma omp parallel for schedule(dynamic, 64) reduction(| : st)
#endif
    for (int64_t i = i0; i < i1; ++i)
        st |= NS(Track_particle_until_turn_objs)(&p, i, L.begin, L.end,
                                                 until_turn);
    close_lattice(&L);
    return st;
}

int32_t ref_track_line(const uint8_t *lattice, void *cols, int64_t n,
                       int64_t i0, int64_t i1, uint64_t lb, uint64_t le,
                       int finish_turn, const orc_monitor_outputs *mon)
{
    ref_lattice L;
    NS(Particles) p;
    int32_t st = 0;
    if (open_lattice(&L, lattice, mon) != 0) return -1;
    make_particles(&p, cols, n);
    for (int64_t i = i0; i < i1; ++i)
        st |= NS(Track_particle_line_objs)(&p, i, L.begin + lb, L.begin + le,
                                           finish_turn != 0);
    close_lattice(&L);
    return st;
}

int32_t ref_track_elem_by_elem(const uint8_t *lattice, void *cols, int64_t n,
                               int64_t i0, int64_t i1,
                               const orc_ebe_config *c, void *out_cols,
                               int64_t out_n, int64_t until_turn,
                               const orc_monitor_outputs *mon)
{
    ref_lattice L;
    NS(Particles) p;
    NS(ElemByElemConfig) cfg;
    NS(ParticlesGenericAddr) out;
    int32_t st = 0;
    if (open_lattice(&L, lattice, mon) != 0) return -1;
    make_particles(&p, cols, n);
    memset(&cfg, 0, sizeof(cfg));
    cfg.order = c->order;
    cfg.num_particles_to_store = c->num_particles_to_store;
    cfg.num_elements_to_store = c->num_elements_to_store;
    cfg.num_turns_to_store = c->num_turns_to_store;
    cfg.min_particle_id = c->min_particle_id;
    cfg.min_element_id = c->min_element_id;
    cfg.min_turn = c->min_turn;
    cfg.max_particle_id = c->max_particle_id;
    cfg.max_element_id = c->max_element_id;
    cfg.max_turn = c->max_turn;
    cfg.is_rolling = c->is_rolling;
    cfg.out_store_addr = 0;
    if (out_cols) {
        fill_generic(&out, out_cols, out_n);
        cfg.out_store_addr = (uint64_t)(uintptr_t)&out;
    }
    for (int64_t i = i0; i < i1; ++i)
        st |= NS(Track_particle_element_by_element_until_turn_objs)(
            &p, i, &cfg, L.begin, L.end, until_turn);
    close_lattice(&L);
    return st;
}

int64_t ref_ebe_store_index(const orc_ebe_config *c, int64_t pid,
                            int64_t at_element, int64_t at_turn)
{
    NS(ElemByElemConfig) cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.order = c->order;
    cfg.num_particles_to_store = c->num_particles_to_store;
    cfg.num_elements_to_store = c->num_elements_to_store;
    cfg.num_turns_to_store = c->num_turns_to_store;
    cfg.min_particle_id = c->min_particle_id;
    cfg.min_element_id = c->min_element_id;
    cfg.min_turn = c->min_turn;
    cfg.max_particle_id = c->max_particle_id;
    cfg.max_element_id = c->max_element_id;
    cfg.max_turn = c->max_turn;
    cfg.is_rolling = c->is_rolling;
    return NS(ElemByElemConfig_get_particles_store_index_details)(
        &cfg, pid, at_element, at_turn);
}

void ref_cerrf(double re, double im, double *wr, double *wi)
{
    cerrf(re, im, wr, wi);
}

void ref_fields_gauss(double x, double y, double sx, double sy, double msd,
                      int skip, double *ex, double *ey, double *gx, double *gy)
{
    NS(get_Ex_Ey_Gx_Gy_gauss)(x, y, sx, sy, msd, skip, ex, ey, gx, gy);
}

/* NS(BeamBeam6D_boost) / NS(BeamBeam6D_inv_boost) (be_beamfields.h:
 * 2101-2230) on one point: `boost` = (sphi, cphi, tphi, salpha, calpha) as
 * in NS(BB6D_boost_data), `c6` = (x, px, y, py, sigma, delta), in place. */
void ref_bb6d_boost(const double *boost, double *c6, int inverse)
{
    NS(BB6D_boost_data) b;
    b.sphi = boost[0];
    b.cphi = boost[1];
    b.tphi = boost[2];
    b.salpha = boost[3];
    b.calpha = boost[4];
    if (inverse)
        NS(BeamBeam6D_inv_boost)(&b, &c6[0], &c6[1], &c6[2], &c6[3], &c6[4], &c6[5]);
    else
        NS(BeamBeam6D_boost)(&b, &c6[0], &c6[1], &c6[2], &c6[3], &c6[4], &c6[5]);
}

/* NS(tricub_construct_coefs) (be_tricub/coefficients.h) on one cell's 64
 * corner values. */
void ref_tricub_coefs(const double *b, double *coefs)
{
    NS(tricub_construct_coefs)(b, coefs);
}

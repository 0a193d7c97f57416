/* bsacl_ref_driver.c -- TEST INFRASTRUCTURE ONLY (part of the parity oracle).
 *
 * Runs the reference's BsaCL Classic kernel (BsaCL/src/bsacl.cl, kernel 2: one work item per
 * frequency pair, one work group column per modal triple) on the host and reduces its
 * work-group partials the way the reference's host code does, giving the reference's own
 * m3mr for a set of frequency pairs.  Built by oracle/bsacl_ref.py from the kernel source
 * where it lies (BSACL_CL_SOURCE), after oracle/bsacl_shim.h; the problem sizes are the
 * kernel's compile-time macros (NTC__, NNL__, NM_EFF__, NN__, NFI__, NFJ__), as the reference
 * passes them to its OpenCL build (bsacl.c:740-790).
 *
 * Host side restated from bsacl.c (bsaclRun): the NDRange, nfi nfj / WIpWG + 1 work groups of
 * BSACL_WIpWG items along dimension 0 and NM^3 along dimension 1 (:1395-1410); the
 * integration weight dInfl = (fi[1] - fi[0]) (fj[1] - fj[0]) 4 pi^2 (:1362-1366); the output
 * h_res[i] = dInfl sum over work groups of m3out[wg + i nwg] (:1565-1572).
 */
#include <stdlib.h>
#include <string.h>

#include BSACL_CL_SOURCE

static __thread size_t t_gid0, t_lid0, t_grp0, t_grp1;
static size_t g_ngrp0;

size_t get_global_id(uint d) { return d == 0 ? t_gid0 : t_grp1; }
size_t get_local_id(uint d) { return d == 0 ? t_lid0 : 0; }
size_t get_group_id(uint d) { return d == 0 ? t_grp0 : t_grp1; }
size_t get_num_groups(uint d) { return d == 0 ? g_ngrp0 : (size_t)NM_EFF__ * NM_EFF__ * NM_EFF__; }

/* a barrier that work items leave when they return */
static pthread_mutex_t b_m = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t b_c = PTHREAD_COND_INITIALIZER;
static int b_expected, b_arrived;
static unsigned long b_gen;

void barrier(int flags) {
    (void)flags;
    pthread_mutex_lock(&b_m);
    if (++b_arrived == b_expected) {
        b_arrived = 0;
        ++b_gen;
        pthread_cond_broadcast(&b_c);
    } else {
        const unsigned long g = b_gen;
        while (g == b_gen) pthread_cond_wait(&b_c, &b_m);
    }
    pthread_mutex_unlock(&b_m);
}

static void barrier_leave(void) {
    pthread_mutex_lock(&b_m);
    --b_expected;
    if (b_arrived > 0 && b_arrived == b_expected) {
        b_arrived = 0;
        ++b_gen;
        pthread_cond_broadcast(&b_c);
    }
    pthread_mutex_unlock(&b_m);
}

typedef struct {
    const uint *tc, *nodes_load;
    const double *phiTc, *nod_corr, *u, *scl, *std;
    const int *winz;
    const double *Mg, *Cg, *Kg;
    double *fi, *fj, *m3out;
    size_t grp0, grp1, lid;
} item_t;

static void *work_item(void *p) {
    const item_t *a = (const item_t *)p;
    t_lid0 = a->lid;
    t_grp0 = a->grp0;
    t_grp1 = a->grp1;
    t_gid0 = a->grp0 * BSACL_WIpWG + a->lid;
    bfm_kernel(a->tc, a->nodes_load, a->phiTc, a->nod_corr, a->u, a->scl, a->std, a->winz, a->Mg, a->Cg, a->Kg,
               a->fi, a->fj, a->m3out);
    barrier_leave();
    return NULL;
}

/* Runs every work group of the NDRange; m3out[g + i nwg] receives work group g's partial of
 * modal triple i (the kernel's own output buffer). */
static int run_all(const uint *tc, const uint *nodes_load, const double *phiTc, const double *nod_corr,
                   const double *u, const double *scl, const double *std, const int *winz, const double *Mg,
                   const double *Cg, const double *Kg, double *fi, double *fj, double *m3out) {
    const size_t dim = (size_t)NM_EFF__ * NM_EFF__ * NM_EFF__;
    const size_t nwg = (size_t)(NFI__ * NFJ__) / BSACL_WIpWG + 1;
    g_ngrp0 = nwg;
    item_t it[BSACL_WIpWG];
    pthread_t th[BSACL_WIpWG];
    for (size_t g1 = 0; g1 < dim; ++g1)
        for (size_t g0 = 0; g0 < nwg; ++g0) {
            b_expected = BSACL_WIpWG;
            b_arrived = 0;
            int started = 0;
            for (int l = 0; l < BSACL_WIpWG; ++l) {
                item_t a = {tc, nodes_load, phiTc, nod_corr, u, scl, std, winz, Mg, Cg, Kg, fi, fj, m3out, g0, g1,
                            (size_t)l};
                it[l] = a;
                if (pthread_create(&th[l], NULL, work_item, &it[l])) break;
                ++started;
            }
            for (int l = started; l < BSACL_WIpWG; ++l) barrier_leave();  /* items never started */
            for (int l = 0; l < started; ++l) pthread_join(th[l], NULL);
            if (started < BSACL_WIpWG) return -2;
        }
    return 0;
}

/* m3mr (NM^3, the kernel's modal order) of the frequency pairs fi x fj (NFI__ x NFJ__). */
int bsacl_ref_run(const uint *tc, const uint *nodes_load, const double *phiTc, const double *nod_corr,
                  const double *u, const double *scl, const double *std, const int *winz, const double *Mg,
                  const double *Cg, const double *Kg, double *fi, double *fj, double *h_res) {
    const size_t dim = (size_t)NM_EFF__ * NM_EFF__ * NM_EFF__;
    const size_t nwg = (size_t)(NFI__ * NFJ__) / BSACL_WIpWG + 1;
    double *m3out = (double *)calloc(dim * nwg, sizeof(double));
    if (!m3out) return -1;
    const int rc = run_all(tc, nodes_load, phiTc, nod_corr, u, scl, std, winz, Mg, Cg, Kg, fi, fj, m3out);
    if (rc) {
        free(m3out);
        return rc;
    }
    double dinfl = (fi[1] - fi[0]) * (fj[1] - fj[0]) * 4.0 * (M_PI * M_PI);
    for (size_t i = 0; i < dim; ++i) {
        double s = 0.0;
        for (size_t g = 0; g < nwg; ++g) s += m3out[g + i * nwg];
        h_res[i] = s * dinfl;
    }
    free(m3out);
    return 0;
}

/* The kernel's per-work-group partials before the host reduction and weight:
 * groups[g dim + i] = sum over work group g's BSACL_WIpWG pairs (work item l of group g takes
 * pair p = g BSACL_WIpWG + l, fi[p % NFI__], fj[p / NFI__]) of the kernel's value for modal
 * triple i.  nwg = NFI__ NFJ__ / BSACL_WIpWG + 1 groups; pairs past the list contribute 0. */
int bsacl_ref_groups(const uint *tc, const uint *nodes_load, const double *phiTc, const double *nod_corr,
                     const double *u, const double *scl, const double *std, const int *winz, const double *Mg,
                     const double *Cg, const double *Kg, double *fi, double *fj, double *groups) {
    const size_t dim = (size_t)NM_EFF__ * NM_EFF__ * NM_EFF__;
    const size_t nwg = (size_t)(NFI__ * NFJ__) / BSACL_WIpWG + 1;
    double *m3out = (double *)calloc(dim * nwg, sizeof(double));
    if (!m3out) return -1;
    const int rc = run_all(tc, nodes_load, phiTc, nod_corr, u, scl, std, winz, Mg, Cg, Kg, fi, fj, m3out);
    if (!rc)
        for (size_t g = 0; g < nwg; ++g)
            for (size_t i = 0; i < dim; ++i) groups[g * dim + i] = m3out[g + i * nwg];
    free(m3out);
    return rc;
}

/* The kernel's nodal wind PSD (evalFct) at one frequency. */
double bsacl_ref_psd(double f, double scl, double std, double ubar) { return evalFct(f, scl, std, ubar); }

// Test infrastructure only: an extern "C" shim over the reference's own SWIG
// glue, scripts/swig/cauchy/pycauchy.hpp, compiled UNMODIFIED from the
// reference sources (no SWIG in this image).  oracle/ref_pycauchy.py turns it
// into a Python module with the SWIG module's names and return tuples, so the
// reference's unmodified scripts/swig/cauchy/cauchy_estimator.py
// (PyCauchyEstimator, PySlidingWindowManager, PySlidingWindowManager_CPP)
// runs on the reference's own C++ to produce the window-manager fixtures.
// Nothing in the product links this file.
//
// As in ref_harness.cpp, NUM_CPUS is redirected by macro (serial term order
// with HARNESS_NUM_CPUS = 1) without touching the reference sources.
#ifndef HARNESS_NUM_CPUS
#define HARNESS_NUM_CPUS 1
#endif

#define NUM_CPUS NUM_CPUS_REFERENCE_DEFAULT
#define NUM_CPUS_FTR NUM_CPUS_FTR_REFERENCE_DEFAULT
#include "cauchy_constants.hpp"
#undef NUM_CPUS
#undef NUM_CPUS_FTR
const int NUM_CPUS = HARNESS_NUM_CPUS;
const int NUM_CPUS_FTR = HARNESS_NUM_CPUS;

#include "pycauchy.hpp"

#include <stdlib.h>
#include <string.h>

typedef void (*dyn_cb_t)(CauchyDynamicsUpdateContainer*);

static void take(double* dst, double* src, int n)
{
    if (dst && src && n > 0) memcpy(dst, src, n * sizeof(double));
    free(src);
}

extern "C" {

void refpy_srand(unsigned seed) { srand(seed); }

void* refpy_initialize_lti(int num_steps, double* A0, int nA0, double* p0, int np0, double* b0, int nb0,
                           double* Phi, int nPhi, double* Gamma, int nGamma, double* B, int nB, double* beta,
                           int nbeta, double* H, int nH, double* gamma, int ngamma, double dt, int init_step,
                           int debug_print)
{
    return pycauchy_initialize_lti(num_steps, A0, nA0, p0, np0, b0, nb0, Phi, nPhi, Gamma, nGamma, B, nB, beta,
                                   nbeta, H, nH, gamma, ngamma, dt, init_step, debug_print != 0);
}

void* refpy_initialize_ltv(int num_steps, double* A0, int nA0, double* p0, int np0, double* b0, int nb0,
                           double* Phi, int nPhi, double* Gamma, int nGamma, double* B, int nB, double* beta,
                           int nbeta, double* H, int nH, double* gamma, int ngamma, void* cb, double dt,
                           int init_step, int debug_print)
{
    return pycauchy_initialize_ltv(num_steps, A0, nA0, p0, np0, b0, nb0, Phi, nPhi, Gamma, nGamma, B, nB, beta,
                                   nbeta, H, nH, gamma, ngamma, (dyn_cb_t)cb, dt, init_step, debug_print != 0);
}

// dyn[6] receive Phi, Gamma, B, H, beta, gamma (LTV only; may be NULL);
// moment outputs hold nm entries (nm = size of msmts).
void refpy_single_step_ltiv(void* h, double* msmts, int nm, double* controls, int nc, double** dyn, int* dyn_sizes,
                            double* fz, double* xhat, double* Phat, double* cfz, double* cx, double* cP, int* err)
{
    double *o[6] = {0, 0, 0, 0, 0, 0}, *f, *x, *P, *a, *b, *c;
    int s[6], sf, sx, sP, sa, sb, sc, se;
    int* e;
    pycauchy_single_step_ltiv(h, msmts, nm, controls, nc, &o[0], &s[0], &o[1], &s[1], &o[2], &s[2], &o[3], &s[3],
                              &o[4], &s[4], &o[5], &s[5], &f, &sf, &x, &sx, &P, &sP, &a, &sa, &b, &sb, &c, &sc, &e,
                              &se);
    for (int i = 0; i < 6; i++) {
        if (dyn_sizes) dyn_sizes[i] = s[i];
        take(dyn ? dyn[i] : nullptr, o[i], s[i]);
    }
    take(fz, f, sf);
    take(xhat, x, sx);
    take(Phat, P, sP);
    take(cfz, a, sa);
    take(cx, b, sb);
    take(cP, c, sc);
    if (err) memcpy(err, e, se * sizeof(int));
    free(e);
}

int refpy_get_number_of_terms(void* h) { return pycauchy_single_step_get_number_of_terms(h); }
void refpy_set_master_step(void* h, int step) { pycauchy_single_step_set_master_step(h, step); }
void refpy_set_window_number(void* h, int w) { pycauchy_single_step_set_window_number(h, w); }
void refpy_reset(void* h, double* A0, int nA0, double* p0, int np0, double* b0, int nb0, double* xbar, int nxbar)
{
    pycauchy_single_step_reset(h, A0, nA0, p0, np0, b0, nb0, xbar, nxbar);
}
void refpy_shutdown(void* h) { pycauchy_single_step_shutdown(h); }

void refpy_get_reinitialization_statistics(void* h, double z, double* xhat, int nx, double* Phat, int nP, double* H,
                                           int nH, double gamma, double* A0, double* p0, double* b0)
{
    double *a, *p, *b;
    int sa, sp, sb;
    pycauchy_get_reinitialization_statistics(h, z, xhat, nx, Phat, nP, H, nH, gamma, &a, &sa, &p, &sp, &b, &sb);
    take(A0, a, sa);
    take(p0, p, sp);
    take(b0, b, sb);
}

void refpy_speyers_window_init(double* xhat, int nx, double* Phat, int nP, double* H, int nH, double gamma, double z,
                               double* A0, double* p0, double* b0)
{
    double *a, *p, *b;
    int sa, sp, sb;
    pycauchy_speyers_window_init(xhat, nx, Phat, nP, H, nH, gamma, z, &a, &sa, &p, &sp, &b, &sb);
    take(A0, a, sa);
    take(p0, p, sp);
    take(b0, b, sb);
}

// root_point[d] and b_pert[max_shape] of an estimator made by pycauchy_initialize_*
void refpy_get_constants(void* h, double* root_point, double* b_pert, int* max_shape)
{
    CauchyEstimator* e = ((PyCauchyDataHandler*)h)->cauchyEst;
    memcpy(root_point, e->root_point, e->d * sizeof(double));
    *max_shape = e->shape_range - 1;
    memcpy(b_pert, e->dce_helper[0].b_pert, (e->shape_range - 1) * sizeof(double));
}

int refpy_set_tr_search_idxs_ordering(int* ordering, int n) { return pycauchy_set_tr_search_idxs_ordering(ordering, n); }

// The C++ window manager (forks one process per window)
void refpy_initialize_lti_window_manager(int num_windows, int num_sim_steps, double* A0, int nA0, double* p0,
                                         int np0, double* b0, int nb0, double* Phi, int nPhi, double* Gamma,
                                         int nGamma, double* B, int nB, double* beta, int nbeta, double* H, int nH,
                                         double* gamma, int ngamma, int debug_print, double dt, int init_step,
                                         double* wvb, int nwvb)
{
    pycauchy_initialize_lti_window_manager(num_windows, num_sim_steps, A0, nA0, p0, np0, b0, nb0, Phi, nPhi, Gamma,
                                           nGamma, B, nB, beta, nbeta, H, nH, gamma, ngamma, debug_print != 0, false,
                                           false, NULL, dt, init_step, wvb, nwvb);
}

void refpy_initialize_ltv_window_manager(int num_windows, int num_sim_steps, double* A0, int nA0, double* p0,
                                         int np0, double* b0, int nb0, double* Phi, int nPhi, double* Gamma,
                                         int nGamma, double* B, int nB, double* beta, int nbeta, double* H, int nH,
                                         double* gamma, int ngamma, void* cb, int debug_print, double dt,
                                         int init_step, double* wvb, int nwvb)
{
    pycauchy_initialize_ltv_window_manager(num_windows, num_sim_steps, A0, nA0, p0, np0, b0, nb0, Phi, nPhi, Gamma,
                                           nGamma, B, nB, beta, nbeta, H, nH, gamma, ngamma, (dyn_cb_t)cb,
                                           debug_print != 0, false, false, NULL, dt, init_step, wvb, nwvb);
}

void refpy_step(double* msmts, int nm, double* controls, int nc, double* fz, double* xhat, double* Phat, double* cfz,
                double* cx, double* cP, int* win_idx, int* err)
{
    double *x, *P;
    int sx, sP;
    pycauchy_step(msmts, nm, controls, nc, fz, &x, &sx, &P, &sP, cfz, cx, cP, win_idx, err);
    take(xhat, x, sx);
    take(Phat, P, sP);
}

void refpy_shutdown_window_manager(void) { pycauchy_shutdown(); }

typedef void (*msmt_cb_t)(CauchyDynamicsUpdateContainer*, double*);

// Extended (nonlinear) mode
void* refpy_initialize_nonlin(int num_steps, double* x0, int nx0, double* A0, int nA0, double* p0, int np0,
                              double* b0, int nb0, double* beta, int nbeta, double* gamma, int ngamma, void* f_dyn,
                              void* f_msmt, void* f_ext, int cmcc, double dt, int init_step, int debug_print)
{
    return pycauchy_initialize_nonlin(num_steps, x0, nx0, A0, nA0, p0, np0, b0, nb0, beta, nbeta, gamma, ngamma,
                                      (dyn_cb_t)f_dyn, (msmt_cb_t)f_msmt, (dyn_cb_t)f_ext, cmcc, dt, init_step,
                                      debug_print != 0);
}

// out[15] receive Phi, Gamma, B, H, beta, gamma, fz, xhat, Phat, xbar, zbar,
// cerr_fz, cerr_xhat, cerr_Phat (doubles) and err_code (ints, out[14]);
// sizes[15] their lengths.
void refpy_single_step_nonlin(void* h, double* msmts, int nm, double* controls, int nc, int with_propagate,
                              void** out, int* sizes)
{
    double* o[14];
    int* e;
    int s[15];
    pycauchy_single_step_nonlin(h, msmts, nm, controls, nc, with_propagate != 0, &o[0], &s[0], &o[1], &s[1], &o[2],
                                &s[2], &o[3], &s[3], &o[4], &s[4], &o[5], &s[5], &o[6], &s[6], &o[7], &s[7], &o[8],
                                &s[8], &o[9], &s[9], &o[10], &s[10], &o[11], &s[11], &o[12], &s[12], &o[13], &s[13],
                                &e, &s[14]);
    for (int i = 0; i < 14; i++) {
        sizes[i] = s[i];
        take((double*)out[i], o[i], s[i]);
    }
    sizes[14] = s[14];
    if (out[14] && s[14] > 0) memcpy(out[14], e, s[14] * sizeof(int));
    free(e);
}

void refpy_initialize_nonlin_window_manager(int num_windows, int num_sim_steps, double* x0, int nx0, double* A0,
                                            int nA0, double* p0, int np0, double* b0, int nb0, double* beta,
                                            int nbeta, double* gamma, int ngamma, void* f_dyn, void* f_msmt,
                                            void* f_ext, int cmcc, int debug_print, double dt, int init_step,
                                            double* wvb, int nwvb)
{
    pycauchy_initialize_nonlin_window_manager(num_windows, num_sim_steps, x0, nx0, A0, nA0, p0, np0, b0, nb0, beta,
                                              nbeta, gamma, ngamma, (dyn_cb_t)f_dyn, (msmt_cb_t)f_msmt,
                                              (dyn_cb_t)f_ext, cmcc, debug_print != 0, false, false, NULL, dt,
                                              init_step, wvb, nwvb);
}

}  // extern "C"

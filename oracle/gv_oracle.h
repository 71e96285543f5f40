/*
 * CPU oracle for the gpuvmem imaging-objective path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may load
 * it.  The product path (gpuvmem_gb300) never links, loads or calls it.
 *
 * It restates, in plain C with FP64 arithmetic, what the reference computes
 * on the GPU (file:line citations are relative to the gpuvmem repository):
 *   - hermitianSymmetry + metres_to_lambda      src/functions.cu:2256-2273,
 *                                               src/MSFITSIO.cu:36-45
 *   - calculateNoiseAndBeam / calc_sBeam /
 *     calc_beamSize / reduceCPU                 src/functions.cu:1655-1814,353-367
 *   - attenuation / GaussianBeam / AiryDiskBeam /
 *     total_attenuation / weight_image /
 *     noise_image, fg_scale, noise_cut          src/functions.cu:2275-2422,
 *                                               src/mfs.cu:630-645,849-916
 *   - chi2(): clip2IWNoise, calculateInu, apply_beam2I, cuFFT C2C inverse,
 *     phase_rotate, vis_mod, residual, chi2Vector   src/functions.cu:4323-4454
 *   - dchi2(): DChi2 + DChi2_total_I_nu_0 / DChi2_total_alpha
 *                                               src/functions.cu:3698-3791,3968-4024,4456-4558
 *   - prior values and gradients (entropy, TSV, TV, L1, Laplacian)
 *                                               src/functions.cu:2878-3545,4633-4964
 *   - ObjectiveFunction::calcFunction/calcGradient
 *                                               include/classes/objectivefunction.cuh:15-57
 *   - ConjugateGradient::optimize (frprmn), LBFGS::optimize, linmin, f1dim,
 *     bracket (mnbrak) and Brent minimisation    src/frprmn.cu:85-195, src/lbfgs.cu:99-341,
 *                                               src/linmin.cu:52-110, src/f1dim.cu:49-80,
 *                                               src/mnbrak.cu:44-98, src/brent.cu:43-121
 *
 * Discrete decisions (mask, beam cut-off, grid cell choice, positivity
 * floors, float lambda) follow the reference's own arithmetic types so that
 * the oracle and the reference pick the same pixels and cells; the values
 * themselves are carried in FP64.  The 2-D FFT is an FP64 radix-2 transform
 * with cuFFT's CUFFT_INVERSE convention (unnormalised, exp(+i)).
 *
 * Parity is pinned against the reference's own kernels run on a GB300 (see
 * the reference harness in oracle/ref_harness/); the reference's own test
 * suite has no golden values for this path.
 */
#ifndef GV_ORACLE_H
#define GV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_AIRYDISK = 0, OR_GAUSSIAN = 1 };
enum {
  OR_FI_CHI2 = 0,
  OR_FI_ENTROPY = 1,
  OR_FI_TSV = 2,
  OR_FI_TV = 3,
  OR_FI_L1 = 4,
  OR_FI_LAPLACIAN = 5,
  OR_FI_GENTROPY = 6,  /* entropy against a prior image, src/gentropy.cu */
  OR_FI_GL1 = 7,       /* L1 norm weighted by a prior image, src/gl1norm.cu */
  OR_FI_QUADRATIC = 8  /* quadratic penalization, src/quadraticpenalization.cu */
};

typedef struct or_term {
  int kind;
  float lambda;      /* penalization factor */
  int image_index;   /* plane the prior is evaluated on */
  int image_to_add;  /* plane its gradient is added to */
  float prior_value; /* entropy G */
  float eta;         /* entropy eta */
  float epsilon;     /* TV / L1 epsilon; GL1Norm epsilon_a */
  const float* prior_image; /* [M*N] GEntropy / GL1Norm prior (already normalised) */
  float epsilon_b;   /* GL1Norm epsilon_b */
} or_term;

/* One imaging problem: one field, nchan channels, one correlation each. */
typedef struct or_problem {
  int M, N; /* image columns (x) and rows (y); M == N */
  double DELTAX, DELTAY; /* degrees */
  float xobs, yobs;      /* reference = phase centre, pixels (float) */
  float nu_0;
  float antenna_diameter, pb_factor, pb_cutoff;
  int primary_beam;
  float eta, minpix, threshold;
  float noise_cut; /* absolute (already multiplied by min noise) */
  float fg_scale;
  int normalize;
  int nchan;
  const float* freq;      /* [nchan] */
  const int64_t* chan_off;/* [nchan+1] offsets into the visibility arrays */
  const double* uvw;      /* [3*V] in lambda, after hermitianSymmetry */
  const float* vo;        /* [2*V] observed visibilities (conjugated where flipped) */
  float* weight;          /* [V]   mutated: vis_mod zeroes out-of-grid weights */
  const float* noise;     /* [M*N] noise image */
  int nterms;
  const or_term* terms;   /* Chi2 first, as the reference requires */
  const float* gcf;       /* [M*N] gridding correction of gridded data, or NULL */
} or_problem;

/* ---- set-up ---------------------------------------------------------- */
void or_hermitian(int64_t n, double* uvw, float* vo, float freq);
/* returns sum of weights; writes vis noise (if *noise <= 0), bmaj/bmin/bpa (deg) */
float or_noise_and_beam(int nchan, const float* freq, const int64_t* chan_off,
                        const double* uvw_m, const float* weight, double* bmaj,
                        double* bmin, double* bpa, float* noise);
float or_attenuation(int i, int j, float xobs, float yobs, double DELTAX,
                     double DELTAY, float freq, float D, float pbf,
                     float cutoff, int primary_beam);
/* noise image; returns fg_scale (= min noise); *noise_cut_abs = factor*min */
float or_noise_image(int M, int N, double DELTAX, double DELTAY, float xobs,
                     float yobs, float nu_0, float D, float pbf, float cutoff,
                     int primary_beam, double bmaj_deg, double bmin_deg,
                     float vis_noise, float noise_cut_factor, float* noise_out,
                     float* noise_cut_abs);

/* ---- objective pieces ------------------------------------------------ */
void or_clip(const or_problem* p, float* img, int flag_opt);
/* chi2() with clip: mutates img and p->weight, writes vr [2*V] (FP64) */
double or_chi2(const or_problem* p, float* img, int flag_opt, double* vr);
/* model visibilities only (no clip): writes vm [2*V] FP64 */
void or_model_vis(const or_problem* p, const float* img, double* vm);
/* dchi2(): adds the chain-ruled chi2 gradient into result [2*M*N] */
void or_dchi2(const or_problem* p, const float* img, const double* vr,
              int flag_opt, double* result);
/* raw DChi2 of one channel: out[M*N] = -fg*A*sum_k w Re(conj(Vr) e^{i phi}) */
void or_dchi2_channel(const or_problem* p, int c, const double* vr,
                      double* out);
/* raw DChi2 sum of channel c at npix pixels (flat indices), FP64 */
void or_dchi2_pixels(const or_problem* p, int c, const double* vr, int npix,
                     const int64_t* pix, double* out);
double or_prior_value(const or_problem* p, const or_term* t, const float* img);
void or_prior_grad(const or_problem* p, const or_term* t, const float* img,
                   double* out /* [M*N] */);

/* ---- ObjectiveFunction + optimisers ----------------------------------- */
typedef struct or_state {
  const or_problem* p;
  int iteration;   /* Fi::iteration, set by calc_gradient */
  int flag_opt;
  double* vr;      /* [2*V] */
  double last_fi[8];
  long nevals, ngrads;
} or_state;

double or_calc_function(or_state* s, float* img);
void or_calc_gradient(or_state* s, float* img, float* xi, int iter);

typedef struct or_opt_report {
  int iterations;
  int exit_reason; /* 0 max iter, 1 ftol, 2 gtol, 3 gg==0 */
  float f_final;
  long nevals, ngrads;
} or_opt_report;

void or_frprmn(or_state* s, float* img, int total_iterations, float ftol,
               float gtol, int positivity, or_opt_report* rep);
void or_lbfgs(or_state* s, float* img, int total_iterations, int K, float ftol,
              float gtol, int positivity, or_opt_report* rep);

/* 2-D inverse FFT (CUFFT_INVERSE convention), FP64, in place, n x n, n = 2^k */
void or_fft2d_inverse(int n, double* data /* [2*n*n] interleaved */);

int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif

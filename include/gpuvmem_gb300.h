/*
 * gpuvmem_gb300 -- C ABI of the GB300-native imaging-objective path.
 *
 * The entry points replace the reference's objective/optimiser plugin
 * surface for one imaging problem (citations are file:line in the gpuvmem
 * repository):
 *
 *   gv_problem_create    MFS::setDevice set-up math (src/mfs.cu:530-943):
 *                        calculateNoiseAndBeam (src/functions.cu:1700-1814),
 *                        hermitianSymmetry (src/functions.cu:2256),
 *                        total_attenuation/weight_image/noise_image and
 *                        fg_scale/noise_cut (src/mfs.cu:849-916), plus
 *                        Fi::configure / ObjectiveFunction::addFi wiring
 *                        (include/classes/fi.cuh:58-89,
 *                        include/classes/objectivefunction.cuh:9-14)
 *   gv_chi2              Chi2::calcFi -> chi2() (src/chi2.cu:44-49,
 *                        src/functions.cu:4323-4454)
 *   gv_dchi2             Chi2::calcGi -> dchi2() (src/chi2.cu:51-53,
 *                        src/functions.cu:4456-4558)
 *   gv_prior_value       Fi::calcFi of Entropy/TSV/TV/L1/Laplacian
 *                        (src/entropy.cu:42, src/totalsquaredvariation.cu:12,
 *                        src/totalvariation.cu:26, src/l1norm.cu:26,
 *                        src/laplacian.cu:12)
 *   gv_prior_gradient    Fi::calcGi + Fi::addToDphi of the same classes
 *   gv_objective         ObjectiveFunction::calcFunction
 *                        (include/classes/objectivefunction.cuh:15-26)
 *   gv_gradient          ObjectiveFunction::calcGradient
 *                        (include/classes/objectivefunction.cuh:28-57)
 *   gv_optimize          Optimizer::optimize of "CG-FRPRMN" and "CG-LBFGS"
 *                        (src/frprmn.cu:85-195, src/lbfgs.cu:99-341) with
 *                        linmin/f1dim/mnbrak/brent (src/linmin.cu:52-110,
 *                        src/f1dim.cu:49-80, src/mnbrak.cu:44-98,
 *                        src/brent.cu:43-121)
 *   gv_dirty_image       the DChi2 adjoint applied to the observed data
 *
 * Conventions: plain pointers and sizes only.  Image buffers are DEVICE
 * pointers owned by the caller: 2 planes (I_nu0, alpha) of N rows x M
 * columns, row-major, plane stride M*N, exactly the reference's layout
 * (index N*M*plane + N*i + j).  Visibility inputs of gv_problem_create are
 * HOST pointers.  Every call returns a gv_status; nothing exits the process.
 * A problem handle is used by one host thread at a time; work is ordered on
 * the problem's CUDA stream (gv_problem_set_stream).
 */
#ifndef GPUVMEM_GB300_H
#define GPUVMEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gv_status {
  GV_OK = 0,
  GV_ERR_INVALID = 1,    /* bad argument or descriptor */
  GV_ERR_CUDA = 2,       /* a CUDA call failed (see gv_last_error) */
  GV_ERR_NOMEM = 3,      /* device allocation failed */
  GV_ERR_UNSUPPORTED = 4,/* size or option not supported by this build */
  GV_ERR_DEVICE = 5      /* a kernel reported an error status */
} gv_status;

/* Objective terms, in the order ObjectiveFunction::addFi receives them.
 * The registration ids of the reference are given for each. */
typedef enum gv_fi_kind {
  GV_FI_CHI2 = 0,      /* "Chi2"                  src/chi2.cu:89 */
  GV_FI_ENTROPY = 1,   /* "Entropy"               src/entropy.cu:75 */
  GV_FI_TSV = 2,       /* "TotalSquaredVariation" src/totalsquaredvariation.cu:44 */
  GV_FI_TV = 3,        /* "TotalVariation"        src/totalvariation.cu:60 */
  GV_FI_L1 = 4,        /* "L1-Norm"               src/l1norm.cu:57 */
  GV_FI_LAPLACIAN = 5, /* "Laplacian"             src/laplacian.cu:43 */
  GV_FI_GENTROPY = 6,  /* "GEntropy"  entropy against a prior image, src/gentropy.cu:131 */
  GV_FI_GL1 = 7,       /* "GL1Norm"   L1 norm over a prior image,   src/gl1norm.cu:165 */
  GV_FI_QUADRATIC = 8  /* "Quadratic" quadratic penalization, src/quadraticpenalization.cu:41 */
} gv_fi_kind;

typedef enum gv_beam { GV_BEAM_AIRYDISK = 0, GV_BEAM_GAUSSIAN = 1 } gv_beam;

typedef struct gv_fi_desc {
  int32_t kind;         /* gv_fi_kind */
  float lambda;         /* penalization factor; terms with 0 are dropped
                           like ObjectiveFunction::addFi */
  int32_t image_index;  /* plane the prior is evaluated on */
  int32_t image_to_add; /* plane its gradient is added to */
  float prior_value;    /* Entropy G (reference default set by main: 0.001) */
  float eta;            /* Entropy eta (reference default -1) */
  float epsilon;        /* TV / L1 epsilon; GL1Norm epsilon_a (reference default 1e-12) */
  /* GEntropy / GL1Norm: the prior image (host, M*N floats), divided by
   * normalization_factor at set-up as their normalizePrior does (0 counts as
   * 1); GL1Norm's epsilon_b (reference default 1e-12) */
  const float* prior_image;
  float normalization_factor;
  float epsilon_b;
} gv_fi_desc;

/* One spectral channel of one field with one correlation, as the
 * reference's per-(channel, stokes) visibility arrays (include/MSFITSIO.cuh:90-100). */
typedef struct gv_channel_desc {
  float freq_hz;
  int64_t nvis;
  const double* uvw;    /* host, 3*nvis: u,v,w in metres (double3 order) */
  const float* vo;      /* host, 2*nvis: observed visibility re,im */
  const float* weight;  /* host, nvis: weights after the weighting scheme */
} gv_channel_desc;

typedef struct gv_problem_desc {
  int32_t M, N;             /* image columns and rows; M == N, power of two */
  double deltax_deg;        /* DELTAX (FITS CDELT1, degrees; negative for RA) */
  double deltay_deg;        /* DELTAY */
  float xobs_pix, yobs_pix; /* phase / pointing centre in pixels (float) */
  float nu_0;               /* reference frequency */
  float antenna_diameter;
  float pb_factor;
  float pb_cutoff;
  int32_t primary_beam;     /* gv_beam */
  float vis_noise;          /* <= 0: 0.5*sqrt(1/sum w) as the reference */
  float noise_cut_factor;   /* -N, reference default 10 */
  float eta;                /* -e, reference default -1 */
  float initial_value;      /* -z first value; MINPIX = initial_value * -eta */
  float threshold;          /* 5 * -T, as src/mfs.cu:107 */
  int32_t normalize;        /* Chi2 normalize flag */
  int32_t nchannels;
  const gv_channel_desc* channels;
  int32_t nterms;
  const gv_fi_desc* terms;
  int32_t dchi2_engine;     /* 0 auto, 1 direct SIMT, 2 tensor-core GEMM */
  /* gridding correction function (host, M*N floats) of gridded data, or
   * NULL: with it chi2() multiplies the beam-weighted image by it before the
   * FFT (apply_GCF, src/functions.cu:2468) and DChi2 takes the GCF variant
   * (src/functions.cu:3793-3888), as when Chi2::setCKernel was called */
  const float* gcf;
} gv_problem_desc;

typedef struct gv_problem gv_problem;

typedef struct gv_problem_info {
  float fg_scale;
  float noise_cut;       /* absolute */
  float vis_noise;
  float minpix;
  double beam_bmaj_deg, beam_bmin_deg, beam_bpa_deg;
  float sum_weights;
  int64_t nvis_total;
  int64_t nvis_in_grid;  /* visibilities whose weight vis_mod keeps */
  int64_t mask_pixels;   /* pixels with noise < noise_cut */
  int32_t dchi2_engine;  /* engine actually used */
  int32_t nterms;        /* terms kept (lambda != 0) */
} gv_problem_info;

gv_status gv_problem_create(const gv_problem_desc* desc, gv_problem** out);
gv_status gv_problem_destroy(gv_problem* p);
gv_status gv_problem_info_get(const gv_problem* p, gv_problem_info* info);
/* cudaStream_t passed as void*; NULL = the legacy default stream */
gv_status gv_problem_set_stream(gv_problem* p, void* stream);
/* Copies the noise image (M*N floats) to a device buffer. */
gv_status gv_noise_image(gv_problem* p, float* d_out);
/* Copies the initial image (plane 0 = MINPIX, plane 1 = 0) to d_img. */
gv_status gv_initial_image(gv_problem* p, float* d_img);

/* Chi2::calcFi: clips d_img in place (clip2IWNoise), evaluates the model
 * visibilities, stores the weighted residuals for gv_dchi2 and returns
 * 0.5*sum w|Vo - Vm|^2 (per-channel /V when normalize). FP64 sum. */
gv_status gv_chi2(gv_problem* p, float* d_img, int32_t flag_opt, double* chi2);
/* Chi2::calcGi: d_result (2*M*N, device) += chain-ruled DChi2 of the
 * residuals stored by the last gv_chi2. */
gv_status gv_dchi2(gv_problem* p, const float* d_img, int32_t flag_opt,
                   float* d_result);
/* Raw DChi2 of one channel (before the chain rule): d_out[M*N] =
 * -fg*A*sum_k w_k Re(conj(Vr_k) e^{i phi}) (/V when normalize). */
gv_status gv_dchi2_channel(gv_problem* p, int32_t channel, float* d_out);
/* Prior value sum (before lambda) of term `term` (index into the kept
 * terms); evaluated whatever the iteration. */
gv_status gv_prior_value(gv_problem* p, int32_t term, const float* d_img,
                         double* value);
/* d_dphi[plane image_to_add] += lambda * dR/dI of term `term`. */
gv_status gv_prior_gradient(gv_problem* p, int32_t term, const float* d_img,
                            float* d_dphi);

/* ObjectiveFunction::calcFunction: sum of lambda*term over the kept terms;
 * priors contribute only after gv_gradient was called with iter > 0 (the
 * reference's Fi::iteration).  fi_values (may be NULL) receives each
 * term's value before lambda.  With graphs on (gv_problem_set_graphs) the
 * kernels are captured on the first call per (d_img, flag_opt, prior
 * gating) and replayed afterwards, as in gv_evaluate (the 8 most recently
 * used keys are kept; results equal the launch-by-launch ones bit for bit). */
gv_status gv_objective(gv_problem* p, float* d_img, int32_t flag_opt,
                       double* f, double* fi_values);
/* calcFunction of `count` images (d_imgs: a host array of device pointers,
 * each 2*M*N floats) with one host synchronisation for all of them (no
 * counterpart in the reference: scores candidate starting images).  Each
 * image is copied into the problem's scratch image and evaluated there, so
 * the images themselves are not clipped; f[i] (and, if not NULL,
 * fi_values[i * nterms + t]) equal what gv_objective returns for image i. */
gv_status gv_objective_many(gv_problem* p, const float* const* d_imgs, int32_t count,
                            int32_t flag_opt, double* f, double* fi_values);
/* ObjectiveFunction::calcGradient into d_xi (2*M*N, device); replayed from
 * a graph per (d_img, d_xi, flag_opt, iter > 0) when graphs are on. */
gv_status gv_gradient(gv_problem* p, float* d_img, float* d_xi, int32_t iter,
                      int32_t flag_opt);

typedef enum gv_optimizer_kind { GV_OPT_FRPRMN = 0, GV_OPT_LBFGS = 1 } gv_optimizer_kind;

typedef struct gv_opt_desc {
  int32_t kind;             /* gv_optimizer_kind */
  int32_t total_iterations; /* Optimizer::setTotalIterations */
  float ftol;               /* Optimizer default 1e-12 */
  float gtol;               /* Optimizer default 1e-12 */
  int32_t K;                /* L-BFGS memory, reference default 100 */
  int32_t flag;             /* Optimizer::setFlag (flag_opt) */
  int32_t positivity;       /* 1: plane 0 floored at -eta*MINPIX (default) */
} gv_opt_desc;

typedef struct gv_opt_report {
  int32_t iterations;
  int32_t exit_reason;      /* 0 max iterations, 1 ftol, 2 gtol, 3 gg == 0 */
  float f_final;
  int64_t n_objective;      /* objective evaluations */
  int64_t n_gradient;       /* gradient evaluations */
  double seconds;
} gv_opt_report;

gv_status gv_optimize(gv_problem* p, const gv_opt_desc* opt, float* d_img,
                      gv_opt_report* report);

/* ObjectiveFunction::calcFunction followed by calcGradient(iter) at the
 * same image (no single counterpart in the reference: frprmn.cu:99-101 and
 * lbfgs.cu:111-113 call the two back to back).  The kernel sequence is
 * captured into a CUDA graph on the first call with a given (d_img, d_xi,
 * flag_opt, prior gating) and replayed with one launch afterwards; the
 * result equals gv_objective then gv_gradient bit for bit.  The first call
 * per key must not happen while the problem's stream is being captured. */
gv_status gv_evaluate(gv_problem* p, float* d_img, float* d_xi, int32_t iter,
                      int32_t flag_opt, double* f, double* fi_values);

/* 1 (default, or GV_GRAPHS unset/not "0" at creation): gv_objective,
 * gv_gradient and the optimiser's evaluations are replayed from CUDA
 * graphs; 0: launched kernel by kernel.  Results are identical either way.
 * The first call per key must not happen while the problem's stream is
 * being captured. */
gv_status gv_problem_set_graphs(gv_problem* p, int32_t enable);

/* gv_optimize that also stops (exit_reason 4) once a line search with the
 * priors active (from the second iteration on, or from the first with
 * priors_from_start) reaches f <= f_target (no counterpart in the
 * reference: used to time convergence to a given objective).  With
 * priors_from_start = 0 the priors are off during the first line search, as
 * in the reference (Fi::iteration is 0 until the first calcGradient);
 * with 1 the first gradient is taken as iteration 1, so they count from the
 * start (used for warm starts, which are already near the solution). */
gv_status gv_optimize_until(gv_problem* p, const gv_opt_desc* opt, float* d_img,
                            double f_target, int32_t priors_from_start,
                            gv_opt_report* report);

/* linmin (src/linmin.cu:52-110): the objective minimised along d_xi from
 * d_p by the bracketing (src/mnbrak.cu:44-98) and Brent (src/brent.cu:43-121,
 * TOL 1e-7) search that gv_optimize's iterations run, then newP
 * (src/functions.cu:2760-2777): d_xi = xmin d_xi and d_p = d_p + d_xi, plane 0
 * floored at -eta*MINPIX with positivity (its d_xi then 0).  *fret is the
 * objective at the minimum and *evals (may be null) the evaluations the search
 * took.  d_p and d_xi are device images (2 x M x N floats).  The priors count
 * as Fi::iteration (gv_set_iteration) says.  The search runs on the GPU as
 * one CUDA-graph launch (a WHILE loop over the evaluations) when graphs are
 * on, else on the host; the two visit the same points. */
gv_status gv_linmin(gv_problem* p, float* d_p, float* d_xi, int32_t flag_opt,
                    int32_t positivity, float* fret, int64_t* evals);

/* Fi::setIteration(iter) on every term: iter > 0 makes the priors count in
 * the next gv_objective (the reference sets it only inside calcGradient,
 * include/classes/objectivefunction.cuh:39). */
gv_status gv_set_iteration(gv_problem* p, int32_t iter);

/* Dirty image: the DChi2 adjoint applied to w*Vo (no beam, no fg_scale):
 * d_out[M*N] = sum_c sum_k w Re(conj(Vo) e^{i phi}). */
gv_status gv_dirty_image(gv_problem* p, float* d_out);

/* Point-spread function: the same adjoint applied to w (Vr := 1), i.e. the
 * dirty image of a 1 Jy point source at the phase centre (no counterpart in
 * the reference; input of the warm-start network). */
gv_status gv_psf_image(gv_problem* p, float* d_out);

/* Copies the weighted residuals w*(Vo-Vm) of the last gv_chi2, in the
 * caller's visibility order, to a host buffer of 2*nvis_total floats. */
gv_status gv_residuals(gv_problem* p, float* h_out);

/* Prior value without any device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- code inside a host
 * framework that owns all device memory, or a real-time loop where an
 * allocation could synchronise the device.  Every input and output comes
 * from the caller: d_plane is one N x N image plane (row-major), d_noise the
 * N x N noise image (a pixel counts when noise < noise_cut, as the
 * reference's mask), d_value one device double receiving the sum of the
 * prior's per-pixel values (before lambda).  kind is GV_FI_ENTROPY ..
 * GV_FI_LAPLACIAN; prior_value/eta/epsilon as gv_fi_desc.  The only scratch
 * is a library-owned static device array of one FP64 partial per row, so
 * n is limited to 8192 (GV_ERR_UNSUPPORTED beyond).  The first call on a
 * device looks up that array's address; make it before any stream capture
 * (a first call inside a capture returns GV_ERR_INVALID).  Calls outside a
 * capture look the address up again, so a cudaDeviceReset in between does
 * not leave a stale address.  Calls share the array: calls that overlap on
 * the GPU race.  Work is enqueued on `stream` (cudaStream_t, NULL = legacy
 * default stream), which must belong to the current device
 * (GV_ERR_INVALID otherwise). */
gv_status gv_prior_value_static(int32_t kind, const float* d_plane, const float* d_noise,
                                float noise_cut, int32_t n, float prior_value, float eta,
                                float epsilon, double* d_value, void* stream);

/* Error images of a solution: calculateErrors (src/functions.cu:4966-5041):
 * d_err (2*M*N, device) = 1/sqrt of the I_nu0 and alpha noise sums of
 * I_nu_0_Noise / alpha_Noise (:4076, :4113), 0 outside the mask.  Evaluates
 * chi2 at d_img first (clipping it, as the reference's last evaluation did)
 * to get the residuals. */
gv_status gv_error_images(gv_problem* p, float* d_img, float* d_err);

/* Visibility weighting on the GPU: NaturalWeightingScheme::apply
 * (src/naturalweightingscheme.cu:9), UniformWeightingScheme::apply
 * (src/uniformweightingscheme.cu:9) and BriggsWeightingScheme::apply
 * (src/briggsweightingscheme.cu:30) for one field and one correlation,
 * without a uv taper.  Reads the channels' host uvw (metres) and weights,
 * writes the new weights to weights_out[c] (host, may alias the input).
 * The result equals the reference's with one OpenMP thread bit for bit
 * (the reference's own result with more threads depends on its schedule). */
typedef enum gv_weighting_kind {
  GV_WEIGHT_NATURAL = 0,  /* "Natural" */
  GV_WEIGHT_UNIFORM = 1,  /* "Uniform" */
  GV_WEIGHT_BRIGGS = 2    /* "Briggs", robust parameter */
} gv_weighting_kind;
gv_status gv_apply_weighting(int32_t scheme, float robust, int32_t M, int32_t N,
                             double deltax_deg, double deltay_deg, int32_t nchannels,
                             const gv_channel_desc* channels, float* const* weights_out,
                             void* stream);

/* Convolution kernels of the gridding path (the CKernel family,
 * include/classes/ckernel.cuh; src/pillBox2D.cu, src/gaussian2D.cu,
 * src/sinc2D.cu, src/gaussianSinc2D.cu, src/pswf_12D.cu; ids as their
 * registrations: "PillBox2D", "Gaussian2D", "Sinc2D", "GaussianSinc2D",
 * "PSWF").  gv_ckernel_defaults fills what the reference's (m, n)
 * constructor sets (PillBox2D's default constructor is 1 x 1). */
typedef enum gv_ckernel_kind {
  GV_CKERNEL_PILLBOX = 0,
  GV_CKERNEL_GAUSSIAN = 1,
  GV_CKERNEL_SINC = 2,
  GV_CKERNEL_GAUSSIAN_SINC = 3,
  GV_CKERNEL_PSWF = 4
} gv_ckernel_kind;
typedef struct gv_ckernel_desc {
  int32_t kind;
  int32_t m, n;  /* table rows and columns; supports are floor(m/2) in x and y */
  float amp;     /* 1 */
  float w;       /* width in cells: Gaussian, Sinc 1; GaussianSinc 2.52; PSWF 6 */
  float alpha;   /* Gaussian exponent, 2 */
  float w2;      /* GaussianSinc's sinc width, 1.55 */
} gv_ckernel_desc;
gv_status gv_ckernel_defaults(int32_t kind, int32_t m, int32_t n, gv_ckernel_desc* out);
/* MFS::configure's kernel set-up (src/mfs.cu:510-516): the m x n table with
 * cell sizes |deltau|, |deltav| (buildKernel) and the M x N gridding
 * correction function with cell sizes |deltax|, |deltay| in radians
 * (initializeGCF).  kernel: m*n floats; gcf: M*N floats or NULL.  has_gcf
 * is 0 for Sinc2D and GaussianSinc2D, which define no GCF (the reference
 * then reads an unset table); the GCF stays unused for them here. */
gv_status gv_ckernel_build(const gv_ckernel_desc* k, int32_t M, int32_t N, double deltax_deg,
                           double deltay_deg, float* kernel, int32_t* support_x,
                           int32_t* support_y, float* gcf, int32_t* has_gcf);

/* A convolution-kernel table as do_gridding reads it (getm, getn,
 * getSupportX/Y, getKernelValue). */
typedef struct gv_grid_kernel {
  int32_t m, n, support_x, support_y;
  const float* values;  /* host, m*n row-major */
} gv_grid_kernel;
/* do_gridding (src/functions.cu:1339-1653) on the GPU: each channel's
 * visibilities and their Hermitian copies are convolved onto the M x N
 * grid (weights, squared-kernel weights and weighted visibilities), each
 * occupied cell's visibility is divided by its weight sum and gets the
 * effective weight ws^2 / sum(w k^2), and the cells with a positive weight
 * become the new visibilities, in row-major cell order, at the cell's
 * (u, v) in metres with w = 0.  in[c]: host uvw (metres), Vo, weights;
 * out[c]: host arrays of capacity M*N (uvw 3*M*N doubles, vo 2*M*N floats,
 * weight M*N floats); out[c].nvis and freq_hz are written.  The result
 * equals the reference's with one OpenMP thread bit for bit. */
gv_status gv_grid_visibilities(const gv_grid_kernel* kernel, int32_t M, int32_t N,
                               double deltax_deg, double deltay_deg, int32_t nchannels,
                               const gv_channel_desc* in, gv_channel_desc* out, void* stream);

/* Device sort and scan of the set-up passes (the reference sorts nothing
 * on the GPU; its gridding walks the visibilities on the host).  The
 * gridding, the weighting schemes and the visibility ordering of
 * gv_problem_create use these; they are exported for tests and tools.
 * Device pointers; work is enqueued on `stream` and the call returns after
 * it has finished (scratch is allocated and freed inside).
 * gv_radix_sort_pairs_*: stable sort of (key, value) pairs by the key bits
 * [begin_bit, end_bit), least significant digit first; keys and values move
 * whole.  Output buffers must not overlap the inputs.  n < 2^32.
 * gv_exclusive_scan_i32: out[i] = in[0] + ... + in[i-1] (out may be in).
 * gv_run_length_encode_u32: runs of equal keys in d_keys: key, first
 * position and length of each run (at most cap runs are written), and the
 * run count in *d_nruns (device int). */
gv_status gv_radix_sort_pairs_u32(const uint32_t* d_keys_in, uint32_t* d_keys_out,
                                  const uint32_t* d_vals_in, uint32_t* d_vals_out, int64_t n,
                                  int32_t begin_bit, int32_t end_bit, void* stream);
gv_status gv_radix_sort_pairs_u64(const uint64_t* d_keys_in, uint64_t* d_keys_out,
                                  const int64_t* d_vals_in, int64_t* d_vals_out, int64_t n,
                                  int32_t begin_bit, int32_t end_bit, void* stream);
gv_status gv_exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream);
gv_status gv_run_length_encode_u32(const uint32_t* d_keys, int64_t n, uint32_t* d_run_keys,
                                   uint32_t* d_run_starts, uint32_t* d_run_lengths, int64_t cap,
                                   int32_t* d_nruns, void* stream);

/* Autotuner (the reference takes its launch shapes from the -X/-Y/-V
 * flags, src/main.cu; here they are measured): times the candidates of the
 * tensor-core DChi2 launch (CTA pairs or single CTAs x split-K counts) and of
 * the degridding launch (block size x blocks per channel) on this problem
 * and keeps the fastest.  Results stay within the parity tolerances of the
 * defaults (only reduction orders change).  Runs a few objective and DChi2
 * evaluations; call it before capturing graphs. */
typedef struct gv_tune_report {
  int32_t tc_pair;         /* 1 CTA pairs, 0 single CTAs (-1: DChi2 not on tensor cores) */
  int32_t tc_nsplit;
  int32_t degrid_threads;
  int32_t degrid_blocks;   /* per channel */
  double dchi2_ms_default, dchi2_ms_tuned;
  double chi2_ms_default, chi2_ms_tuned;
  int32_t candidates;      /* launch configurations timed */
} gv_tune_report;
gv_status gv_autotune(gv_problem* p, gv_tune_report* report);

/* ---- Batches of independent problems (no counterpart in the reference,
 * which runs problems one after another) ---------------------------------
 * One objective + gradient evaluation of every problem of the batch
 * (different sizes and visibility counts allowed) is captured into one CUDA
 * graph with a branch per problem and replayed with one launch and one
 * synchronisation.  f[i] is problem i's objective; each problem's stored
 * residuals, prior gating and scalars end as after gv_objective +
 * gv_gradient.  A problem must not be in two batches evaluated at once. */
typedef struct gv_batch gv_batch;
gv_status gv_batch_create(gv_problem* const* problems, int32_t n, gv_batch** out);
gv_status gv_batch_destroy(gv_batch* b);
/* 1 (default): one graph launch; 0: kernel by kernel, each problem on its own stream */
gv_status gv_batch_set_graphs(gv_batch* b, int32_t enable);
gv_status gv_batch_evaluate(gv_batch* b, float* const* d_imgs, float* const* d_xis,
                            int32_t iter, int32_t flag_opt, double* f);

/* ---- Learned warm start (no counterpart in the reference) --------------
 * A 2-D U-Net that maps the dirty image and the PSF to a warm-start image
 * for the solver.  Every convolution (forward, backward data, backward
 * weight) runs as a BF16 GEMM on the tensor cores with FP32 accumulation;
 * parameters, gradients and Adam state are FP32.  Tensors are NCHW FP32
 * device buffers.  Parameters are one flat vector, layer by layer (weights
 * [Cout][Cin][k][k] then bias [Cout]): encoder levels 0..L-1 (two 3x3
 * convolutions each, ReLU), decoder levels L-2..0 (two 3x3 convolutions on
 * [upsampled deeper level, encoder skip], ReLU), then a linear 1x1 output
 * convolution.  Down-sampling is 2x2 averaging, up-sampling nearest. */
typedef struct gv_unet gv_unet;
typedef struct gv_unet_desc {
  int32_t height, width;     /* square, divisible by 2^(levels-1) */
  int32_t in_channels;       /* e.g. 2: dirty image and PSF */
  int32_t base_channels;     /* channels at level 0 (multiple of 8); doubles per level, <= 256 */
  int32_t levels;
  int32_t max_batch;
  uint64_t seed;             /* He-normal initialisation */
} gv_unet_desc;
gv_status gv_unet_create(const gv_unet_desc* desc, gv_unet** out);
gv_status gv_unet_destroy(gv_unet* net);
gv_status gv_unet_set_stream(gv_unet* net, void* stream);
gv_status gv_unet_num_params(const gv_unet* net, int64_t* count);
gv_status gv_unet_get_params(gv_unet* net, float* d_out);      /* device, num_params floats */
gv_status gv_unet_set_params(gv_unet* net, const float* d_in); /* also resets Adam */
gv_status gv_unet_get_grads(gv_unet* net, float* d_out);       /* of the last loss_grad / step */
/* d_in: batch x in_channels x H x W; d_out: batch x 1 x H x W */
gv_status gv_unet_forward(gv_unet* net, const float* d_in, int32_t batch, float* d_out);
/* mean squared error against d_target (batch x 1 x H x W) and its gradient */
gv_status gv_unet_loss_grad(gv_unet* net, const float* d_in, const float* d_target,
                            int32_t batch, double* loss);
/* loss_grad followed by one Adam step (beta 0.9 / 0.999, eps 1e-8) */
gv_status gv_unet_train_step(gv_unet* net, const float* d_in, const float* d_target,
                             int32_t batch, float lr, double* loss);
/* One convolution layer on the tensor cores (test and tool entry points):
 * y = act(conv_ks(x, w) + bias) with zero padding ks/2, act = ReLU if relu;
 * backward: dx = conv^T(dz, w), dw, db from x and dz (dz is the gradient at
 * the pre-activation). */
gv_status gv_conv2d_forward(const float* x, const float* w, const float* bias, float* y,
                            int32_t B, int32_t Cin, int32_t Cout, int32_t H, int32_t W,
                            int32_t ks, int32_t relu, void* stream);
gv_status gv_conv2d_backward(const float* x, const float* w, const float* dz, float* dx,
                             float* dw, float* db, int32_t B, int32_t Cin, int32_t Cout,
                             int32_t H, int32_t W, int32_t ks, void* stream);

const char* gv_last_error(void);
const char* gv_version(void);
/* Diagnostics (no counterpart in the reference): number of kernels the
 * library has launched in this process. */
int64_t gv_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif

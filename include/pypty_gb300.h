/*
 * pypty_gb300 C ABI -- far-field multislice ptychography hot path on one GB300 (sm_103a).
 *
 * Plain C types only. Every device buffer (inputs, outputs, workspace) is allocated by the
 * caller; no entry point allocates device memory. Entry points are asynchronous with
 * respect to the host on the given CUDA stream (a cudaStream_t passed as void*; NULL is
 * the legacy default stream) except for the small host-to-device copies of the scan
 * geometry, which follow cudaMemcpyAsync semantics for the host memory they are given
 * (fully asynchronous only from page-locked memory).
 *
 * Array layouts are the reference's (C order, complex64 = interleaved float pairs):
 *   object        (obj_ny, obj_nx, n_slices, n_obj_modes)
 *   probe         (window, window, n_probe_modes)
 *   positions     (n_positions, 2) int32 [y, x] integer pixel positions
 *   pos_correction(n_positions, 2) float32 [dy, dx] sub-pixel corrections
 *   measured      (n_positions, window, window) float32 detector-plane intensities
 *   sequence      (n_sequence) int32 indices into the position list
 *
 * Return value: PTY_OK (0) or a negative PTY_ERR_* code. Errors detected on the host
 * (shapes, position range, workspace size) are returned before anything is launched.
 */
#ifndef PYPTY_GB300_H
#define PYPTY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTY_OK 0
#define PTY_ERR_INVALID (-1)     /* null pointer or non-positive size */
#define PTY_ERR_UNSUPPORTED (-2) /* window not 64/128, Mp*Mo > 8, unknown algorithm */
#define PTY_ERR_POSITION (-3)    /* a window leaves the object or a sequence entry is out of range */
#define PTY_ERR_WORKSPACE (-4)   /* workspace smaller than pty_workspace_bytes() */
#define PTY_ERR_CUDA (-5)        /* a CUDA launch or copy failed */

/* loss functions: pypty/objective.py:527-558 (algorithm_type strings) */
#define PTY_LSQ_SQRT 0   /* "lsq_sqrt"   amplitude L2 */
#define PTY_ML 1         /* "ml"         Poisson negative log-likelihood */
#define PTY_LSQ 2        /* "lsq"        intensity L2 */
#define PTY_LSQ_SQRT_2 3 /* "lsq_sqrt_2" */
/* compressed-detector losses on detector coefficients (pypty/objective.py:560-585); only
   pty_loss_and_direction_variants accepts them */
#define PTY_LSQ_COMPRESSED 4     /* "lsq_compressed" */
#define PTY_GAUSS_COMPRESSED 5   /* "gauss_compressed" */
#define PTY_POISSON_COMPRESSED 6 /* "poisson_compressed" */

typedef struct pty_problem {
  int32_t window;         /* W, probe window size in px: 64 or 128 */
  int32_t obj_ny, obj_nx; /* object extent in px */
  int32_t n_slices;       /* Z */
  int32_t n_obj_modes;    /* Mo */
  int32_t n_probe_modes;  /* Mp */
  int32_t n_positions;    /* rows of positions / pos_correction / measured */
  int32_t n_sequence;     /* entries of the sequence (this_chopped_sequence) */
  int32_t compute_batch;  /* positions per internal batch (compute_batch) */
  int32_t algorithm;      /* PTY_LSQ_SQRT, PTY_ML, PTY_LSQ or PTY_LSQ_SQRT_2 */
  int32_t step_obj;       /* nonzero: produce the object gradient */
  int32_t step_probe;     /* nonzero: produce the probe gradient */
  int32_t step_pos;       /* nonzero: produce the position gradient (needs probe_shift) */
  int32_t probe_shift;    /* nonzero: sub-pixel shift of the probe by Fourier ramps */
  float wavelength;       /* electron wavelength, Angstrom */
  float pixel_size_x;     /* Angstrom */
  float pixel_size_y;     /* Angstrom */
  float slice_distance;   /* Angstrom, one distance for all slices */
  float edge_mult;        /* first-slice thickness multiplier (propagator power) */
  float damping_cutoff;   /* band-limit cutoff as a fraction of Nyquist (2/3 default) */
  float smooth_rolloff;   /* cosine roll-off width of the band limit */
  float loss_weight;      /* this_loss_weight */
  int32_t checkpoint_every; /* 256-px windows: keep every k-th slice's wave and recompute the
                               others in the adjoint (k <= 1: keep all). No counterpart in the
                               reference, which keeps every slice (multislice_core.py:66). */
  const float* slice_distances; /* NULL: slice_distance for every step. Else n_slices - 1
                               distances in HOST memory, step z (slice z to z + 1) using entry z:
                               the reference's this_distances with more than one entry
                               (is_single_dist false, multislice_core.py:69-74, 164-174) */
} pty_problem_t;

/* Library version (major * 10000 + minor * 100 + patch). */
int pty_version(void);

/* Human-readable text of a PTY_* status code (static storage). */
const char* pty_status_string(int status);

/* Device workspace (bytes) that pty_loss_and_direction / pty_simulate_patterns need (0 for an
 * empty sequence). */
int pty_workspace_bytes(const pty_problem_t* problem, size_t* bytes);

/*
 * Loss, sum of squared errors and Wirtinger gradients dL/dz* of the far-field multislice
 * model over the positions of `sequence`, processed in batches of compute_batch.
 * Replaces pypty.objective.loss_and_direction (pypty/objective.py:47-967) for
 * recon_type "far_field", propmethod "multislice", no tilts, phase plates, aberration
 * arrays, beam-current fluctuations, static background or regularisers.
 *   obj, probe, measured        device, complex64 / float32, reference layouts
 *   positions_host, sequence_host   host memory (checked on the host)
 *   pos_correction_host         host or device memory (NULL: all zero)
 *   loss_sse                    device, 2 doubles: loss * loss_weight, sse
 *   object_grad                 device, complex64 (obj_ny, obj_nx, Z, Mo), overwritten
 *   probe_grad                  device, complex64 (W, W, Mp), overwritten (band-limited)
 *   pos_grad                    device, float32 (n_positions, 2), overwritten; rows not
 *                               in the sequence are zero
 * An empty sequence (n_sequence = 0) gives a zero loss, sse and gradients, as the reference's
 * loop over no batches does; the workspace is not used then.
 */
int pty_loss_and_direction(const pty_problem_t* problem, const void* obj, const void* probe,
                           const int32_t* positions_host, const float* pos_correction_host,
                           const int32_t* sequence_host, const float* measured,
                           double* loss_sse, void* object_grad, void* probe_grad,
                           float* pos_grad, void* workspace, size_t workspace_bytes,
                           void* stream);

/*
 * Mean-over-modes far-field intensities of the positions of `sequence`
 * (n_sequence, W, W) float32 in detector (fftshifted) order: the forward half of
 * pypty.objective.loss_and_direction with data_simulation_flag set
 * (pypty/objective.py:501-526). `measured` is not read.
 */
int pty_simulate_patterns(const pty_problem_t* problem, const void* obj, const void* probe,
                          const int32_t* positions_host, const float* pos_correction_host,
                          const int32_t* sequence_host, float* patterns, void* workspace,
                          size_t workspace_bytes, void* stream);

/*
 * The same computation as pty_loss_and_direction split into its two halves, for autograd
 * and for callers that want the loss before deciding on a gradient. pty_forward runs the
 * forward multislice and the loss for every position of the sequence (compute_batch is
 * ignored: one batch) and keeps the wave stack and dL/d(exit wave) in the workspace;
 * pty_backward, called later on the same stream with the same problem and the same
 * untouched workspace, runs the adjoint and writes the gradients (and loss_sse again).
 * No counterpart in the reference, which always computes both (pypty/objective.py:47).
 * The workspace size is pty_split_workspace_bytes (it holds every position at once).
 */
int pty_split_workspace_bytes(const pty_problem_t* problem, size_t* bytes);
int pty_forward(const pty_problem_t* problem, const void* obj, const void* probe,
                const int32_t* positions_host, const float* pos_correction_host,
                const int32_t* sequence_host, const float* measured, double* loss_sse,
                void* workspace, size_t workspace_bytes, void* stream);
int pty_backward(const pty_problem_t* problem, double* loss_sse, void* object_grad,
                 void* probe_grad, float* pos_grad, void* workspace, size_t workspace_bytes,
                 void* stream);

/*
 * The multislice_core functions on caller-given windows, reference layouts (modes innermost):
 *   probe_b   (batch, W, W, Mp)          incoming probe of every position
 *   obj_b     (batch, W, W, Z, Mo)       object windows (already band-limited by the caller)
 *   propagator (W, W) complex64          Fresnel propagator with the mask applied
 *   waves     (batch, W, W, Z, Mp, Mo)   conjugated input wave of every slice
 *   exit_wave / d_exit (batch, W, W, Mp, Mo)
 *   mask_clean (W, W) float32            band limit of the gradient windows
 *   object_grad (obj_ny, obj_nx, Z, Mo)  accumulated (+=), as the reference does
 *   probe_grad (batch, W, W, Mp)         sum over object modes of the probe-plane gradient
 * pty_multislice replaces pypty.multislice_core.multislice (pypty/multislice_core.py:9-82,
 * one slice distance, no tilts); pty_multislice_grads replaces multislice_grads
 * (pypty/multislice_core.py:85-200, no tilts; positions_host (batch, 2) are the windows'
 * top-left pixels, i.e. masked_pixels_y/x[:, 0, 0]); pty_scatteradd replaces scatteradd
 * (pypty/multislice_core.py:206-230) for window-shaped index arrays: chop (batch, W, W,
 * n_planes) is added into full (obj_ny, obj_nx, n_planes) in position order without atomics.
 */
int pty_multislice_workspace_bytes(int32_t batch, int32_t window, int32_t n_slices, int32_t n_probe_modes,
                                   int32_t n_obj_modes, int32_t obj_ny, int32_t obj_nx, size_t* bytes);
int pty_multislice(const void* probe_b, const void* obj_b, const void* propagator, float edge_mult,
                   int32_t batch, int32_t window, int32_t n_slices, int32_t n_probe_modes,
                   int32_t n_obj_modes, void* waves, void* exit_wave, void* workspace,
                   size_t workspace_bytes, void* stream);
int pty_multislice_grads(const void* d_exit, const void* waves, const void* obj_b, const void* propagator,
                         float edge_mult, const float* mask_clean, const int32_t* positions_host,
                         int32_t batch, int32_t window, int32_t n_slices, int32_t n_probe_modes,
                         int32_t n_obj_modes, int32_t obj_ny, int32_t obj_nx, int32_t step_obj,
                         void* object_grad, void* probe_grad, void* workspace, size_t workspace_bytes,
                         void* stream);
int pty_scatteradd_workspace_bytes(int32_t batch, int32_t window, int32_t n_planes, int32_t obj_ny,
                                   int32_t obj_nx, size_t* bytes);
int pty_scatteradd(void* full, int32_t obj_ny, int32_t obj_nx, int32_t n_planes,
                   const int32_t* positions_host, int32_t batch, int32_t window, const void* chop,
                   void* workspace, size_t workspace_bytes, void* stream);

/*
 * Batched 2D FFT of `batch` contiguous W x W complex64 windows (W = 64 or 128).
 * inverse = 0: unnormalised forward transform; inverse = 1: inverse scaled by 1/W^2.
 * shift = 1 applies fftshift to the forward output / ifftshift to the inverse input.
 * Replaces pypty.fft.fft2 / ifft2 / shift_fft2 / ifft2_ishift over axes (1, 2) of a
 * (batch, W, W) array (pypty/fft.py:91-178). in and out may alias.
 */
int pty_fft2(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse,
             int32_t shift, void* workspace, size_t workspace_bytes, void* stream);

/* Workspace for pty_fft2 (twiddle tables). */
int pty_fft2_workspace_bytes(int32_t window, size_t* bytes);

/*
 * The same batched 2D DFT of `batch` contiguous W x W complex64 windows (W = 64, 128, 256) as
 * dense GEMMs on the tensor cores (tcgen05, BF16x3 split precision: every FP32 operand is
 * hi + lo in BF16 and the three significant products accumulate in FP32 in tensor memory).
 * inverse = 1: scaled by 1/W^2. No shift. in and out must not alias. Relative error ~1e-5
 * against an FP64 DFT (the FP32 register FFT, pty_fft2, is ~1e-7). Replaces pypty.fft.fft2 /
 * ifft2 over axes (1, 2) (pypty/fft.py:114-156) in the precision sweep; no counterpart in
 * the reference.
 */
int pty_fft2_bf16x3_workspace_bytes(int32_t batch, int32_t window, size_t* bytes);
int pty_fft2_bf16x3(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse,
                    void* workspace, size_t workspace_bytes, void* stream);

/* The same with three BF16 terms per FP32 operand and the six significant products (BF16x6):
 * twice the tensor work of BF16x3, FP32-level error (~2e-7 relative against an FP64 DFT). */
int pty_fft2_bf16x6_workspace_bytes(int32_t batch, int32_t window, size_t* bytes);
int pty_fft2_bf16x6(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse,
                    void* workspace, size_t workspace_bytes, void* stream);

/* window-DFT engines of the precision sweep */
#define PTY_DFT_FP32_FFT 0 /* the FP32 register FFT (pty_fft2) */
#define PTY_DFT_BF16X3 1   /* tensor-core GEMMs in BF16x3 split precision (pty_fft2_bf16x3) */
#define PTY_DFT_BF16X6 2   /* tensor-core GEMMs in BF16x6 split precision (pty_fft2_bf16x6) */

/*
 * pty_loss_and_direction computed as batched passes over natural-layout windows with every
 * window DFT on the chosen engine: the precision sweep of pypty.objective.loss_and_direction
 * (pypty/objective.py:47-967, same flag set, same arguments and outputs; pos_correction may be
 * host or device memory). Its own workspace: pty_layered_workspace_bytes. Batches are limited
 * to compute_batch * max(Z * Mo, Mp * Mo) <= 65535 windows (else PTY_ERR_UNSUPPORTED).
 * No counterpart in the reference (which has one FFT precision per dtype).
 */
int pty_layered_workspace_bytes(const pty_problem_t* problem, int32_t engine, size_t* bytes);
int pty_loss_and_direction_layered(const pty_problem_t* problem, int32_t engine, const void* obj,
                                   const void* probe, const int32_t* positions_host,
                                   const float* pos_correction, const int32_t* sequence_host,
                                   const float* measured, double* loss_sse, void* object_grad,
                                   void* probe_grad, float* pos_grad, void* workspace,
                                   size_t workspace_bytes, void* stream);

/*
 * The other propagation, loss and probe branches of pypty.objective.loss_and_direction
 * (pypty/objective.py:283-742), computed like pty_loss_and_direction_layered on the FP32
 * FFT engine (pypty/objective.py line numbers below):
 *   near-field propagation (recon_type "near_field", one defocus, Cs: 504-508, 598-604);
 *   compressed-detector losses (algorithm PTY_*_COMPRESSED on n_masks detector masks,
 *     560-585; measured is then (n_positions, n_masks));
 *   beam-current fluctuations and their gradient (448-452, 687-697);
 *   per-position aberration phase plates and their gradient (324-329, 459-463, 676-684);
 *   one inside beam tilt, tilt_mode 0 (337-345, 505).
 * The variant fields that are off (recon_type 0, n_masks 0, NULL arrays) leave the far-field
 * path of pty_loss_and_direction_layered. Replaces the same loss_and_direction call
 * (pypty/objective.py:47) with those arguments set. Device arrays: masks (n_masks, W, W) in
 * pattern order (fftshifted detector order for the far field, real-space order for the
 * near field), beam_current / beam_current_grad (n_positions), aberrations /
 * aberrations_grad (n_aberration_sets, n_aberrations), aberration_marker (n_positions); a
 * marker outside [0, n_aberration_sets) leaves its position without a plate.
 * The near-field partial-coherence correction (alpha_near_field > 0) has no counterpart:
 * the reference raises on it.
 */
typedef struct pty_variant {
  int32_t recon_type;          /* 0: far field, 1: near field */
  float defocus;               /* near field: defocus_array[0], Angstrom */
  float cs;                    /* near field: spherical aberration Cs, Angstrom */
  float tan_x, tan_y;          /* inside tilt (tilts[0, 3], tilts[0, 2]) */
  int32_t n_masks;             /* compressed losses: number of detector masks */
  const float* masks;
  const float* beam_current;   /* NULL: no beam-current fluctuations */
  int32_t step_beam_current;
  float* beam_current_grad;
  int32_t n_aberrations;       /* coefficients per aberration set (Krivanek order) */
  int32_t n_aberration_sets;
  const float* aberrations;    /* NULL: no aberration plates */
  const int32_t* aberration_marker;
  int32_t step_aberrations;
  float* aberrations_grad;
  /* per-batch measured-data preprocessing (pypty/utils.py:626-652 as objective.py:411-412
     calls it; not for the compressed losses): the measured patterns are
     (W - 2 data_pad)^2, rolled by (shift_y, shift_x) with the reference's zeroed rows and
     columns, scaled by data_multiplier, then zero-padded to W (use_padded_intensity != 0) or
     compared with the model pattern cropped by data_pad (use_padded_intensity == 0,
     objective.py:516-517, 592-593) */
  int32_t data_pad;
  int32_t use_padded_intensity;
  int32_t shift_y, shift_x;
  float data_multiplier;   /* 0 is read as 1: a zero-initialised struct leaves the data unscaled */
  /* beam tilts (pypty/objective.py:302-345, 464-499, 605-673; multislice_core.py:76-77,
     178-182): n_tilts rows (1, or one per position) of [tan_y, tan_x] before / inside / after
     the specimen in HOST memory (the reference's tilt array plus its correction); tilt_mode
     0-4 as the reference's; with step_tilts the gradient (n_tilts, 6) goes to tilts_grad
     (device). n_tilts = 0: one inside tilt (tan_x, tan_y) and no tilt gradient. One row with
     step_tilts and tilt_mode 0, 3 or 4 returns the sum over positions of the inside-tilt
     gradient (the reference raises there unless compute_batch is 1). */
  int32_t n_tilts;
  const float* tilts_host;
  int32_t tilt_mode;
  int32_t step_tilts;
  float* tilts_grad;
  /* detector upsampling (pypty/objective.py:523-524, 590-591; utils.py:376-426): the model
     pattern, after the data_pad crop, is summed over upsample_pattern^2 blocks before the
     loss and dL/dI is repeated back over each block; the measured patterns are then
     (S / u - 2 po)^2 with S the cropped side and po = data_pad / u when use_padded_intensity.
     0 or 1: none. S must be a multiple of u; not with the compressed losses. */
  int32_t upsample_pattern;
  /* static background (pypty/objective.py:359-361, 525-526, 588-589): W x W float32 on the
     device or NULL; the pattern gets static_background^2 * band-limit mask (detector order)
     before the loss. With step_static_background its gradient
     sum_b dL/dI * 2 * static_background * loss_weight goes to static_background_grad
     (W x W, device). Needs data_pad = 0 or use_padded_intensity, and no upsampling (the
     reference's shapes do not broadcast otherwise). */
  const float* static_background;
  int32_t step_static_background;
  float* static_background_grad;
  /* near field: one defocus per position (device, n_positions entries; the reference's
     defocus_array with more than one entry, is_single_defocus false, objective.py:413-418),
     or NULL: `defocus` for every position. The reference's (B,) array broadcasts against its
     (1, W, W) grids only for batches of one position; here every batch size applies each
     position's own defocus. */
  const float* defocus_per_position;
  /* several probe scenarios (pypty/objective.py:285, 355-356, 443-444, 700-701, 754-755):
     n_probe_scenarios = S > 1 makes probe and probe_grad (W, W, Mp, S) arrays and gives every
     position the scenario probe_marker[position] (device int32, n_positions entries in
     [0, S); an entry outside that range reads scenario 0). 0 or 1: one probe. */
  int32_t n_probe_scenarios;
  const int32_t* probe_marker;
  /* NULL, or device complex64 [n_sequence][Mp][Mo][W][W]: the exit wave of every position of
     the sequence (after a tilt after the specimen), as data_simulation_exitwave saves it
     (pypty/objective.py:289-291, 518-520) */
  void* exit_waves;
  /* the tilt rows of tilts_host in DEVICE memory instead (n_tilts rows of 6 float32), or
     NULL: an optimizer's trial tilts stay on the device. When set, tilts_host is not read. */
  const float* tilts_device;
} pty_variant_t;

int pty_variants_workspace_bytes(const pty_problem_t* problem, const pty_variant_t* variant, size_t* bytes);
int pty_loss_and_direction_variants(const pty_problem_t* problem, const pty_variant_t* variant,
                                    const void* obj, const void* probe, const int32_t* positions_host,
                                    const float* pos_correction, const int32_t* sequence_host,
                                    const float* measured, double* loss_sse, void* object_grad,
                                    void* probe_grad, float* pos_grad, void* workspace,
                                    size_t workspace_bytes, void* stream);

/*
 * pty_fft2 without a workspace argument; it allocates nothing. No counterpart in the
 * reference: it exists for callers that cannot allocate device memory -- an application
 * whose own memory pool owns every device allocation, code running while a CUDA graph is
 * captured (cudaMalloc is not allowed then), or a loop that must not pay for an allocation.
 * The twiddle tables live in a fixed 3 KiB array of device memory inside the library,
 * created on every GPU that loads the library and kept until the process exits.
 * Limits: window 64 or 128 only (anything else returns PTY_ERR_UNSUPPORTED); batch > 0.
 * The first call on a device looks up the array's device address (with that device
 * current); make that first call before any stream capture. All calls share the array and
 * each call rewrites the table it uses, so calls that overlap on the GPU (different
 * streams) race: serialise them, or use pty_fft2 with a workspace per stream.
 * Same arguments and results as pty_fft2.
 */
int pty_fft2_noalloc(const void* in, void* out, int32_t batch, int32_t window, int32_t inverse,
                     int32_t shift, void* stream);

/*
 * ---------------------------------------------------------------------------------------
 * Optimizer step around loss_and_direction: the band limit `fourier_clean` and the
 * L-BFGS / Wolfe line-search algebra of `bfgs_update`. The host keeps the loop (trial
 * steps, Wolfe decisions, history list); every array operation and every scalar of the
 * recursion runs on the device.
 */

/*
 * out = fourier_clean(x + step * dx) over axes 0 and 1 of an (ny, nx, k) complex64 array
 * (k = every trailing axis flattened; replaces pypty/utils.py:102-150 for 2D, 3D and 4D
 * arrays): fftshift(fft2) times the band-limit mask, then ifft2(ifftshift).
 * The mask is utils.fourier_clean's: radius 0.5 * cutoff in cycles per pixel, cosine roll-off
 * of width `rolloff` (0: none), computed with the reference's float32 / float64 promotions;
 * or, when mask_shifted is not NULL, the caller's (ny, nx) float32 mask in fftshifted order
 * (the `mask=` argument). dx may be NULL (then step is ignored); x may be NULL (in place on
 * out); x and out may alias. ny and nx: powers of two in [64, 8192], else
 * PTY_ERR_UNSUPPORTED.
 */
int pty_fourier_clean_workspace_bytes(int32_t ny, int32_t nx, size_t* bytes);
int pty_fourier_clean(const void* x, const void* dx, double step, void* out, int32_t ny, int32_t nx,
                      int64_t k, float cutoff, float rolloff, const float* mask_shifted,
                      void* workspace, size_t workspace_bytes, void* stream);
/* pty_fourier_clean in two halves, for repeated cleans with one band limit: _prepare writes
 * the twiddle and mask tables into the workspace, _apply uses them (the workspace must hold
 * the tables of the same ny, nx and band limit, unmodified since _prepare). */
int pty_fourier_clean_prepare(int32_t ny, int32_t nx, float cutoff, float rolloff, const float* mask_shifted,
                              void* workspace, size_t workspace_bytes, void* stream);
int pty_fourier_clean_apply(const void* x, const void* dx, double step, void* out, int32_t ny, int32_t nx,
                            int64_t k, const void* workspace, size_t workspace_bytes, void* stream);

/*
 * The optimizer's vector space: up to PTY_VSPACE_MAX_SEG float32 segments (the object, the
 * probe, the position corrections, the tilt corrections, the static background, the
 * aberration arrays and the beam currents of pypty/iterative.py:583-672, in that order; a
 * complex64 element counts as two floats). Every
 * inner product is sum_seg weight[seg] * <a_seg, b_seg>; the reference's weights are 2 for
 * the complex segments and 1 for the real ones (iterative.py:597-609). Each segment has its
 * own Barzilai-Borwein gamma (iterative.py:626-647, 869-916). obj_seg names the object
 * segment for the first step's normalisation (-1: none). Vectors are passed as arrays of
 * n_seg device pointers.
 */
#define PTY_VSPACE_MAX_SEG 7
typedef struct pty_vspace {
  int32_t n_seg;
  int32_t obj_seg;
  int64_t n[PTY_VSPACE_MAX_SEG];
  double weight[PTY_VSPACE_MAX_SEG];
} pty_vspace_t;

/* Device bytes of the optimizer state (FP64 scalars, partial sums); caller-allocated. */
int pty_lbfgs_state_bytes(size_t* bytes);
/* Clear the state: weights from vs, gammas 1 (pypty/iterative.py:1055-1103). */
int pty_lbfgs_reset(const pty_vspace_t* vs, void* state, void* stream);
/* Empty history: dir = -g scaled per segment so that every segment's step matches the
 * object's (iterative.py:562-571); d_value = <dir, g>. */
int pty_lbfgs_first_direction(const pty_vspace_t* vs, float* const* grad, float* const* dir, void* state,
                              void* stream);
/* Steepest-descent fallback of a non-negative d_value (iterative.py:691-724): dir = -gamma g. */
int pty_lbfgs_steepest(const pty_vspace_t* vs, float* const* grad, float* const* dir, void* state,
                       void* stream);
/* L-BFGS two-loop recursion (iterative.py:583-681): dir = -H g from m history pairs
 * (s_hist, y_hist: m x n_seg pointers, oldest first; slots: their rho/alpha slots < 64).
 * The caller band-limits the object segment of dir afterwards and calls pty_lbfgs_dot. */
int pty_lbfgs_two_loop(const pty_vspace_t* vs, float* const* grad, float* const* dir, int32_t m,
                       float* const* s_hist, float* const* y_hist, const int32_t* slots, void* state,
                       void* stream);
/* Weighted inner product <x, y> into d_value (target 0, iterative.py:684-690) or
 * new_d_value (target 1, iterative.py:811-817). */
int pty_lbfgs_dot(const pty_vspace_t* vs, float* const* x, float* const* y, int32_t target, void* state,
                  void* stream);
/* out = a + step * b per segment (trial points, iterative.py:759-771). */
int pty_lbfgs_axpy(const pty_vspace_t* vs, float* const* out, float* const* a, float* const* b, double step,
                   void* stream);
/* Accepted step (iterative.py:849-916): s_out = step * dir, y_out = new_grad - grad,
 * gamma_seg = weight <y, s> / <y, y>, rho[slot] = 1 / sum_seg weight <y, s>. */
int pty_lbfgs_accept(const pty_vspace_t* vs, double step, float* const* dir, float* const* grad,
                     float* const* new_grad, float* const* s_out, float* const* y_out, int32_t slot,
                     void* state, void* stream);
/* Synchronising read of 2 + 2 * PTY_VSPACE_MAX_SEG doubles: d_value, new_d_value,
 * gamma[PTY_VSPACE_MAX_SEG], last reduced dots[PTY_VSPACE_MAX_SEG]. */
int pty_lbfgs_read(const void* state, double* out, void* stream);
/* Gram-Schmidt over the modes of a (n_pixels, n_modes) complex64 probe, in place
 * (pypty/objective.py:1119-1141, keep_probe_states_orthogonal). */
int pty_orthogonalize_modes(void* probe, int64_t n_pixels, int32_t n_modes, void* stream);

/*
 * ---------------------------------------------------------------------------------------
 * Learned warm start (no counterpart in the reference, whose warm starts are non-learned,
 * pypty/initialize.py:629): the kernels of a small U-Net that maps per-position
 * centre-of-mass / virtual-bright-field maps to an object phase stack, and of its training.
 * Tensors are NCHW; activations and their gradients BF16 (void*), weights and their gradients
 * FP32. 3x3 convolutions need H and W multiples of 32; 1x1 convolutions at most 64 channels.
 */
/* out = act(conv3x3(x, w) + b), zero padding 1; transpose = 1: the data gradient
 * (x = dL/d(layer output) with Ci = the layer's Co, out = dL/d(layer input), Co = the layer's Ci). */
int pty_nn_conv3x3(const void* x, const float* w, const float* bias, void* out, int32_t N, int32_t Ci,
                   int32_t Co, int32_t H, int32_t W, int32_t relu, int32_t transpose, void* stream);
/* dw (Co, Ci, 3, 3) and db (Co) of a 3x3 convolution, deterministic (fixed-order block sums). */
int pty_nn_conv3x3_wgrad_workspace_floats(int32_t N, int32_t Ci, int32_t Co, int32_t H, int32_t W, int64_t* n);
int pty_nn_conv3x3_wgrad(const void* dy, const void* x, float* dw, float* db, int32_t N, int32_t Ci, int32_t Co,
                         int32_t H, int32_t W, float* workspace, void* stream);
int pty_nn_conv1x1(const void* x, const float* w, const float* b, void* out, int32_t N, int32_t Ci, int32_t Co,
                   int64_t plane, void* stream);
int pty_nn_conv1x1_workspace_floats(int32_t N, int32_t Ci, int32_t Co, int64_t plane, int64_t* n);
int pty_nn_conv1x1_backward(const void* dy, const void* x, const float* w, void* dx, float* dw, float* db,
                            int32_t N, int32_t Ci, int32_t Co, int64_t plane, float* workspace, void* stream);
/* dst += src (BF16) */
int pty_nn_add(void* dst, const void* src, int64_t n, void* stream);
/* dy *= (y > 0) */
int pty_nn_relu_mask(void* dy, const void* y, int64_t n, void* stream);
/* 2x2 average pooling (backward = 1: its adjoint, x = dL/dy of size H/2 x W/2, y = dL/dx of H x W) */
int pty_nn_avgpool2(const void* x, void* y, int64_t nplanes, int32_t H, int32_t W, int32_t backward, void* stream);
/* nearest 2x upsampling of x (N, C, H, W) into channels [c_off, c_off + C) of y (N, Ct, 2H, 2W); backward: adjoint */
int pty_nn_upsample2(const void* x, void* y, int32_t N, int32_t C, int32_t Ct, int32_t c_off, int32_t H, int32_t W,
                     int32_t backward, void* stream);
/* copy (N, C, plane) into (into = 1) or out of channels [c_off, c_off + C) of (N, Ct, plane) */
int pty_nn_channel_copy(const void* src, void* dst, int32_t N, int32_t C, int32_t Ct, int32_t c_off, int64_t plane,
                        int32_t into, void* stream);
/* bilinear float (N, C, h, w) -> BF16 (N, Cd, H, W): output pixel (Y, X) samples the map at
 * ((Y - oy) / sy, (X - ox) / sx), zero outside it; channels >= C zero */
int pty_nn_bilinear(const float* src, void* dst, int32_t N, int32_t C, int32_t Cd, int32_t h, int32_t w, int32_t H,
                    int32_t W, float oy, float ox, float sy, float sx, void* stream);
/* mean squared error: 256 FP64 partial sums (sum them for n * loss) and dL/dpred */
int pty_nn_mse(const void* pred, const float* target, void* dpred, double* partials, int64_t n, void* stream);
/* Adam step with the bias-corrected learning rate lr_t */
int pty_nn_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr_t, float b1, float b2, float eps,
                void* stream);
/* per pattern (detector order): centre of mass x, y (pixels from the centre) and the bright-field
 * disk sum within r_bf pixels (pypty/dpc.py:137-151); out (n_patterns, 3) */
int pty_virtual_detectors(const float* patterns, int32_t n_patterns, int32_t window, float r_bf, float* out,
                          void* stream);
/* Gaussian-atom phase slices (atoms: (n_slices, n_atoms, 3) = y, x [px], peak phase [rad]) into
 * phase (n_slices, ny, nx) float and, if obj != NULL, exp(i phase) into obj (ny, nx, n_slices, 1) complex64 */
int pty_atom_slices(const float* atoms, int32_t n_atoms, int32_t ny, int32_t nx, int32_t n_slices, float sigma_px,
                    float* phase, void* obj, void* stream);

/*
 * Launch profiler (no counterpart in the reference, which only logs wall time,
 * pypty/utils.py:1894). While enabled, every kernel launch of the library records a CUDA
 * event on its stream just before the launch, and every call records one when its last
 * launch is queued. pty_profile_end synchronises, disables profiling and returns, per
 * kernel class, the summed device time between each launch's event and the next event on
 * the same stream (ms) and the launch count. Class names: pty_kernel_name(0 ..
 * pty_kernel_count()-1). While enabled, pty_loss_and_direction issues its batches on the
 * caller's stream one launch after another (without profiling, consecutive batches overlap
 * on three streams), so each timed interval is one kernel running alone.
 * Single-threaded use only. Returns PTY_ERR_WORKSPACE if more than max_launches launches
 * were made (the extra ones are not timed).
 */
int pty_profile_begin(int32_t max_launches);
int pty_profile_end(double* ms_by_kernel, int32_t* launches_by_kernel, int32_t n_kinds);
const char* pty_kernel_name(int32_t id);
int pty_kernel_count(void);

/*
 * Launch-graph cache of pty_loss_and_direction (no counterpart in the reference, which
 * issues its array operations one by one from Python). The second call with the same
 * problem (every field, and the values of slice_distances), the same pointers, workspace
 * size and stream captures the call's launch sequence into a CUDA graph; later calls with
 * that key replay it with one graph launch. The graph's copies of positions_host,
 * pos_correction_host and sequence_host read those buffers when it runs, so their current
 * contents are used; the host checks of every call still run first. Not cached: calls while
 * the launch profiler records, calls on a stream that is itself being captured, 256 px
 * windows, and calls whose host buffers are pageable (their copies cannot be captured).
 * Up to 16 keys are kept (least recently used replaced). pty_graph_cache_info reports the
 * keys seen, the graphs built, the keys found uncapturable and the calls served by replay.
 */
int pty_graph_cache_info(int32_t* keys, int32_t* graphs, int32_t* uncapturable, int64_t* replays);

#ifdef __cplusplus
}
#endif

#endif /* PYPTY_GB300_H */

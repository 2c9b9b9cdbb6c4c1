/*
 * bmnd_gb300.h -- C ABI of the GB300 (sm_103a) BMND collaborative-filtering path.
 *
 * The reference (cduhme/bmnd) is a pure-Python/Numba package whose only
 * boundary is the Python function bmnd() (src/bmnd/bmndalgo.py:71-83).  This
 * library replaces the work that function does below its argument validation:
 * the reference schedule, block matching, group filtering (transforms,
 * direct-Poisson noise statistics, hard thresholding / Wiener shrinkage,
 * aggregation weights) and the weighted aggregation with the final division.
 *
 * Conventions
 *   - Plain C types only.  Volumes are C-ordered float32, patch-grid indices
 *     ("lin") are C-ordered int32 over the patch grid counts[a] = shape[a] -
 *     block[a] + 1, exactly the linear index the reference uses
 *     (src/bmnd/blockmatching.py:1112-1114).
 *   - Device pointers are CUDA device (or managed) memory owned by the caller;
 *     the library never allocates or frees caller memory and never calls
 *     cudaMalloc.  Scratch space is a caller-provided workspace whose size
 *     bmnd_workspace_bytes() reports.
 *   - "stream" is a cudaStream_t passed as uint64_t (0 = legacy default stream).
 *     Every launch of a call goes on that stream; calls return after
 *     enqueueing (device work is asynchronous) unless stated otherwise.
 *   - Every function returns BMND_OK (0) or a negative BMND_ERR_* code; the
 *     message of the last failure on the calling thread is bmnd_last_error().
 */
#ifndef BMND_GB300_H
#define BMND_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BMND_ABI_VERSION 3
#define BMND_MAX_DIMS 3
#define BMND_MAX_EDGE 8       /* largest patch edge per axis */
#define BMND_MAX_PATCH 512    /* largest patch volume */
#define BMND_MAX_STACK 32     /* largest group size */

/* return codes */
#define BMND_OK 0
#define BMND_ERR_INVALID_ARG (-1)
#define BMND_ERR_UNSUPPORTED (-2)
#define BMND_ERR_WORKSPACE (-3)
#define BMND_ERR_CUDA (-4)
#define BMND_ERR_TIMEOUT (-5)

/* block-matching distances (src/bmnd/blockmatching.py:13-16) */
#define BMND_DIST_SSD 0
#define BMND_DIST_POISSON_DEVIANCE 1
#define BMND_DIST_PEARSON 2
#define BMND_DIST_ANSCOMBE_SSD 3

/* group filters */
#define BMND_FILTER_HARD_THRESHOLD 0 /* src/bmnd/bmndalgo.py:335-559 */
#define BMND_FILTER_WIENER 1         /* src/bmnd/bmndalgo.py:760-981 */

/* transform along the group axis (src/bmnd/transforms.py:393-440) */
#define BMND_GROUP_HAAR 0 /* hierarchical Haar for power-of-two sizes, DCT-II otherwise */
#define BMND_GROUP_DCT 1  /* orthonormal DCT-II for every size */
#define BMND_GROUP_NONE 2 /* identity */

/* aggregation weight model (src/bmnd/enums.py:30-33); scope is always "patch" */
#define BMND_WEIGHT_CLASSIC 0
#define BMND_WEIGHT_VARIANCE 1
#define BMND_WEIGHT_RISK 2 /* Wiener stage only: adds (1 - a)^2 x signal power */

/* noise model of a stage */
#define BMND_NOISE_POISSON 0  /* variance volume max(count_scale * max(x, 0), floor) */
#define BMND_NOISE_GAUSSIAN 1 /* stationary noise given by cov_maps (bmndalgo.py:404-454, :826-870) */

/* matching precision */
#define BMND_MATCH_EXACT 0 /* FP32 per-term distances for every candidate */
#define BMND_MATCH_FAST 1  /* approximate screening pass + exact FP32 rescoring inside a margin */
#define BMND_MATCH_APPROX 2 /* screening distances select the group; only the selected candidates
                               are rescored exactly (Poisson deviance only; the match set may
                               differ from the exact one where the two orders disagree) */
#define BMND_MATCH_SUBSAMPLED 3 /* as BMND_MATCH_APPROX after a prescreen: the screening form on the
                                   patch's even sub-lattice for every candidate, the full form for
                                   the 4 x max_matches smallest only */

/*
 * Block matching on one patch grid.  Replaces
 * _fused_blockmatch_groups_batch_numba (src/bmnd/blockmatching.py:1045-1205)
 * as driven by blockmatch_groups (:1393-1511).
 */
typedef struct BmndMatchParams {
    int32_t ndim;                          /* 1..BMND_MAX_DIMS */
    int32_t counts[BMND_MAX_DIMS];         /* patch-grid extents */
    int32_t search_radius[BMND_MAX_DIMS];  /* window = clip(center +- radius) */
    int32_t max_matches;                   /* 1..BMND_MAX_STACK */
    int32_t min_matches;                   /* >= 1 */
    int32_t prefer_power_of_two;           /* truncate to the largest 2^j (>= min) */
    int32_t distance;                      /* BMND_DIST_* */
    int32_t stabilize_ties;                /* canonical-key comparisons (Poisson) */
    int32_t precision;                     /* BMND_MATCH_* */
    double count_scale;                    /* poisson_count_scale (> 0) */
} BmndMatchParams;

/*
 * One filtering stage (hard thresholding or Wiener) on a volume.
 * Replaces bmndalgo.py:230-633 (stage 1) and :648-1046 (stage 2).
 */
typedef struct BmndStageParams {
    int32_t ndim;                            /* 1..BMND_MAX_DIMS */
    int32_t shape[BMND_MAX_DIMS];            /* volume extents */
    int32_t block[BMND_MAX_DIMS];            /* patch extents */
    int32_t search_radius[BMND_MAX_DIMS];
    int32_t max_stack;                       /* 1..BMND_MAX_STACK */
    int32_t min_stack;
    int32_t distance;                        /* BMND_DIST_* */
    int32_t stabilize_ties;
    int32_t match_precision;                 /* BMND_MATCH_* */
    int32_t filter;                          /* BMND_FILTER_* */
    int32_t group_transform;                 /* BMND_GROUP_* */
    int32_t variance_k;                      /* exact overlap-aware planes (k) */
    int32_t weight_model;                    /* BMND_WEIGHT_* */
    int32_t windowed_synthesis;              /* weight domain windowed_synthesis */
    float match_threshold;                   /* raw distance threshold (non-SSD) */
    float ht_lambda;                         /* hard-threshold multiplier */
    float wiener_scale;                      /* mu^2 */
    float reserved0;
    double count_scale;                      /* poisson_count_scale (> 0) */
    double variance_floor;                   /* poisson_variance_floor (>= 0) */
    double eps;                              /* 1e-10 in the reference */
    /* per-axis spatial transforms, row-major edge x edge, float32 */
    float spatial_fwd[BMND_MAX_DIMS][BMND_MAX_EDGE * BMND_MAX_EDGE];
    float spatial_inv[BMND_MAX_DIMS][BMND_MAX_EDGE * BMND_MAX_EDGE];
    /* Kaiser aggregation window (C order over the patch), float32 */
    float window[BMND_MAX_PATCH];
    /* diag(S_inv^T diag(w^2) S_inv), float64; used only for windowed_synthesis */
    double spatial_metric_diag[BMND_MAX_PATCH];
    /* ---- noise model (ABI version 2) ---- */
    int32_t noise_model;                     /* BMND_NOISE_POISSON or BMND_NOISE_GAUSSIAN */
    int32_t cov_domain[BMND_MAX_DIMS];       /* Gaussian: lag domain of cov_maps (nf) */
    /* Gaussian: device table [lag][coefficient], lag C-ordered over cov_domain:
     * covariance of transformed patch coefficient c between two patches whose
     * origins differ by lag (mod cov_domain) (variance.py:1791-1886) */
    const float* cov_maps;
    /* SSD matching: device table over the search offsets (C order over
     * 2 r + 1 per axis) subtracted times ssd_gamma from every distance
     * (blockmatching.py:1133-1139), or NULL */
    const float* match_noise_ssd;
    float ssd_gamma;
    /* Poisson SSD matching: 1 subtracts ssd_gamma * sum_p count_scale *
     * (r_p + c_p) over r_p + c_p > 0 from every candidate's SSD but the
     * reference's own (blockmatching.py:1140-1145, :432-443); 0 none */
    int32_t ssd_poisson_bias;
    /* the stage's match threshold in float64: for SSD matching the threshold
     * is float32(ssd_threshold * (max - min)^2) over the matched volume
     * (blockmatching.py:168-184), evaluated on the device; the
     * reference-finite-count policy uses it as its multiplier t */
    double ssd_threshold;
    /* Poisson group-mass conservation of this stage (poisson.py:161-265,
     * bmndalgo.py:610-625 / :1023-1038): after the usual aggregation, every
     * group's coefficients are corrected along the group's constant synthesis
     * direction so that its normalised-occurrence-weighted output matches the
     * same functional of its noisy patches, the numerator is re-aggregated and
     * the estimate is numerator / denominator (no eps) */
    int32_t mass_conserve;
    /* Poisson Wiener options (bmndalgo.py:635-646, :720-741; wiener.py:24-95) */
    int32_t wiener_gain_mode;        /* BMND_GAIN_VARIANCE_SCALED (default), _CLASSIC, _NOISE_FLOOR */
    int32_t wiener_variance_source;  /* BMND_SOURCE_PILOT (default) or BMND_SOURCE_OBSERVATION */
    int32_t wiener_match_source;     /* BMND_SOURCE_PILOT (default) or BMND_SOURCE_OBSERVATION */
    /* hard-thresholding stage: soft thresholding, sign(c) max(|c| - lambda sigma, 0)
     * (bmndalgo.py:476-486) */
    int32_t soft_threshold;
    /* Poisson HT match policy (blockmatching.py:29-148, :372-428) */
    int32_t match_policy;            /* BMND_POLICY_FIXED (default), _REFERENCE_FINITE_COUNT, _CANDIDATE_STANDARDIZED */
    int32_t null_max_count;          /* poisson_ht_match_moment_max_count */
    /* device: null means then null variances of the per-voxel distance of two
     * Poisson counts with a pooled count k = 0..null_max_count, float64 */
    const double* null_moments;
    double policy_beta;              /* poisson_ht_match_structure_beta */
    double policy_power;             /* poisson_ht_match_intensity_power */
    /* one aggregation weight per group (weight_scope "group") instead of one
     * per patch */
    int32_t weight_group_scope;
    /* Haar group axis by its sum pyramid instead of the matrix product (same
     * transform, different rounding; used by the fast path) */
    int32_t fast_group_transform;
    /* covariance-aware exact group weighting (bmndalgo.py:363-377, :491-503,
     * :752-758, :913-927; wiener.py:638-822): with weight_group_scope,
     * windowed_synthesis and variance_k > 0, the group's weight is
     * 1 / (risk + eps) with the noise risk of the first min(k, n) planes
     * summed exactly over the group's union voxels,
     *   sum_u V_u sum_g (a_g o c_u[g])^T SM (a_g o c_u[g]),
     * c_u[g] the coefficients of plane g that voxel u reaches, a the
     * attenuation and SM = S_inv^T diag(w^2) S_inv; the other planes and the
     * bias term use the coefficient-metric diagonal.  Patches of at most 128
     * voxels. */
    int32_t exact_risk_weights;
    /* Gaussian noise with exact_risk_weights: the (white) noise variance of
     * every union voxel (variance.py:1451-1496) */
    float exact_source_variance;
} BmndStageParams;

#define BMND_GAIN_VARIANCE_SCALED 0
#define BMND_GAIN_CLASSIC 1
#define BMND_GAIN_NOISE_FLOOR 2
#define BMND_POLICY_FIXED 0
#define BMND_POLICY_REFERENCE_FINITE_COUNT 1
#define BMND_POLICY_CANDIDATE_STANDARDIZED 2
#define BMND_SOURCE_PILOT 0
#define BMND_SOURCE_OBSERVATION 1

/* ABI version this library was built with (BMND_ABI_VERSION). */
int32_t bmnd_abi_version(void);

/* Message of the last failure on the calling thread ("" if none). */
const char* bmnd_last_error(void);

/* Kernel launches this library has made since it was loaded (all threads);
 * the difference of two readings counts the launches between them. */
int32_t bmnd_launch_count(uint64_t* count);

/* Device allocations this library has made itself since it was loaded (a
 * scratch array allocated on the stream when the caller's workspace has no
 * room for it; bmnd_stage_noalloc never allocates). */
int32_t bmnd_device_alloc_count(uint64_t* count);

/* *direct = 1 when `device` reads pageable host memory through the host's page
 * tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables, e.g. a Grace host
 * over NVLink-C2C): copies from and to ordinary host memory then run at the
 * link's rate and need no page-locked staging buffer; else 0. */
int32_t bmnd_host_memory_direct(int32_t device, int32_t* direct);

/*
 * Host-only.  GENERATED reference schedule: replaces get_reference_schedule
 * with mode="generated" (src/bmnd/shifts.py:405-423, :519-576, :229-266).
 * Writes up to `capacity` rows of reference_abs / reference_shifted / shift
 * (each n x ndim int32, any may be NULL) and the total count to *out_count.
 * Call with capacity 0 to size the buffers.
 */
int32_t bmnd_reference_schedule(int32_t ndim, const int32_t* counts, const int32_t* block,
                                const int32_t* step, double shift_density,
                                int32_t schedule_density, int32_t* out_abs,
                                int32_t* out_shifted, int32_t* out_shift, int64_t capacity,
                                int64_t* out_count);

/*
 * Block matching over an explicit patch table d_patches (n_patches x
 * patch_vol float32, row = patch-grid lin).  Replaces blockmatch_groups
 * (src/bmnd/blockmatching.py:1393-1511).  d_refs: n_refs x ndim int32 patch-grid
 * positions; d_thresholds: n_refs float32 raw thresholds.  Outputs (device):
 * d_sel n_refs x max_matches int32 (selected lins, reference first, -1
 * padded), d_count n_refs int32 (final_count), d_accepted n_refs int32
 * (accepted_count).
 */
int32_t bmnd_blockmatch_patches(const BmndMatchParams* params, const float* d_patches,
                                int32_t patch_vol, const int32_t* d_refs, int64_t n_refs,
                                const float* d_thresholds, int32_t* d_sel, int32_t* d_count,
                                int32_t* d_accepted, uint64_t stream);

/*
 * Block matching where the patch at grid position q is the block of
 * d_volume starting at q (the reference's extract_patches_strided view,
 * src/bmnd/utils.py:15-31, without materialising it).  Same outputs as
 * bmnd_blockmatch_patches; `block` gives the patch extents, params->counts
 * must equal shape - block + 1.
 */
int32_t bmnd_blockmatch_volume(const BmndMatchParams* params, const float* d_volume,
                               const int32_t* shape, const int32_t* block,
                               const int32_t* d_refs, int64_t n_refs,
                               const float* d_thresholds, int32_t* d_sel, int32_t* d_count,
                               int32_t* d_accepted, uint64_t stream);

/*
 * bmnd_blockmatch_volume with the SSD noise-bias correction of
 * blockmatch_groups(gaussian_noise_ssd=..., gamma=...) (blockmatching.py:1133-1139):
 * every SSD distance minus gamma * d_noise_ssd[offset], the offset of the
 * candidate from the reference in C order over 2 * search_radius + 1 per axis.
 * params->distance must be BMND_DIST_SSD.
 */
int32_t bmnd_blockmatch_volume_biased(const BmndMatchParams* params, const float* d_volume,
                                      const int32_t* shape, const int32_t* block,
                                      const int32_t* d_refs, int64_t n_refs,
                                      const float* d_thresholds, const float* d_noise_ssd, float gamma,
                                      int32_t* d_sel, int32_t* d_count, int32_t* d_accepted,
                                      uint64_t stream);

/*
 * bmnd_blockmatch_volume with the Poisson SSD noise-bias correction of
 * blockmatch_groups(poisson_gamma=True, gamma=...) (blockmatching.py:1140-1145,
 * :432-443): every candidate's SSD but the reference's own minus
 * gamma * sum_p count_scale * (r_p + c_p) over r_p + c_p > 0, float32 in
 * patch order.  params->distance must be BMND_DIST_SSD and
 * params->count_scale the profile's poisson_count_scale.
 */
int32_t bmnd_blockmatch_volume_poisson_biased(const BmndMatchParams* params, const float* d_volume,
                                              const int32_t* shape, const int32_t* block,
                                              const int32_t* d_refs, int64_t n_refs,
                                              const float* d_thresholds, float gamma,
                                              int32_t* d_sel, int32_t* d_count, int32_t* d_accepted,
                                              uint64_t stream);

/*
 * Workspace bytes bmnd_stage() needs for `params` and n_refs references.
 */
int32_t bmnd_stage_workspace_bytes(const BmndStageParams* params, int64_t n_refs,
                                   uint64_t* out_bytes);

/*
 * One filtering stage on the device.
 *   d_noisy     observation (shape), float32
 *   d_pilot     stage-1 estimate for the Wiener stage (matching source,
 *               Wiener reference coefficients and variance source), NULL for
 *               hard thresholding
 *   d_refs      n_refs x ndim int32 reference positions (patch grid)
 *   d_out       estimate: where(den > 0, num / (den + eps), noisy)
 *               (bmndalgo.py:626-631, :1039-1044)
 *   d_sel/d_count/d_accepted  optional (NULL) copies of the match sets, laid
 *               out as in bmnd_blockmatch_patches
 * The workspace must be at least bmnd_stage_workspace_bytes() bytes and
 * 256-byte aligned.  d_refs positions must lie on the patch grid (0 <= ref[d]
 * < shape[d] - block[d] + 1, as bmnd_reference_schedule() makes them); they are
 * not checked on the device.
 */
int32_t bmnd_stage(const BmndStageParams* params, const float* d_noisy, const float* d_pilot,
                   const int32_t* d_refs, int64_t n_refs, float* d_out, int32_t* d_sel,
                   int32_t* d_count, int32_t* d_accepted, void* d_workspace,
                   uint64_t workspace_bytes, uint64_t stream);

/*
 * bmnd_stage() plus the stage's sigma map (the reference's return_sigma_map,
 * bmndalgo.py:253-256, :576-597, :874-875, :1001-1010, :1048-1062): every
 * group's noise sigma is aggregated with the weights of its estimate, per
 * coefficient for hard thresholding and as the group mean for Wiener, and
 * divided by the aggregated weight; voxels no patch covers get global_sigma.
 * d_sel/d_count/d_accepted are optional as in bmnd_stage().  The workspace is
 * bmnd_stage_sigma_workspace_bytes() bytes, 256-byte aligned.
 */
int32_t bmnd_stage_sigma_workspace_bytes(const BmndStageParams* params, int64_t n_refs,
                                         uint64_t* out_bytes);
int32_t bmnd_stage_sigma(const BmndStageParams* params, const float* d_noisy, const float* d_pilot,
                         const int32_t* d_refs, int64_t n_refs, float* d_out, float* d_sigma_map,
                         float global_sigma, int32_t* d_sel, int32_t* d_count, int32_t* d_accepted,
                         void* d_workspace, uint64_t workspace_bytes, uint64_t stream);

/*
 * Both stages back to back (hard thresholding, then Wiener on the pilot),
 * i.e. the body of bmnd() for a direct-Poisson profile.  ht/wiener are the
 * stage parameters, refs_ht/refs_wiener their schedules; d_ht_out receives
 * the stage-1 estimate (required: it is the Wiener pilot), d_out the result.
 * The workspace must hold max(stage workspaces).
 */
int32_t bmnd_run(const BmndStageParams* ht, const BmndStageParams* wiener,
                 const float* d_noisy, const int32_t* d_refs_ht, int64_t n_refs_ht,
                 const int32_t* d_refs_wiener, int64_t n_refs_wiener, float* d_ht_out,
                 float* d_out, void* d_workspace, uint64_t workspace_bytes, uint64_t stream);

/*
 * Group probe: filter explicit groups and return their intermediate arrays
 * instead of aggregating them.  Replaces, for testing and inspection, the body
 * of the reference's per-group closures filter_ht_group / filter_wiener_group
 * (src/bmnd/bmndalgo.py:335-559, :760-981): the forward transform
 * (transforms.py:209-255), the noise std (variance.py:1634-1711), the
 * hard-threshold mask (poisson.py:30-46) or Wiener gain (wiener.py:78-95), the
 * aggregation weights (aggregationweights.py:633-653) and the inverse
 * transform.  Group i has d_count[i] members d_sel[i * max_stack + g]
 * (patch-grid lins, 0 <= lin < prod(shape - block + 1)).  Outputs (device, any
 * may be NULL; rows of members >= d_count[i] are left untouched):
 *   d_coef, d_sigma, d_atten, d_filt  n_groups x max_stack x P float32
 *   d_weights                          n_groups x max_stack float32
 * params->mass_conserve must be 0.  The workspace (256-byte aligned) holds
 * bmnd_group_probe_workspace_bytes() bytes.  The call synchronises the stream
 * and returns BMND_ERR_INVALID_ARG if a group had a member outside the patch
 * grid, more than max_stack members, or a union box the kernel's shared-memory
 * layout cannot hold (such groups are skipped, their outputs untouched).
 */
int32_t bmnd_group_probe_workspace_bytes(const BmndStageParams* params, uint64_t* out_bytes);
int32_t bmnd_group_probe(const BmndStageParams* params, const float* d_noisy, const float* d_pilot,
                         const int32_t* d_sel, const int32_t* d_count, int64_t n_groups, float* d_coef,
                         float* d_sigma, float* d_atten, float* d_weights, float* d_filt, void* d_workspace,
                         uint64_t workspace_bytes, uint64_t stream);

/*
 * Allocation-free variant of bmnd_stage().  It has no counterpart in the
 * reference.  It is meant for callers that may not allocate device memory
 * after start-up: hosts whose memory pool owns the whole device (acquisition
 * pipelines that reserve all memory up front), or bindings that have no way
 * to call into the CUDA allocator.  The caller still passes inputs and
 * outputs; the stage's scratch space (aggregation arrays, match table) is a
 * fixed array of BMND_STATIC_SCRATCH_BYTES compiled into
 * this library, held by every GPU that loads it until the process exits.
 *   - A stage needing more scratch than that is rejected with
 *     BMND_ERR_WORKSPACE before any device work (see
 *     bmnd_stage_workspace_bytes for the requirement).
 *   - The first call on a device looks up the array's device address (once
 *     per CUDA context, with that device current; a context re-created after
 *     cudaDeviceReset is looked up again); make that first call before any
 *     stream capture.
 *   - Precision BMND_MATCH_APPROX and BMND_MATCH_SUBSAMPLED stages keep their
 *     per-voxel screening arrays in the same array, as bmnd_stage keeps them
 *     in its workspace, so both entry points run the same kernels.
 *   - d_refs holds reference positions on the patch grid (0 <= ref[d] <
 *     shape[d] - block[d] + 1), as from bmnd_reference_schedule(); positions
 *     outside it are not checked on the device.
 *   - Every call shares the one array and leaves its contents behind; the
 *     accumulators are cleared at the start of each call.  Calls whose device
 *     work overlaps (other streams, other host threads) race on the array.
 * This function performs no cudaMalloc / cudaFree and calls no allocating
 * library routine.
 */
#define BMND_STATIC_SCRATCH_BYTES (64ull << 20)
int32_t bmnd_stage_noalloc(const BmndStageParams* params, const float* d_noisy,
                           const float* d_pilot, const int32_t* d_refs, int64_t n_refs,
                           float* d_out, uint64_t stream);

/*
 * Measurement support (no counterpart in the reference): the issue rates, per
 * second, of the two units that bound this path's kernels on the current
 * device at its current clock: MUFU lg2.approx (one per Poisson-deviance voxel
 * term in the screening forms of matching) and FP32 fused multiply-add (the
 * exact variance).  Runs two short kernels of independent dependency chains on
 * every SM and synchronises the stream; d_sink is a device buffer of at least
 * 4 bytes.
 */
int32_t bmnd_unit_rates(double* lg2_per_s, double* ffma_per_s, void* d_sink, uint64_t stream);

/*
 * Measurement support (no counterpart in the reference): for each of `count`
 * configurations, the mean clocks one tcgen05.mma kind::f16 (BF16 in, FP32
 * accumulate, M = 128, N = n_cols[i], K = 16, operands in shared memory) takes
 * on every SM when issuers[i] threads of a CTA (1..4, one per warp) issue them
 * back to back into accumulators of their own.  n_cols[i] is 16..256 in steps
 * of 16 and n_cols[i] x issuers[i] <= 512.  d_scratch: device memory of at
 * least 8 x (SM count + 1) bytes.  Synchronises the stream.
 */
int32_t bmnd_mma_rates(int32_t count, const int32_t* n_cols, const int32_t* issuers, double* clocks_per_mma,
                       void* d_scratch, uint64_t stream);

/* ------------------------------------------------------------------------
 * Learned stage-1 pilot (fast path).  No counterpart in the reference: a
 * residual 3x3 (2-D) or 3x3x3 (3-D) convolution net in the Anscombe domain,
 *   a = 2 sqrt(max(x, 0) + 3/8),  h_1 = relu(W_0 * a + b_0),
 *   h_l = relu(W_{l-1} * h_{l-1} + b_{l-1}),  y = a + W_{L-1} * h_{L-1} + b_{L-1},
 *   pilot = max((y / 2)^2 - 3/8, 0),
 * with BF16 weights and hidden activations and FP32 accumulation; the
 * C -> C layers run on the tensor cores.  Parameters are one flat FP32
 * vector, layer by layer: W_l[tap][ci][co] (taps in C order over offsets
 * -1..1) then b_l[co]; layer 0 has ci = 1, layer L-1 has co = 1.
 * ------------------------------------------------------------------------ */
typedef struct {
    int32_t ndim;     /* 2 or 3 */
    int32_t channels; /* hidden channels: 32 or 48 */
    int32_t layers;   /* convolution layers, 3..32 */
    int32_t batch;    /* volumes (images) in the batch */
    int32_t shape[3]; /* D, H, W (3-D) or H, W (2-D); the batch is C-ordered before them */
} BmndPilotNet;

/* Number of FP32 parameters. */
int32_t bmnd_pilotnet_param_count(const BmndPilotNet* net, int64_t* count);
/* Bytes of the packed (BF16, fragment-ordered) weights bmnd_pilotnet_pack writes. */
int32_t bmnd_pilotnet_packed_bytes(const BmndPilotNet* net, uint64_t* bytes);
/* Workspace bytes for inference (training = 0) or a gradient pass (training = 1). */
int32_t bmnd_pilotnet_workspace_bytes(const BmndPilotNet* net, int32_t training, uint64_t* bytes);
/* Round the FP32 parameters to BF16 and lay them out for the kernels. */
int32_t bmnd_pilotnet_pack(const BmndPilotNet* net, const float* d_params, void* d_packed, uint64_t stream);
/* Inference: d_pilot (count domain) and/or d_y (Anscombe-domain output), either may be NULL. */
int32_t bmnd_pilotnet_forward(const BmndPilotNet* net, const void* d_packed, const float* d_noisy,
                              float* d_pilot, float* d_y, void* d_workspace, uint64_t workspace_bytes,
                              uint64_t stream);
/* Loss mean((y - A(target))^2) with A the Anscombe transform, and its gradient
 * with respect to every parameter (flat, same layout as the parameters). */
int32_t bmnd_pilotnet_gradient(const BmndPilotNet* net, const void* d_packed, const float* d_noisy,
                               const float* d_target, float* d_grad, double* d_loss, void* d_workspace,
                               uint64_t workspace_bytes, uint64_t stream);
/* Status of the most recent forward or gradient call that used d_workspace:
 * synchronises the stream, then BMND_OK, or BMND_ERR_TIMEOUT when a bounded
 * wait of a tensor-core layer ran out (the outputs are then incomplete). */
int32_t bmnd_pilotnet_status(const BmndPilotNet* net, const void* d_workspace, uint64_t stream);
/* Engine of the C -> C layers, process-wide: BMND_CONV_TCGEN05 (default: one
 * tcgen05.mma per 128-voxel tile and K = 16 slice, accumulator in tensor
 * memory) or BMND_CONV_MMA_SYNC (warp-level mma.sync, kept for comparison). */
#define BMND_CONV_TCGEN05 0
#define BMND_CONV_MMA_SYNC 1
int32_t bmnd_pilotnet_set_conv_engine(int32_t engine);

/* Failure-detection test hook (process-wide): with ns > 0 (at most 1e9), every
 * following tensor-core layer launch first waits up to ns nanoseconds on an
 * mbarrier that nothing completes.  The wait runs out before any copy or
 * product is issued; the launch stops as on a real timeout, frees its tensor
 * memory, and bmnd_pilotnet_status then reports BMND_ERR_TIMEOUT.  0, the
 * default, turns it off. */
int32_t bmnd_pilotnet_set_wait_probe(uint64_t ns);
int32_t bmnd_pilotnet_get_conv_engine(int32_t* engine);
/* Residual check of a pilot, per tile of edge `edge` (cubes in 3-D, squares in
 * 2-D; shape as in BmndPilotNet): d_out[3 * tile + (0, 1, 2)] = observed Poisson
 * deviance sum_v 2 [x ln(x / mu) - (x - mu)] of the input x against the pilot
 * mu, and its expectation and variance under Poisson noise of mean mu, read from
 * d_table (n_table expectations then n_table variances, at ln mu = ln_mu0 +
 * i * d_ln).  Tiles are ordered x fastest, then y, z, batch. */
int32_t bmnd_pilot_tile_deviance(int32_t ndim, int32_t batch, const int32_t* shape, int32_t edge,
                                 const float* d_noisy, const float* d_pilot, const float* d_table,
                                 int32_t n_table, float ln_mu0, float d_ln, double* d_out, uint64_t stream);
/* One Adam step (bias-corrected, step counts from 1) on the gradient scaled to
 * an L2 norm of at most clip_norm (clip_norm <= 0: no clipping); d_sumsq is one
 * double of scratch that receives the squared gradient norm. */
int32_t bmnd_pilotnet_adam(int64_t n, float* d_params, const float* d_grad, float* d_m, float* d_v,
                           int32_t step, float lr, float beta1, float beta2, float eps, float clip_norm,
                           double* d_sumsq, uint64_t stream);

#ifdef __cplusplus
}
#endif

#endif /* BMND_GB300_H */

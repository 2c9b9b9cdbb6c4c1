// abi.cu -- the extern "C" entry points declared in include/bmnd_gb300.h.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <set>
#include <string>
#include <vector>

#include "bmnd_common.cuh"

namespace bmnd {

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
std::atomic<uint64_t> g_device_allocs{0};
}

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void note_device_alloc() { g_device_allocs.fetch_add(1, std::memory_order_relaxed); }
void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
int32_t fail(int32_t code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
int32_t cuda_fail(cudaError_t err, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) + ")";
    return BMND_ERR_CUDA;
}

int64_t group_filter_smem_bytes(const BmndStageParams& sp);

namespace {
struct ShapeKey {
    int dev;
    const void* fn;
    int threads;
    size_t smem;
    bool fit;
    bool operator<(const ShapeKey& o) const {
        return std::tie(dev, fn, threads, smem, fit) < std::tie(o.dev, o.fn, o.threads, o.smem, o.fit);
    }
};
struct FnState {
    size_t smem_limit = 0;  // the kernel's dynamic shared-memory limit as set
    int carveout = -1;      // its preferred carveout as set
};
std::mutex g_shape_mutex;
std::map<ShapeKey, std::pair<int, int>> g_shapes;       // -> (resident CTAs per SM, carveout)
std::map<std::pair<int, const void*>, FnState> g_fns;  // per device and kernel
std::map<int, int> g_sm_count;                          // per device
}  // namespace

int32_t kernel_residency(const void* fn, int threads, size_t smem, bool fit_carveout, int* per_sm, int* sms) {
    int dev = 0;
    BMND_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> guard(g_shape_mutex);
    auto sit = g_sm_count.find(dev);
    if (sit == g_sm_count.end()) {
        int n = 0;
        BMND_CUDA_TRY(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
        sit = g_sm_count.emplace(dev, n).first;
    }
    FnState& st = g_fns[{dev, fn}];
    if (smem > st.smem_limit) {
        BMND_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        st.smem_limit = smem;
    }
    const ShapeKey key{dev, fn, threads, smem, fit_carveout};
    auto it = g_shapes.find(key);
    if (it == g_shapes.end()) {
        int resident = 0, pct = -1;
        if (fit_carveout) {
            BMND_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
            st.carveout = 100;
        }
        BMND_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, fn, threads, smem));
        if (fit_carveout && resident > 0) {
            int smem_sm = 0;
            BMND_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
            const int64_t want = static_cast<int64_t>(resident) * (static_cast<int64_t>(smem) + 1024);
            pct = smem_sm > 0 ? static_cast<int>((want * 100 + smem_sm - 1) / smem_sm) : 100;
            if (pct > 100) pct = 100;
        }
        it = g_shapes.emplace(key, std::make_pair(resident, pct)).first;
    }
    const int pct = it->second.second;
    if (fit_carveout && pct >= 0 && pct != st.carveout) {
        BMND_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
        st.carveout = pct;
    }
    *per_sm = it->second.first;
    *sms = sit->second;
    return BMND_OK;
}

namespace {

// ---------------------------------------------------------------------------
// GENERATED reference schedule (src/bmnd/shifts.py:229-266, :519-576)
// ---------------------------------------------------------------------------
std::vector<int> axis_shifts(int block, int step, bool allow_multiple, double density) {
    if (!allow_multiple || block < 3 || step < 1 || step > block) return {0};
    double safe = density > 0.0 ? density : 0.0;
    int count = static_cast<int>(std::ceil(safe * (block - 1) / static_cast<double>(step)));
    count = std::max(count, 1);
    count = std::min(count, block);
    if (count == 1) return {0};
    // np.linspace(0, block - 1, count), rounded half to even, plus 0, sorted unique
    std::set<int> values{0};
    double stop = static_cast<double>(block - 1);
    double delta = stop / static_cast<double>(count - 1);
    for (int i = 0; i < count; ++i) {
        double v = (i == count - 1) ? stop : i * delta;
        values.insert(static_cast<int>(std::nearbyint(v)));
    }
    return std::vector<int>(values.begin(), values.end());
}

int32_t validate_stage(const BmndStageParams& sp) {
    if (sp.ndim < 1 || sp.ndim > BMND_MAX_DIMS) return fail(BMND_ERR_INVALID_ARG, "ndim must be 1..3");
    int P = 1;
    int64_t vox = 1;
    for (int d = 0; d < sp.ndim; ++d) {
        if (sp.shape[d] < 1) return fail(BMND_ERR_INVALID_ARG, "shape must be positive");
        if (sp.block[d] < 1 || sp.block[d] > sp.shape[d])
            return fail(BMND_ERR_INVALID_ARG, "block must be in [1, shape]");
        if (sp.block[d] > BMND_MAX_EDGE) return fail(BMND_ERR_UNSUPPORTED, "patch edge above 8");
        if (sp.search_radius[d] < 0) return fail(BMND_ERR_INVALID_ARG, "search radius must be >= 0");
        if (2 * static_cast<int64_t>(sp.search_radius[d]) + sp.block[d] > 1000)
            return fail(BMND_ERR_UNSUPPORTED, "search window too large");
        P *= sp.block[d];
        vox *= sp.shape[d];
    }
    if (P > BMND_MAX_PATCH) return fail(BMND_ERR_UNSUPPORTED, "patch volume above 512");
    if (vox > 0x7fffffffLL) return fail(BMND_ERR_UNSUPPORTED, "volume above 2^31 voxels");
    if (sp.max_stack < 1 || sp.max_stack > BMND_MAX_STACK)
        return fail(BMND_ERR_UNSUPPORTED, "max_stack must be in [1, 32]");
    if (sp.min_stack < 1 || sp.min_stack > sp.max_stack)
        return fail(BMND_ERR_INVALID_ARG, "min_stack must be in [1, max_stack]");
    if (sp.distance < 0 || sp.distance > 3) return fail(BMND_ERR_INVALID_ARG, "unknown distance");
    if (sp.filter != BMND_FILTER_HARD_THRESHOLD && sp.filter != BMND_FILTER_WIENER)
        return fail(BMND_ERR_INVALID_ARG, "unknown filter");
    if (sp.group_transform < 0 || sp.group_transform > 2)
        return fail(BMND_ERR_INVALID_ARG, "unknown group transform");
    if (sp.variance_k < 0) return fail(BMND_ERR_INVALID_ARG, "variance_k must be >= 0");
    if (sp.weight_model != BMND_WEIGHT_CLASSIC && sp.weight_model != BMND_WEIGHT_VARIANCE &&
        sp.weight_model != BMND_WEIGHT_RISK)
        return fail(BMND_ERR_INVALID_ARG, "unknown weight model");
    if (sp.weight_model == BMND_WEIGHT_RISK && sp.filter != BMND_FILTER_WIENER)
        return fail(BMND_ERR_INVALID_ARG, "risk weights apply to the Wiener stage");
    if (!(sp.count_scale > 0.0) || !std::isfinite(sp.count_scale))
        return fail(BMND_ERR_INVALID_ARG, "count_scale must be finite and positive");
    if (!(sp.variance_floor >= 0.0)) return fail(BMND_ERR_INVALID_ARG, "variance_floor must be >= 0");
    if (!(sp.eps > 0.0)) return fail(BMND_ERR_INVALID_ARG, "eps must be positive");
    if (!(sp.match_threshold >= 0.0f) || !std::isfinite(sp.match_threshold))
        return fail(BMND_ERR_INVALID_ARG, "match threshold must be finite and >= 0");
    if (sp.wiener_gain_mode < 0 || sp.wiener_gain_mode > 2) return fail(BMND_ERR_INVALID_ARG, "unknown gain mode");
    if (sp.match_policy < 0 || sp.match_policy > 2) return fail(BMND_ERR_INVALID_ARG, "unknown match policy");
    if (sp.match_policy != BMND_POLICY_FIXED) {
        if (!sp.null_moments || sp.null_max_count < 1)
            return fail(BMND_ERR_INVALID_ARG, "the match policy needs the null moment table");
        if (sp.distance == BMND_DIST_SSD)
            return fail(BMND_ERR_INVALID_ARG, "the match policy needs a Poisson distance");
    }
    if ((sp.wiener_variance_source != 0 && sp.wiener_variance_source != 1) ||
        (sp.wiener_match_source != 0 && sp.wiener_match_source != 1))
        return fail(BMND_ERR_INVALID_ARG, "unknown Wiener source");
    if (sp.noise_model != BMND_NOISE_POISSON && sp.noise_model != BMND_NOISE_GAUSSIAN)
        return fail(BMND_ERR_INVALID_ARG, "unknown noise model");
    if (sp.noise_model == BMND_NOISE_GAUSSIAN) {
        if (!sp.cov_maps) return fail(BMND_ERR_INVALID_ARG, "Gaussian noise needs the covariance maps");
        for (int d = 0; d < sp.ndim; ++d)
            if (sp.cov_domain[d] < 1) return fail(BMND_ERR_INVALID_ARG, "covariance domain must be positive");
    }
    if ((sp.match_noise_ssd || sp.ssd_poisson_bias) && sp.distance != BMND_DIST_SSD)
        return fail(BMND_ERR_INVALID_ARG, "the noise-bias correction applies to SSD matching only");
    if (sp.ssd_poisson_bias != 0 && sp.ssd_poisson_bias != 1)
        return fail(BMND_ERR_INVALID_ARG, "ssd_poisson_bias must be 0 or 1");
    if (sp.ssd_poisson_bias && (sp.noise_model != BMND_NOISE_POISSON || sp.match_noise_ssd))
        return fail(BMND_ERR_INVALID_ARG, "the Poisson SSD noise bias needs the Poisson model and no bias table");
    if ((sp.match_noise_ssd || sp.ssd_poisson_bias) && (!(sp.ssd_gamma >= 0.0f) || !std::isfinite(sp.ssd_gamma)))
        return fail(BMND_ERR_INVALID_ARG, "gamma must be finite and non-negative");
    if (sp.distance == BMND_DIST_SSD && (!(sp.ssd_threshold >= 0.0) || !std::isfinite(sp.ssd_threshold)))
        return fail(BMND_ERR_INVALID_ARG, "SSD threshold multiplier must be finite and >= 0");
    if (sp.exact_risk_weights != 0 && sp.exact_risk_weights != 1)
        return fail(BMND_ERR_INVALID_ARG, "exact_risk_weights must be 0 or 1");
    if (sp.exact_risk_weights) {
        if (!sp.weight_group_scope || !sp.windowed_synthesis || sp.variance_k <= 0 ||
            sp.weight_model == BMND_WEIGHT_CLASSIC)
            return fail(BMND_ERR_INVALID_ARG,
                        "exact risk weights need group scope, windowed synthesis, variance or risk weights and k > 0");
        if (P > 128) return fail(BMND_ERR_UNSUPPORTED, "exact risk weights need patches of at most 128 voxels");
        if (sp.noise_model == BMND_NOISE_GAUSSIAN &&
            (!(sp.exact_source_variance >= 0.0f) || !std::isfinite(sp.exact_source_variance)))
            return fail(BMND_ERR_INVALID_ARG, "exact_source_variance must be finite and >= 0");
    }
    if (group_filter_smem_bytes(sp) > 227 * 1024)
        return fail(BMND_ERR_UNSUPPORTED, "profile needs more than 227 KB of shared memory per group");
    return BMND_OK;
}

// Stages aggregate deterministically (aggregate.cu) unless they conserve group
// mass (whose second pass re-aggregates against the first pass's denominator)
// or their patches exceed 128 voxels; the others, and the sigma-map entry
// point, add into float64 volumes with atomics.
bool deterministic_aggregation(const BmndStageParams& sp) {
    return sp.mass_conserve == 0 && patch_volume(sp) <= 128;
}

struct StageWorkspace {
    double* num;  // float64 accumulators of the atomic aggregation, or null
    double* den;
    char* agg_base;  // deterministic aggregation region, or null
    AggregationLayout agg;
    int32_t* sel;
    int32_t* count;
    int32_t* accepted;
    float* st;  // P x kron_stride(P) Kronecker table of the patch transforms
    uint32_t* mm;  // SSD threshold: order bits of the matched volume's min and max
    float* thr;    // SSD threshold, computed on the device
    float* thr_ref;  // per-reference thresholds (reference-finite-count policy)
    float* aux;      // approximate screening form: per-voxel arrays of the matched volume
    int64_t aux_floats;
    char* ssd;       // tensor-core SSD matching: norms, screening distances, tiles
    uint64_t ssd_bytes;
    uint64_t bytes;
};

uint64_t align256(uint64_t v) { return (v + 255) & ~uint64_t(255); }

BmndMatchParams match_params_of(const BmndStageParams& sp);

StageWorkspace carve(const BmndStageParams& sp, int64_t n_refs, void* base) {
    StageWorkspace w{};
    uint64_t vox = static_cast<uint64_t>(volume_voxels(sp));
    uint64_t off = 0;
    auto take = [&](uint64_t bytes) {
        uint64_t o = off;
        off += align256(bytes);
        return o;
    };
    const bool det = deterministic_aggregation(sp);
    if (det) w.agg = aggregation_layout(sp, n_refs);
    uint64_t o_num = det ? 0 : take(8 * vox);
    uint64_t o_den = det ? 0 : take(8 * vox);
    uint64_t o_agg = det ? take(w.agg.bytes) : 0;
    uint64_t o_sel = take(4ull * n_refs * sp.max_stack);
    uint64_t o_cnt = take(4ull * n_refs);
    uint64_t o_acc = take(4ull * n_refs);
    const uint64_t P = static_cast<uint64_t>(patch_volume(sp));
    // the Kronecker table, the risk metric SM (exact risk weights), the group matrices
    uint64_t o_st = take(4ull * stage_table_floats(static_cast<int>(P)));
    uint64_t o_mm = take(16);
    uint64_t o_tr = take(sp.match_policy == BMND_POLICY_REFERENCE_FINITE_COUNT ? 4ull * n_refs : 16);
    const BmndMatchParams mp = match_params_of(sp);
    w.aux_floats = approx_scratch_floats(mp, sp.shape, sp.block);
    uint64_t o_aux = take(w.aux_floats > 0 ? 4ull * static_cast<uint64_t>(w.aux_floats) : 16);
    w.ssd_bytes = ssd_tc_scratch_bytes(mp, sp.block, n_refs, sp.ssd_poisson_bias != 0);
    uint64_t o_ssd = take(w.ssd_bytes > 0 ? w.ssd_bytes : 16);
    w.bytes = off;
    if (base) {
        char* b = static_cast<char*>(base);
        w.num = det ? nullptr : reinterpret_cast<double*>(b + o_num);
        w.den = det ? nullptr : reinterpret_cast<double*>(b + o_den);
        w.agg_base = det ? b + o_agg : nullptr;
        w.sel = reinterpret_cast<int32_t*>(b + o_sel);
        w.count = reinterpret_cast<int32_t*>(b + o_cnt);
        w.accepted = reinterpret_cast<int32_t*>(b + o_acc);
        w.st = reinterpret_cast<float*>(b + o_st);
        w.mm = reinterpret_cast<uint32_t*>(b + o_mm);
        w.thr = reinterpret_cast<float*>(b + o_mm + 8);
        w.thr_ref = reinterpret_cast<float*>(b + o_tr);
        w.aux = w.aux_floats > 0 ? reinterpret_cast<float*>(b + o_aux) : nullptr;
        w.ssd = w.ssd_bytes > 0 ? b + o_ssd : nullptr;
    }
    return w;
}

BmndMatchParams match_params_of(const BmndStageParams& sp) {
    BmndMatchParams mp{};
    // SSD matching of a 2-D image: the tensor-core screening with exact
    // rescoring gives the exact kernel's match sets (see ssd_select_kernel), so
    // exact requests take it.  In 3-D the exact kernel stays: a tile's union box
    // of candidates is 8x a reference's window (about 6 % of the tensor
    // products are used), and on a denoised pilot the screening bound leaves
    // most of the window to rescore; measured at 256^3 the whole Gaussian call
    // took 810 ms with the screening and 780 ms without.
    mp.ndim = sp.ndim;
    for (int d = 0; d < sp.ndim; ++d) {
        mp.counts[d] = sp.shape[d] - sp.block[d] + 1;
        mp.search_radius[d] = sp.search_radius[d];
    }
    mp.max_matches = sp.max_stack;
    mp.min_matches = sp.min_stack;
    mp.prefer_power_of_two = 1;
    mp.distance = sp.distance;
    mp.stabilize_ties = sp.stabilize_ties;
    mp.precision = sp.match_precision;
    if (sp.distance == BMND_DIST_SSD && sp.match_precision == BMND_MATCH_EXACT && !sp.ssd_poisson_bias &&
        sp.ndim == 2)
        mp.precision = BMND_MATCH_FAST;
    mp.count_scale = sp.count_scale;
    return mp;
}

// bytes of the stage workspace followed by the float64 numerator, denominator
// and sigma-map numerator of the atomic aggregation the sigma maps use
uint64_t sigma_workspace_bytes(const BmndStageParams& sp, int64_t n_refs) {
    return carve(sp, n_refs, nullptr).bytes + 3 * align256(8ull * static_cast<uint64_t>(volume_voxels(sp)));
}

int32_t run_stage(const BmndStageParams& sp, const float* noisy, const float* pilot,
                  const int32_t* refs, int64_t n_refs, float* out, int32_t* sel, int32_t* count,
                  int32_t* accepted, void* ws, uint64_t ws_bytes, cudaStream_t stream,
                  float* sigma_out = nullptr, float global_sigma = 0.0f, bool allow_alloc = true) {
    int32_t rc = validate_stage(sp);
    if (rc) return rc;
    if (!noisy || !out) return fail(BMND_ERR_INVALID_ARG, "noisy and out are required");
    if (sp.filter == BMND_FILTER_WIENER && !pilot)
        return fail(BMND_ERR_INVALID_ARG, "the Wiener stage needs the pilot estimate");
    if (n_refs < 0 || (n_refs > 0 && !refs)) return fail(BMND_ERR_INVALID_ARG, "bad reference list");
    StageWorkspace need = carve(sp, n_refs, nullptr);
    const uint64_t need_bytes = sigma_out ? sigma_workspace_bytes(sp, n_refs) : need.bytes;
    if (!ws || ws_bytes < need_bytes) return fail(BMND_ERR_WORKSPACE, "workspace too small");
    if (reinterpret_cast<uintptr_t>(ws) % 256 != 0)
        return fail(BMND_ERR_INVALID_ARG, "workspace must be 256-byte aligned");
    StageWorkspace w = carve(sp, n_refs, ws);
    if (sel) w.sel = sel;
    if (count) w.count = count;
    if (accepted) w.accepted = accepted;
    uint64_t vox = static_cast<uint64_t>(volume_voxels(sp));
    const bool det = w.agg_base != nullptr && !sigma_out;
    double* sig_num = nullptr;
    if (sigma_out) {
        char* extra = static_cast<char*>(ws) + need.bytes;
        w.num = reinterpret_cast<double*>(extra);
        w.den = reinterpret_cast<double*>(extra + align256(8 * vox));
        sig_num = reinterpret_cast<double*>(extra + 2 * align256(8 * vox));
        BMND_CUDA_TRY(cudaMemsetAsync(sig_num, 0, 8 * vox, stream));
    }
    if (!det) {
        BMND_CUDA_TRY(cudaMemsetAsync(w.num, 0, 8 * vox, stream));
        BMND_CUDA_TRY(cudaMemsetAsync(w.den, 0, 8 * vox, stream));
    }
    BmndMatchParams mp = match_params_of(sp);
    const bool on_pilot = sp.filter == BMND_FILTER_WIENER && sp.wiener_match_source == BMND_SOURCE_PILOT;
    const float* match_src = on_pilot ? pilot : noisy;
    // the real-valued pilot: the bounded screening of the Poisson deviance
    // (SSD matching keeps its tensor-core screening, which any values suit)
    if (on_pilot && sp.match_precision == BMND_MATCH_EXACT && sp.distance != BMND_DIST_SSD)
        mp.precision = BMND_MATCH_REAL_VALUED;
    const float* thr_dev = nullptr;
    if (sp.distance == BMND_DIST_SSD) {
        rc = launch_ssd_threshold(match_src, static_cast<int64_t>(vox), sp.ssd_threshold, w.mm, w.thr, stream);
        if (rc) return rc;
        thr_dev = w.thr;
    }
    // Poisson HT match policies (blockmatching.py:29-148, :372-428)
    const float* thr_per_ref = nullptr;
    const double* null_moments = nullptr;
    if (sp.filter == BMND_FILTER_HARD_THRESHOLD && sp.match_policy == BMND_POLICY_REFERENCE_FINITE_COUNT) {
        int32_t counts[BMND_MAX_DIMS];
        for (int d = 0; d < sp.ndim; ++d) counts[d] = sp.shape[d] - sp.block[d] + 1;
        rc = launch_reference_thresholds(match_src, refs, n_refs, sp.ndim, counts, sp.block, sp.shape,
                                         sp.count_scale, sp.null_moments, sp.null_max_count, sp.ssd_threshold,
                                         sp.policy_beta, sp.policy_power, w.thr_ref, stream);
        if (rc) return rc;
        thr_per_ref = w.thr_ref;
    } else if (sp.filter == BMND_FILTER_HARD_THRESHOLD && sp.match_policy == BMND_POLICY_CANDIDATE_STANDARDIZED) {
        null_moments = sp.null_moments;
        mp.precision = BMND_MATCH_EXACT;
    }
    rc = launch_blockmatch_volume(mp, match_src, sp.shape, sp.block, refs, n_refs, thr_per_ref,
                                  sp.match_threshold, w.sel, w.count, w.accepted, stream, thr_dev,
                                  sp.match_noise_ssd, sp.ssd_gamma, allow_alloc, null_moments,
                                  sp.null_max_count, sp.ssd_poisson_bias != 0, w.aux, w.aux_floats, w.ssd,
                                  w.ssd_bytes);
    if (rc) return rc;
    if (det) {
        rc = launch_entry_index(sp, w.sel, w.count, n_refs, w.agg_base, w.agg, stream);
        if (rc) return rc;
        const AggStore store{reinterpret_cast<float*>(w.agg_base + w.agg.o_store),
                             reinterpret_cast<float*>(w.agg_base + w.agg.o_wstore),
                             reinterpret_cast<const int32_t*>(w.agg_base + w.agg.o_slot),
                             static_cast<int>(agg_row_floats(sp))};
        rc = launch_group_filter(sp, noisy, pilot, w.sel, w.count, n_refs, nullptr, nullptr, w.st, nullptr, stream,
                                 nullptr, nullptr, nullptr, &store);
        if (rc) return rc;
        return launch_gather(sp, noisy, out, w.agg_base, w.agg, stream);
    }
    rc = launch_group_filter(sp, noisy, pilot, w.sel, w.count, n_refs, w.num, w.den, w.st, sig_num, stream);
    if (rc) return rc;
    if (sp.mass_conserve) {
        // group-mass conservation: re-aggregate the numerator against the
        // first pass's denominator (poisson.py:231-265)
        BMND_CUDA_TRY(cudaMemsetAsync(w.num, 0, 8 * vox, stream));
        rc = launch_group_filter(sp, noisy, pilot, w.sel, w.count, n_refs, w.num, w.den, w.st, nullptr, stream,
                                 w.den);
        if (rc) return rc;
    }
    if (sigma_out) {
        rc = launch_finalize_sigma(sp, sig_num, w.den, global_sigma, sigma_out, stream);
        if (rc) return rc;
    }
    return launch_finalize(sp, w.num, w.den, noisy, out, stream);
}

// Fixed scratch array behind bmnd_stage_noalloc.  Host code must not use the
// symbol itself as a device pointer: its device address is looked up with
// cudaGetSymbolAddress once per CUDA context (a device's primary context, or a
// new one after cudaDeviceReset, which reloads the module at a new address) and
// cached.
static __device__ __align__(256) unsigned char g_static_scratch[BMND_STATIC_SCRATCH_BYTES];

std::mutex g_static_scratch_mutex;
std::map<CUcontext, void*> g_static_scratch_ptr;

// the calling thread's current context, through the driver entry point the
// runtime hands out (no link-time dependency on the driver library)
int32_t current_context(CUcontext* ctx) {
    using CtxGetCurrent = CUresult (*)(CUcontext*);
    static CtxGetCurrent get = nullptr;
    if (!get) {
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        void* fn = nullptr;
        BMND_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !fn) return fail(BMND_ERR_CUDA, "cuCtxGetCurrent not available");
        get = reinterpret_cast<CtxGetCurrent>(fn);
    }
    if (get(ctx) != CUDA_SUCCESS) return fail(BMND_ERR_CUDA, "cuCtxGetCurrent failed");
    return BMND_OK;
}

int32_t static_scratch_address(void** out) {
    int dev = 0;
    BMND_CUDA_TRY(cudaGetDevice(&dev));
    CUcontext ctx = nullptr;
    if (int32_t rc = current_context(&ctx)) return rc;
    std::lock_guard<std::mutex> guard(g_static_scratch_mutex);
    auto it = ctx ? g_static_scratch_ptr.find(ctx) : g_static_scratch_ptr.end();
    if (it == g_static_scratch_ptr.end()) {
        // the first call in this context: the lookup also makes the context current
        void* p = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_static_scratch);
        if (err != cudaSuccess) return cuda_fail(err, "cudaGetSymbolAddress(static scratch)");
        if (!p) return fail(BMND_ERR_CUDA, "static scratch has no device address");
        if (!ctx && (current_context(&ctx) != BMND_OK || !ctx))
            return fail(BMND_ERR_CUDA, "no current CUDA context after the scratch lookup");
        it = g_static_scratch_ptr.emplace(ctx, p).first;
    }
    *out = it->second;
    return BMND_OK;
}

}  // namespace
}  // namespace bmnd

using namespace bmnd;

extern "C" {

int32_t bmnd_abi_version(void) { return BMND_ABI_VERSION; }

const char* bmnd_last_error(void) { return g_last_error.c_str(); }

int32_t bmnd_launch_count(uint64_t* count) {
    clear_error();
    if (!count) return fail(BMND_ERR_INVALID_ARG, "null argument");
    *count = g_launches.load(std::memory_order_relaxed);
    return BMND_OK;
}

int32_t bmnd_device_alloc_count(uint64_t* count) {
    clear_error();
    if (!count) return fail(BMND_ERR_INVALID_ARG, "null argument");
    *count = g_device_allocs.load(std::memory_order_relaxed);
    return BMND_OK;
}

int32_t bmnd_host_memory_direct(int32_t device, int32_t* direct) {
    clear_error();
    if (!direct) return fail(BMND_ERR_INVALID_ARG, "null argument");
    int v = 0;
    BMND_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device));
    *direct = v ? 1 : 0;
    return BMND_OK;
}

int32_t bmnd_reference_schedule(int32_t ndim, const int32_t* counts, const int32_t* block,
                                const int32_t* step, double shift_density,
                                int32_t schedule_density, int32_t* out_abs, int32_t* out_shifted,
                                int32_t* out_shift, int64_t capacity, int64_t* out_count) {
    clear_error();
    if (ndim < 1 || ndim > BMND_MAX_DIMS) return fail(BMND_ERR_INVALID_ARG, "ndim must be 1..3");
    if (!counts || !block || !step || !out_count) return fail(BMND_ERR_INVALID_ARG, "null argument");
    std::vector<std::vector<int>> shifts(ndim);
    int last[BMND_MAX_DIMS], slots[BMND_MAX_DIMS];
    int64_t total_slots = 1, grid = 1;
    for (int d = 0; d < ndim; ++d) {
        if (step[d] < 1) return fail(BMND_ERR_INVALID_ARG, "step must be positive");
        if (counts[d] < 1) return fail(BMND_ERR_INVALID_ARG, "counts must be positive");
        shifts[d] = axis_shifts(block[d], step[d], d < std::max(ndim - 1, 0), shift_density);
        last[d] = std::max(counts[d] - 1, 0);
        slots[d] = (last[d] + step[d] - 1) / step[d] + 1;
        total_slots *= slots[d];
        grid *= counts[d];
    }
    int phases = std::max(1, static_cast<int>(schedule_density));
    std::vector<uint8_t> seen(static_cast<size_t>(grid), 0);
    int64_t n = 0;
    int slot[BMND_MAX_DIMS];
    for (int64_t s = 0; s < total_slots; ++s) {
        int64_t rem = s;
        for (int d = ndim - 1; d >= 0; --d) {
            slot[d] = static_cast<int>(rem % slots[d]);
            rem /= slots[d];
        }
        for (int ph = 0; ph < phases; ++ph) {
            int abs_pos[BMND_MAX_DIMS], base[BMND_MAX_DIMS];
            int64_t lin = 0;
            for (int d = 0; d < ndim; ++d) {
                int b = std::min(slot[d] * step[d], last[d]);
                int offset = 0;
                if (d < ndim - 1) {
                    const std::vector<int>& sh = shifts[d];
                    offset = sh[(slot[d + 1] + ph) % static_cast<int>(sh.size())];
                }
                int a = std::min(std::max(b - offset, 0), last[d]);
                if (slot[d] == slots[d] - 1) a = last[d];
                base[d] = b;
                abs_pos[d] = a;
                lin = lin * counts[d] + a;
            }
            if (seen[lin]) continue;
            seen[lin] = 1;
            if (n < capacity) {
                for (int d = 0; d < ndim; ++d) {
                    if (out_abs) out_abs[n * ndim + d] = abs_pos[d];
                    if (out_shifted) out_shifted[n * ndim + d] = base[d];
                    if (out_shift) out_shift[n * ndim + d] = base[d] - abs_pos[d];
                }
            }
            ++n;
        }
    }
    *out_count = n;
    return BMND_OK;
}

int32_t bmnd_blockmatch_patches(const BmndMatchParams* params, const float* d_patches,
                                int32_t patch_vol, const int32_t* d_refs, int64_t n_refs,
                                const float* d_thresholds, int32_t* d_sel, int32_t* d_count,
                                int32_t* d_accepted, uint64_t stream) {
    clear_error();
    if (!params || !d_patches || !d_thresholds || !d_sel || !d_count || !d_accepted ||
        (n_refs > 0 && !d_refs))
        return fail(BMND_ERR_INVALID_ARG, "null argument");
    return launch_blockmatch_patches(*params, d_patches, patch_vol, d_refs, n_refs, d_thresholds,
                                     d_sel, d_count, d_accepted, reinterpret_cast<cudaStream_t>(stream));
}

int32_t bmnd_blockmatch_volume_biased(const BmndMatchParams* params, const float* d_volume,
                                      const int32_t* shape, const int32_t* block, const int32_t* d_refs,
                                      int64_t n_refs, const float* d_thresholds, const float* d_noise_ssd,
                                      float gamma, int32_t* d_sel, int32_t* d_count, int32_t* d_accepted,
                                      uint64_t stream) {
    clear_error();
    if (!params || !d_volume || !shape || !block || !d_thresholds || !d_noise_ssd || !d_sel || !d_count ||
        !d_accepted || (n_refs > 0 && !d_refs))
        return fail(BMND_ERR_INVALID_ARG, "null argument");
    return launch_blockmatch_volume(*params, d_volume, shape, block, d_refs, n_refs, d_thresholds, 0.0f, d_sel,
                                    d_count, d_accepted, reinterpret_cast<cudaStream_t>(stream), nullptr,
                                    d_noise_ssd, gamma);
}

int32_t bmnd_blockmatch_volume_poisson_biased(const BmndMatchParams* params, const float* d_volume,
                                              const int32_t* shape, const int32_t* block, const int32_t* d_refs,
                                              int64_t n_refs, const float* d_thresholds, float gamma,
                                              int32_t* d_sel, int32_t* d_count, int32_t* d_accepted,
                                              uint64_t stream) {
    clear_error();
    if (!params || !d_volume || !shape || !block || !d_thresholds || !d_sel || !d_count || !d_accepted ||
        (n_refs > 0 && !d_refs))
        return fail(BMND_ERR_INVALID_ARG, "null argument");
    return launch_blockmatch_volume(*params, d_volume, shape, block, d_refs, n_refs, d_thresholds, 0.0f, d_sel,
                                    d_count, d_accepted, reinterpret_cast<cudaStream_t>(stream), nullptr, nullptr,
                                    gamma, true, nullptr, 0, true);
}

int32_t bmnd_blockmatch_volume(const BmndMatchParams* params, const float* d_volume,
                               const int32_t* shape, const int32_t* block, const int32_t* d_refs,
                               int64_t n_refs, const float* d_thresholds, int32_t* d_sel,
                               int32_t* d_count, int32_t* d_accepted, uint64_t stream) {
    clear_error();
    if (!params || !d_volume || !shape || !block || !d_thresholds || !d_sel || !d_count ||
        !d_accepted || (n_refs > 0 && !d_refs))
        return fail(BMND_ERR_INVALID_ARG, "null argument");
    return launch_blockmatch_volume(*params, d_volume, shape, block, d_refs, n_refs, d_thresholds,
                                    0.0f, d_sel, d_count, d_accepted,
                                    reinterpret_cast<cudaStream_t>(stream));
}

int32_t bmnd_stage_workspace_bytes(const BmndStageParams* params, int64_t n_refs,
                                   uint64_t* out_bytes) {
    clear_error();
    if (!params || !out_bytes || n_refs < 0) return fail(BMND_ERR_INVALID_ARG, "bad argument");
    int32_t rc = validate_stage(*params);
    if (rc) return rc;
    *out_bytes = carve(*params, n_refs, nullptr).bytes;
    return BMND_OK;
}

int32_t bmnd_stage(const BmndStageParams* params, const float* d_noisy, const float* d_pilot,
                   const int32_t* d_refs, int64_t n_refs, float* d_out, int32_t* d_sel,
                   int32_t* d_count, int32_t* d_accepted, void* d_workspace,
                   uint64_t workspace_bytes, uint64_t stream) {
    clear_error();
    if (!params) return fail(BMND_ERR_INVALID_ARG, "null params");
    return run_stage(*params, d_noisy, d_pilot, d_refs, n_refs, d_out, d_sel, d_count, d_accepted,
                     d_workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

int32_t bmnd_stage_sigma_workspace_bytes(const BmndStageParams* params, int64_t n_refs, uint64_t* out_bytes) {
    clear_error();
    if (!params || !out_bytes) return fail(BMND_ERR_INVALID_ARG, "null argument");
    if (int32_t rc = validate_stage(*params)) return rc;
    if (n_refs < 0) return fail(BMND_ERR_INVALID_ARG, "n_refs must be >= 0");
    *out_bytes = sigma_workspace_bytes(*params, n_refs);
    return BMND_OK;
}

int32_t bmnd_stage_sigma(const BmndStageParams* params, const float* d_noisy, const float* d_pilot,
                         const int32_t* d_refs, int64_t n_refs, float* d_out, float* d_sigma_map,
                         float global_sigma, int32_t* d_sel, int32_t* d_count, int32_t* d_accepted,
                         void* d_workspace, uint64_t workspace_bytes, uint64_t stream) {
    clear_error();
    if (!params) return fail(BMND_ERR_INVALID_ARG, "null params");
    if (!d_sigma_map) return fail(BMND_ERR_INVALID_ARG, "d_sigma_map is required");
    return run_stage(*params, d_noisy, d_pilot, d_refs, n_refs, d_out, d_sel, d_count, d_accepted, d_workspace,
                     workspace_bytes, reinterpret_cast<cudaStream_t>(stream), d_sigma_map, global_sigma);
}

int32_t bmnd_run(const BmndStageParams* ht, const BmndStageParams* wiener, const float* d_noisy,
                 const int32_t* d_refs_ht, int64_t n_refs_ht, const int32_t* d_refs_wiener,
                 int64_t n_refs_wiener, float* d_ht_out, float* d_out, void* d_workspace,
                 uint64_t workspace_bytes, uint64_t stream) {
    clear_error();
    if (!ht || !wiener || !d_ht_out) return fail(BMND_ERR_INVALID_ARG, "null argument");
    if (ht->filter != BMND_FILTER_HARD_THRESHOLD || wiener->filter != BMND_FILTER_WIENER)
        return fail(BMND_ERR_INVALID_ARG, "bmnd_run takes a hard-threshold then a Wiener stage");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int32_t rc = run_stage(*ht, d_noisy, nullptr, d_refs_ht, n_refs_ht, d_ht_out, nullptr, nullptr,
                           nullptr, d_workspace, workspace_bytes, s);
    if (rc) return rc;
    return run_stage(*wiener, d_noisy, d_ht_out, d_refs_wiener, n_refs_wiener, d_out, nullptr,
                     nullptr, nullptr, d_workspace, workspace_bytes, s);
}

// The probe's groups need not come from matching, so its layout covers a
// union box as large as the volume when that fits in shared memory (the
// kernel skips and reports any group wider than its layout).
BmndStageParams probe_layout_params(const BmndStageParams& sp) {
    BmndStageParams q = sp;
    for (int d = 0; d < sp.ndim; ++d) q.search_radius[d] = std::max(sp.search_radius[d], sp.shape[d]);
    return group_filter_smem_bytes(q) <= 227 * 1024 ? q : sp;
}

int32_t bmnd_group_probe_workspace_bytes(const BmndStageParams* params, uint64_t* out_bytes) {
    clear_error();
    if (!params || !out_bytes) return fail(BMND_ERR_INVALID_ARG, "null argument");
    if (int32_t rc = validate_stage(*params)) return rc;
    const uint64_t P = static_cast<uint64_t>(patch_volume(*params));
    // the Kronecker table, the risk metric and the group matrices, then the status word
    *out_bytes = align256(4ull * stage_table_floats(static_cast<int>(P))) + 256;
    return BMND_OK;
}

int32_t bmnd_group_probe(const BmndStageParams* params, const float* d_noisy, const float* d_pilot,
                         const int32_t* d_sel, const int32_t* d_count, int64_t n_groups, float* d_coef,
                         float* d_sigma, float* d_atten, float* d_weights, float* d_filt, void* d_workspace,
                         uint64_t workspace_bytes, uint64_t stream) {
    clear_error();
    if (!params) return fail(BMND_ERR_INVALID_ARG, "null params");
    const BmndStageParams& sp = *params;
    if (int32_t rc = validate_stage(sp)) return rc;
    if (sp.mass_conserve) return fail(BMND_ERR_INVALID_ARG, "the group probe has no mass-conservation pass");
    if (!d_noisy) return fail(BMND_ERR_INVALID_ARG, "d_noisy is required");
    if (sp.filter == BMND_FILTER_WIENER && !d_pilot)
        return fail(BMND_ERR_INVALID_ARG, "the Wiener filter needs the pilot");
    if (n_groups < 0 || (n_groups > 0 && (!d_sel || !d_count)))
        return fail(BMND_ERR_INVALID_ARG, "bad group list");
    uint64_t need = 0;
    if (int32_t rc = bmnd_group_probe_workspace_bytes(params, &need)) return rc;
    if (!d_workspace || workspace_bytes < need) return fail(BMND_ERR_WORKSPACE, "workspace too small");
    if (reinterpret_cast<uintptr_t>(d_workspace) % 256 != 0)
        return fail(BMND_ERR_INVALID_ARG, "workspace must be 256-byte aligned");
    GroupProbe probe{1, d_coef, d_sigma, d_atten, d_weights, d_filt};
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int* status = reinterpret_cast<int*>(static_cast<char*>(d_workspace) + need - 256);
    BMND_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
    const BmndStageParams q = probe_layout_params(sp);
    int32_t rc = launch_group_filter(q, d_noisy, d_pilot, d_sel, d_count, n_groups, nullptr, nullptr,
                                     static_cast<float*>(d_workspace), nullptr, s, nullptr, status, &probe);
    if (rc) return rc;
    int h_status = 0;
    BMND_CUDA_TRY(cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, s));
    BMND_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_status)
        return fail(BMND_ERR_INVALID_ARG, "a group has a member outside the patch grid, more members than "
                                          "max_stack, or a union box larger than the kernel's layout");
    return BMND_OK;
}

int32_t bmnd_stage_noalloc(const BmndStageParams* params, const float* d_noisy,
                           const float* d_pilot, const int32_t* d_refs, int64_t n_refs,
                           float* d_out, uint64_t stream) {
    clear_error();
    if (!params) return fail(BMND_ERR_INVALID_ARG, "null params");
    int32_t rc = validate_stage(*params);
    if (rc) return rc;
    if (n_refs < 0) return fail(BMND_ERR_INVALID_ARG, "bad reference list");
    uint64_t need = carve(*params, n_refs, nullptr).bytes;
    if (need > BMND_STATIC_SCRATCH_BYTES)
        return fail(BMND_ERR_WORKSPACE,
                    "stage needs " + std::to_string(need) + " scratch bytes; the static scratch of "
                    "bmnd_stage_noalloc holds " + std::to_string(BMND_STATIC_SCRATCH_BYTES) +
                    " (use bmnd_stage with a caller workspace)");
    void* scratch = nullptr;
    rc = static_scratch_address(&scratch);
    if (rc) return rc;
    return run_stage(*params, d_noisy, d_pilot, d_refs, n_refs, d_out, nullptr, nullptr, nullptr,
                     scratch, BMND_STATIC_SCRATCH_BYTES, reinterpret_cast<cudaStream_t>(stream), nullptr, 0.0f,
                     false);
}

}  // extern "C"

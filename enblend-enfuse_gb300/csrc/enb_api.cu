// enb_api.cu -- C ABI of the GB300 enblend/enfuse path: context, pyramid
// handles, primitive entry points and the enfuse/enblend drivers (host C++).
#include <cuda_runtime.h>

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "enb_internal.h"
#include "enbgpu.h"

using namespace enb;

// Scratch of enb_gaussian_pyramid_noalloc: the alpha planes of pyramid levels
// 1..L-1.  Host code must not use this name as an address; it looks the
// device address up with cudaGetSymbolAddress (noalloc_scratch below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[ENB_NOALLOC_SCRATCH_BYTES];

struct enb_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    uint64_t launches = 0;
    // kernel profiling (enb_profile_*)
    struct ProfKernel {
        std::string name;
        uint64_t launches = 0;
        double ms = 0.0;
        double bytes = 0.0;
    };
    struct ProfPending {
        size_t k;
        cudaEvent_t a, b;
    };
    bool prof = false;
    std::vector<ProfKernel> kernels;
    std::vector<ProfPending> pending;
    std::vector<cudaEvent_t> pool;
    // cached enfuse weight tables
    std::string table_key;
    void* table_mem = nullptr;
    WeightTables tables{};
    // host-transfer stream and events of the banded host-buffer path
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> io_events;
    // batched stacks: plan (workspace, job tables) and graph of the last
    // batch geometry, staging buffers of host-buffer batches
    struct BatchCache {
        std::string key;
        BatchPlan* plan = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaStream_t gs = nullptr;
        cudaEvent_t ev[2] = {nullptr, nullptr};
        void* stage = nullptr;
        ~BatchCache()
        {
            if (exec) {
                cudaGraphExecDestroy(exec);
            }
            batch_plan_destroy(plan);
            cudaFree(stage);
            for (cudaEvent_t e : ev) {
                if (e) {
                    cudaEventDestroy(e);
                }
            }
            if (gs) {
                cudaStreamDestroy(gs);
            }
        }
    };
    std::unique_ptr<BatchCache> batch;
    // device error word of the kernels' bounded waits (bit 0: a TMA tile
    // pipeline wait timed out); read after synchronisations
    unsigned int* dev_err = nullptr;
    // coarse thresholds chosen by enb_fuse_stacks_tune, per batch geometry
    std::map<std::string, int32_t> tuned;
    // enb_debug_overarm_tile_waits: bytes the level-0 pipeline's stage
    // barriers expect beyond their copies (0 in normal operation)
    uint32_t tx_extra = 0;
};

struct enb_pyramid {
    int levels = 0;
    int C = 0;
    int dtype = ENB_I32;
    int w[kMaxLevels + 1] = {};
    int h[kMaxLevels + 1] = {};
    int64_t pitch[kMaxLevels + 1] = {};  // elements
    int64_t offset[kMaxLevels + 1] = {}; // bytes from base
    void* base = nullptr;
    size_t bytes = 0;
};

namespace {

// The context's device error word, allocated (zeroed) on first use; null
// when it cannot be allocated (the kernels that need it are then not used).
unsigned int* device_error_word(enb_ctx* ctx)
{
    if (!ctx->dev_err) {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(unsigned int)) != cudaSuccess || cudaMemset(p, 0, sizeof(unsigned int)) != cudaSuccess) {
            cudaGetLastError();
            if (p) {
                cudaFree(p);
            }
            return nullptr;
        }
        ctx->dev_err = static_cast<unsigned int*>(p);
    }
    return ctx->dev_err;
}

// After a synchronisation of the context's stream: a kernel that gave up a
// bounded wait fails the call (and the word is cleared).
enb_status check_device_error(enb_ctx* ctx)
{
    if (!ctx->dev_err) {
        return ENB_OK;
    }
    unsigned int v = 0;
    if (cudaMemcpy(&v, ctx->dev_err, sizeof v, cudaMemcpyDeviceToHost) != cudaSuccess) {
        ctx->err = "reading the device error word failed";
        cudaGetLastError();
        return ENB_ERR_CUDA;
    }
    if (v) {
        cudaMemset(ctx->dev_err, 0, sizeof v);
        ctx->err = (v & 1u) ? "a kernel's wait for its tile copies timed out (TMA pipeline)"
                            : "a coarse item's wait for its predecessor step timed out (batched fuse)";
        return ENB_ERR_CUDA;
    }
    return ENB_OK;
}

size_t dtype_size(int dt)
{
    switch (dt) {
    case ENB_U8: return 1;
    case ENB_U16: return 2;
    case ENB_I16: return 2;
    case ENB_F32: return 4;
    case ENB_I32: return 4;
    default: return 0;
    }
}

enb_status fail(enb_ctx* ctx, enb_status st, const std::string& msg)
{
    if (ctx) {
        ctx->err = msg;
    }
    return st;
}

enb_status cuda_fail(enb_ctx* ctx, cudaError_t e, const char* where)
{
    return fail(ctx, ENB_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

cudaEvent_t prof_event(enb_ctx* ctx)
{
    if (!ctx->pool.empty()) {
        cudaEvent_t e = ctx->pool.back();
        ctx->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

cudaEvent_t prof_begin(enb_ctx* ctx)
{
    if (!ctx->prof) {
        return nullptr;
    }
    cudaEvent_t a = prof_event(ctx);
    cudaEventRecord(a, ctx->stream);
    return a;
}

void prof_end(enb_ctx* ctx, cudaEvent_t a)
{
    if (!a) {
        return;
    }
    cudaEvent_t b = prof_event(ctx);
    cudaEventRecord(b, ctx->stream);
    const LaunchInfo& li = last_launch();
    size_t k = 0;
    while (k < ctx->kernels.size() && ctx->kernels[k].name != li.name) {
        ++k;
    }
    if (k == ctx->kernels.size()) {
        ctx->kernels.push_back(enb_ctx::ProfKernel{li.name, 0, 0.0, 0.0});
    }
    ctx->kernels[k].launches++;
    ctx->kernels[k].bytes += li.bytes;
    ctx->pending.push_back(enb_ctx::ProfPending{k, a, b});
}

// Sum the elapsed times of finished launches (synchronises the stream).
void prof_resolve(enb_ctx* ctx)
{
    if (ctx->pending.empty()) {
        return;
    }
    cudaStreamSynchronize(ctx->stream);
    for (auto& p : ctx->pending) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            ctx->kernels[p.k].ms += ms;
        }
        ctx->pool.push_back(p.a);
        ctx->pool.push_back(p.b);
    }
    ctx->pending.clear();
}

#define ENB_LAUNCH(ctx, call)                                  \
    do {                                                       \
        cudaEvent_t a_ = prof_begin(ctx);                      \
        last_launch().kernels = 1;                             \
        cudaError_t e_ = (call);                               \
        prof_end((ctx), a_);                                   \
        (ctx)->launches += (uint64_t)last_launch().kernels;    \
        if (e_ != cudaSuccess) {                               \
            return cuda_fail((ctx), e_, #call);                \
        }                                                      \
    } while (0)

#define ENB_CUDA(ctx, call)                                    \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) {                               \
            return cuda_fail((ctx), e_, #call);                \
        }                                                      \
    } while (0)

#define ENB_CHECK(ctx, cond, msg)                              \
    do {                                                       \
        if (!(cond)) {                                         \
            return fail((ctx), ENB_ERR_INVALID, (msg));        \
        }                                                      \
    } while (0)

#define ENB_TRY(call)                                          \
    do {                                                       \
        enb_status s_ = (call);                                \
        if (s_ != ENB_OK) {                                    \
            return s_;                                         \
        }                                                      \
    } while (0)

// Stream-ordered device allocation freed on scope exit.
struct DevBuf {
    void* p = nullptr;
    cudaStream_t st = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf()
    {
        if (p) {
            cudaFreeAsync(p, st);
        }
    }
    cudaError_t alloc(size_t bytes, cudaStream_t s)
    {
        st = s;
        return cudaMallocAsync(&p, bytes == 0 ? 1 : bytes, s);
    }
};

int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// ---- descriptor -> view conversions ------------------------------------

bool planar_ok(const enb_image* im)
{
    return im && im->data && im->planar && (im->dtype == ENB_I16 || im->dtype == ENB_I32 || im->dtype == ENB_F32) &&
           im->width > 0 &&
           im->height > 0 && im->channels >= 1 && im->pitch % (int64_t)dtype_size(im->dtype) == 0 &&
           im->plane_pitch % (int64_t)dtype_size(im->dtype) == 0 && im->pitch >= im->width * (int64_t)dtype_size(im->dtype);
}

PlanarView planar_view(const enb_image* im)
{
    const int64_t es = (int64_t)dtype_size(im->dtype);
    return PlanarView{im->data, im->pitch / es, im->plane_pitch / es, im->width, im->height, im->channels, im->dtype};
}

bool pixels_ok(const enb_image* im)
{
    if (!im || !im->data || im->planar || (im->dtype != ENB_U8 && im->dtype != ENB_U16 && im->dtype != ENB_F32) ||
        im->width <= 0 || im->height <= 0) {
        return false;
    }
    if (im->channels != 1 && im->channels != 3) {
        return false;
    }
    const int stride = im->pix_stride > 0 ? im->pix_stride : im->channels;
    return stride >= im->channels && stride <= 4 && im->pitch % (int64_t)dtype_size(im->dtype) == 0 &&
           im->pitch >= (int64_t)im->width * stride * (int64_t)dtype_size(im->dtype);
}

PixelView pixel_view(const enb_image* im)
{
    const int64_t es = (int64_t)dtype_size(im->dtype);
    const int stride = im->pix_stride > 0 ? im->pix_stride : im->channels;
    return PixelView{im->data, im->pitch / es, im->width, im->height, im->channels, stride, im->dtype};
}

bool bytes_ok(const enb_image* im, int w, int h)
{
    return im && im->data && im->dtype == ENB_U8 && im->width == w && im->height == h && im->pitch >= w;
}

BytePlane byte_plane(const enb_image* im)
{
    return BytePlane{(uint8_t*)im->data, im->pitch, im->width, im->height};
}

bool floats_ok(const enb_image* im, int w, int h)
{
    return im && im->data && im->dtype == ENB_F32 && im->width == w && im->height == h && im->pitch % 4 == 0 &&
           im->pitch >= (int64_t)w * 4;
}

FloatPlane float_plane(const enb_image* im) { return FloatPlane{(float*)im->data, im->pitch / 4, im->width, im->height}; }

PlanarView level_view(const enb_pyramid* p, int l)
{
    return PlanarView{(char*)p->base + p->offset[l], p->pitch[l], p->pitch[l] * p->h[l], p->w[l], p->h[l], p->C,
                      p->dtype};
}

// Alpha source of an interleaved image: explicit plane, thresholded 4th
// component (src/assemble.h:240-253: Threshold(max/2, max) -> 0/255), or opaque.
AlphaSrc alpha_source(const enb_image* img, const enb_image* alpha)
{
    AlphaSrc a{};
    if (alpha && alpha->data) {
        a.mode = kAlphaPlane;
        a.plane = byte_plane(alpha);
    } else if (img->pix_stride == 4) {
        a.mode = kAlphaChannel3;
        a.pix = pixel_view(img);
        const uint32_t maxv = img->dtype == ENB_U8 ? 255u : 65535u;
        a.lo = (uint32_t)(maxv / 2.0);  // static_cast of range.second / 2.0
        a.hi = maxv;
        a.flo = 0.5f;  // float images: range (0, 1), src/common.h:594
        a.fhi = 1.0f;
    } else {
        a.mode = kAlphaOpaque;
    }
    return a;
}

// ---- pyramids -------------------------------------------------------------

enb_status pyramid_alloc(enb_ctx* ctx, int levels, int w, int h, int C, int dtype, enb_pyramid** out)
{
    ENB_CHECK(ctx, levels >= 1 && levels <= kMaxLevels, "pyramid: levels outside 1..29");
    ENB_CHECK(ctx, w > 0 && h > 0 && (C == 1 || C == 3), "pyramid: bad size or channel count");
    ENB_CHECK(ctx, dtype == ENB_I16 || dtype == ENB_I32 || dtype == ENB_F32,
              "pyramid: dtype must be ENB_I16, ENB_I32 or ENB_F32");
    std::unique_ptr<enb_pyramid> p(new enb_pyramid());
    p->levels = levels;
    p->C = C;
    p->dtype = dtype;
    const int64_t es = (int64_t)dtype_size(dtype);
    int64_t off = 0;
    int lw = w, lh = h;
    for (int l = 0; l < levels; ++l) {
        p->w[l] = lw;
        p->h[l] = lh;
        p->pitch[l] = round_up(lw, 128 / es);  // 128-byte aligned rows
        p->offset[l] = off;
        off += round_up(p->pitch[l] * lh * C * es, 256);
        lw = (lw + 1) >> 1;
        lh = (lh + 1) >> 1;
    }
    p->bytes = (size_t)off;
    cudaError_t e = cudaMallocAsync(&p->base, p->bytes, ctx->stream);
    if (e != cudaSuccess) {
        return fail(ctx, ENB_ERR_NOMEM, std::string("pyramid allocation: ") + cudaGetErrorString(e));
    }
    *out = p.release();
    return ENB_OK;
}

void pyramid_release(enb_ctx* ctx, enb_pyramid* p)
{
    if (p) {
        if (p->base) {
            cudaFreeAsync(p->base, ctx->stream);
        }
        delete p;
    }
}

struct PyrHolder {
    enb_ctx* ctx;
    enb_pyramid* p = nullptr;
    explicit PyrHolder(enb_ctx* c) : ctx(c) {}
    ~PyrHolder() { pyramid_release(ctx, p); }
};

// Alpha planes of levels 1..L-1 (level l at offset[l]); level 0 is the source alpha.
struct AlphaChain {
    DevBuf mem;
    int64_t pitch[kMaxLevels + 1] = {};
    int64_t offset[kMaxLevels + 1] = {};
    int w[kMaxLevels + 1] = {}, h[kMaxLevels + 1] = {};
    cudaError_t alloc(int levels, int w0, int h0, cudaStream_t st)
    {
        int64_t off = 0;
        int lw = w0, lh = h0;
        for (int l = 0; l < levels; ++l) {
            w[l] = lw;
            h[l] = lh;
            pitch[l] = round_up(lw, 128);
            offset[l] = off;
            off += round_up(pitch[l] * lh, 256);
            lw = (lw + 1) >> 1;
            lh = (lh + 1) >> 1;
        }
        return mem.alloc((size_t)off, st);
    }
    BytePlane level(int l) { return BytePlane{(uint8_t*)mem.p + offset[l], pitch[l], w[l], h[l]}; }
};

// Reduce chain of a pyramid whose level 0 is filled (gaussianPyramid,
// src/pyramid.h:1500-1530 with alpha, :1590-1610 without).
enb_status gaussian_levels(enb_ctx* ctx, int wrap, enb_pyramid* p, const BytePlane* alpha0)
{
    if (p->levels <= 1) {
        return ENB_OK;
    }
    if (!alpha0) {
        for (int l = 1; l < p->levels; ++l) {
            ENB_CHECK(ctx, p->w[l - 1] > 1 && p->h[l - 1] > 1, "reduce: src image too small in reduce");
            ENB_LAUNCH(ctx, launch_reduce(wrap, level_view(p, l - 1), nullptr, level_view(p, l), nullptr, ctx->stream));
        }
        return ENB_OK;
    }
    AlphaChain ac;
    ENB_CUDA(ctx, ac.alloc(p->levels, p->w[0], p->h[0], ctx->stream));
    for (int l = 1; l < p->levels; ++l) {
        ENB_CHECK(ctx, p->w[l - 1] > 1 && p->h[l - 1] > 1, "reduce: src image too small in reduce");
        const BytePlane src_a = l == 1 ? *alpha0 : ac.level(l - 1);
        const BytePlane dst_a = ac.level(l);
        ENB_LAUNCH(ctx, launch_reduce(wrap, level_view(p, l - 1), &src_a, level_view(p, l), &dst_a, ctx->stream));
    }
    return ENB_OK;
}

enb_status laplacian_levels(enb_ctx* ctx, int wrap, enb_pyramid* p)
{
    for (int l = 0; l + 1 < p->levels; ++l) {
        ENB_LAUNCH(ctx, launch_expand(0, wrap, level_view(p, l + 1), level_view(p, l), ctx->stream));
    }
    return ENB_OK;
}

enb_status collapse_levels(enb_ctx* ctx, int wrap, enb_pyramid* p)
{
    for (int l = p->levels - 2; l >= 0; --l) {
        ENB_LAUNCH(ctx, launch_expand(1, wrap, level_view(p, l + 1), level_view(p, l), ctx->stream));
    }
    return ENB_OK;
}

// ---- enfuse weight tables --------------------------------------------------

constexpr double kFwhmGaussian = 2.3548200450309493820231386529193992755;
constexpr double kFwhmLorentzian = 2.8284271247461900976033774484193961571;
constexpr double kFwhmHalfSine = 2.0943951023931954923084289221863352561;
constexpr double kFwhmFullSine = 3.14159265358979323846;
constexpr double kFwhmBisquare = 1.6817928305074290860622509524664297901;

// Built-in exposure weight functions of src/exposure_weight.h:44-128, each
// with its width rescaled to the Gaussian's FWHM.
double exposure_fn(int fn, double y, double opt, double width)
{
    double wd = width;
    switch (fn) {
    case ENB_EXP_LORENTZIAN: wd = width * kFwhmGaussian / kFwhmLorentzian; break;
    case ENB_EXP_HALF_SINE: wd = width * kFwhmGaussian / kFwhmHalfSine; break;
    case ENB_EXP_FULL_SINE: wd = width * kFwhmGaussian / kFwhmFullSine; break;
    case ENB_EXP_BISQUARE: wd = width * kFwhmGaussian / kFwhmBisquare; break;
    default: break;
    }
    const double z = (y - opt) / wd;
    switch (fn) {
    case ENB_EXP_LORENTZIAN: return 1.0 / (1.0 + 0.5 * z * z);
    case ENB_EXP_HALF_SINE: return fabs(z) <= 1.57079632679489661923 ? cos(z) : 0.0;
    case ENB_EXP_FULL_SINE: return fabs(z) <= 3.14159265358979323846 ? 0.5 + cos(z) / 2.0 : 0.0;
    case ENB_EXP_BISQUARE: {
        if (fabs(z) <= 1.0) {
            const double z2 = z * z;
            return (1.0 - z2) * (1.0 + z2);
        }
        return 0.0;
    }
    default: return exp(-0.5 * z * z);
    }
}

enb_status build_tables(enb_ctx* ctx, const enb_enfuse_params* prm, uint32_t maxv)
{
    const bool user_table = prm->exposure_table != nullptr && prm->w_exposure > 0.0;
    if (user_table) {
        if (maxv == 1u) {
            return fail(ctx, ENB_ERR_UNSUPPORTED,
                        "exposure_table: user exposure weight tables apply to 8- and 16-bit images only");
        }
        ENB_CHECK(ctx, prm->exposure_table_size == (int32_t)maxv + 1,
                  "exposure_table: one entry per sample value (256 for 8-bit, 65536 for 16-bit images)");
    }
    // a user table enters the cache key through a hash of its contents
    uint64_t th = 0;
    if (user_table) {
        th = 1469598103934665603ull;
        const unsigned char* tb = reinterpret_cast<const unsigned char*>(prm->exposure_table);
        for (size_t i = 0; i < (size_t)prm->exposure_table_size * sizeof(double); ++i) {
            th = (th ^ tb[i]) * 1099511628211ull;
        }
    }
    char key[512];
    snprintf(key, sizeof key, "%u|%.17g|%.17g|%.17g|%.17g|%.17g|%.17g|%d|%d|%d|%llx", maxv, prm->w_exposure,
             prm->w_contrast, prm->w_entropy, prm->w_saturation, prm->exp_optimum, prm->exp_width, prm->exp_function,
             prm->entropy_window, user_table ? 1 : 0, (unsigned long long)th);
    if (ctx->table_mem && ctx->table_key == key) {
        return ENB_OK;
    }
    const int n = (int)maxv + 1;
    const int nmax = prm->entropy_window * prm->entropy_window;
    const int nt = (nmax + 1) * (nmax + 1);
    std::vector<float> exposure(n), contrast(n), entropy(n);
    for (int g = 0; g < n; ++g) {
        const double y = (double)g / (double)maxv;
        // fromRealPromote(weight_ * weight_function_->weight(y)) (src/enfuse.h:638-639)
        const double f = user_table ? prm->exposure_table[g]
                                    : exposure_fn(prm->exp_function, y, prm->exp_optimum, prm->exp_width);
        exposure[g] = (float)(prm->w_exposure * f);
        contrast[g] = (float)(prm->w_contrast * (double)g / (double)maxv);
        entropy[g] = (float)(prm->w_entropy * (double)(float)g);
    }
    std::vector<double> plogp(nt, 0.0), logb(nmax + 1, 0.0);
    std::vector<long long> plogp_fx(nt, 0);
    std::vector<float> scale_logb(nmax + 1, 0.0f);
    std::vector<unsigned long long> scale_fx(nmax + 1, 0ull);
    for (int tot = 1; tot <= nmax; ++tot) {
        for (int c = 1; c <= tot; ++c) {
            const double p = (double)c / (double)tot;
            const double v = p * log(p);
            plogp[(size_t)tot * (nmax + 1) + c] = v;
            plogp_fx[(size_t)tot * (nmax + 1) + c] = llround(v * 72057594037927936.0);  // 2^56
        }
    }
    for (int b = 1; b <= nmax; ++b) {
        logb[b] = log((double)b);
        scale_logb[b] = b >= 2 ? (float)((double)maxv / logb[b]) : 0.0f;
        scale_fx[b] = b >= 2 ? (unsigned long long)llround(ldexp((double)maxv / logb[b], 40)) : 0ull;
    }
    // float images with entropy windows of 3 or 5: the clip-bin entropy table
    const bool clip_table = maxv == 1u && nmax <= 25;
    const size_t sz_f = (size_t)n * 4, sz_pl = (size_t)nt * 8, sz_lb = (size_t)(nmax + 1) * 8,
                 sz_sl = (size_t)(nmax + 1) * 4, sz_sf = (size_t)(nmax + 1) * 8,
                 sz_ch = clip_table ? (size_t)(nmax + 1) * (nmax + 1) * (nmax + 1) * 4 : 0;
    const size_t o_exp = 0, o_con = round_up((int64_t)(o_exp + sz_f), 256), o_ent = round_up((int64_t)(o_con + sz_f), 256),
                 o_pl = round_up((int64_t)(o_ent + sz_f), 256), o_fx = round_up((int64_t)(o_pl + sz_pl), 256),
                 o_lb = round_up((int64_t)(o_fx + sz_pl), 256), o_sl = round_up((int64_t)(o_lb + sz_lb), 256),
                 o_sf = round_up((int64_t)(o_sl + sz_sl), 256), o_ch = round_up((int64_t)(o_sf + sz_sf), 256),
                 total = round_up((int64_t)(o_ch + sz_ch), 256);
    if (ctx->table_mem) {
        cudaFreeAsync(ctx->table_mem, ctx->stream);
        ctx->table_mem = nullptr;
    }
    ENB_CUDA(ctx, cudaMallocAsync(&ctx->table_mem, total, ctx->stream));
    char* b = (char*)ctx->table_mem;
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_exp, exposure.data(), sz_f, cudaMemcpyHostToDevice, ctx->stream));
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_con, contrast.data(), sz_f, cudaMemcpyHostToDevice, ctx->stream));
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_ent, entropy.data(), sz_f, cudaMemcpyHostToDevice, ctx->stream));
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_pl, plogp.data(), sz_pl, cudaMemcpyHostToDevice, ctx->stream));
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_fx, plogp_fx.data(), sz_pl, cudaMemcpyHostToDevice, ctx->stream));
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_lb, logb.data(), sz_lb, cudaMemcpyHostToDevice, ctx->stream));
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_sl, scale_logb.data(), sz_sl, cudaMemcpyHostToDevice, ctx->stream));
    ENB_CUDA(ctx, cudaMemcpyAsync(b + o_sf, scale_fx.data(), sz_sf, cudaMemcpyHostToDevice, ctx->stream));
    WeightTables tab{(const float*)(b + o_exp), (const float*)(b + o_con), (const float*)(b + o_ent),
                     (const double*)(b + o_pl), (const long long*)(b + o_fx), (const double*)(b + o_lb),
                     (const float*)(b + o_sl), (const unsigned long long*)(b + o_sf), nullptr};
    if (clip_table) {
        ENB_CUDA(ctx, launch_clip_entropy_table(tab, nmax, (float*)(b + o_ch), ctx->stream));
        tab.clip_h = (const float*)(b + o_ch);
    }
    // pageable sources: make sure the copies consumed them before the vectors go
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->tables = tab;
    ctx->table_key = key;
    return ENB_OK;
}

enb_status check_params(enb_ctx* ctx, const enb_enfuse_params* p, int w, int h)
{
    ENB_CHECK(ctx, p, "enfuse params: NULL");
    ENB_CHECK(ctx, p->exp_optimum >= 0.0 && p->exp_optimum <= 1.0, "exposure optimum outside [0, 1]");
    ENB_CHECK(ctx, p->exp_width > 0.0, "exposure width must be positive");
    ENB_CHECK(ctx, p->exp_function >= ENB_EXP_GAUSSIAN && p->exp_function <= ENB_EXP_BISQUARE,
              "unknown exposure weight function");
    ENB_CHECK(ctx, p->gray_projector >= ENB_GRAY_AVERAGE && p->gray_projector <= ENB_GRAY_MIXER,
              "unknown grayscale projector");
    ENB_CHECK(ctx,
              p->exp_cutoff_lower_projector >= ENB_GRAY_AVERAGE && p->exp_cutoff_lower_projector <= ENB_GRAY_MIXER &&
                  p->exp_cutoff_upper_projector >= ENB_GRAY_AVERAGE && p->exp_cutoff_upper_projector <= ENB_GRAY_MIXER,
              "unknown grayscale projector of the exposure cutoff");
    if (p->w_contrast > 0.0) {
        ENB_CHECK(ctx, p->contrast_window >= 3 && (p->contrast_window & 1) && p->contrast_window <= kMaxContrastWindow,
                  "contrast window must be odd, 3..31");
        ENB_CHECK(ctx, w >= p->contrast_window && h >= p->contrast_window, "localStdDevIf(): window larger than image");
    }
    if (p->w_entropy > 0.0) {
        ENB_CHECK(ctx, p->entropy_window >= 3 && (p->entropy_window & 1) && p->entropy_window <= kMaxEntropyWindow,
                  "entropy window must be odd, 3..15");
        ENB_CHECK(ctx, w >= p->entropy_window && h >= p->entropy_window, "localEntropyIf(): window larger than image");
    }
    if (p->gray_projector == ENB_GRAY_MIXER) {
        ENB_CHECK(ctx, p->mixer[0] >= 0 && p->mixer[1] >= 0 && p->mixer[2] >= 0 &&
                           p->mixer[0] + p->mixer[1] + p->mixer[2] != 0.0,
                  "channel-mixer weights must be non-negative with a non-zero sum");
    }
    return ENB_OK;
}

// Effective width of the built-in exposure weight functions: the user width
// rescaled to the Gaussian's FWHM (src/exposure_weight.h:56-116).
double exposure_effective_width(int fn, double width)
{
    switch (fn) {
    case ENB_EXP_LORENTZIAN: return width * kFwhmGaussian / kFwhmLorentzian;
    case ENB_EXP_HALF_SINE: return width * kFwhmGaussian / kFwhmHalfSine;
    case ENB_EXP_FULL_SINE: return width * kFwhmGaussian / kFwhmFullSine;
    case ENB_EXP_BISQUARE: return width * kFwhmGaussian / kFwhmBisquare;
    default: return width;
    }
}

// Scale of float samples: enb_enfuse_params.float_range, 0 = the reference's
// NumericTraits<float>::max().
double float_range_of(const enb_enfuse_params* prm)
{
    return prm->float_range > 0.0 ? prm->float_range : 3.4028234663852886e38;
}

// AlternativePercentage::is_effective / CompactifiedAlternativePercentage::
// is_effective (src/alternativepercentage.h:44-52, 76-83) for samples whose
// maximum is maxv.
bool cutoff_effective(double v, int pct, double maxv, bool compact)
{
    if (compact) {
        return v != 0.0 && ((pct && fabs(v) != 100.0) || (!pct && v != maxv));
    }
    return v > 0.0 && ((pct && v < 100.0) || (!pct && v < maxv));
}

// instantiate<t> (src/alternativepercentage.h:54-60, 85-95): the limit in
// sample units, truncated toward zero for integer samples, rounded to float
// for float samples; the compactified form counts a negative value down
// from the maximum.
double cutoff_value(double v, int pct, double maxv, bool integral, bool compact)
{
    double c;
    if (compact) {
        c = pct ? (v >= 0.0 ? v : 100.0 + v) * maxv / 100.0 : (v >= 0.0 ? v : maxv + v);
    } else {
        c = pct ? v * maxv / 100.0 : v;
    }
    return integral ? trunc(c) : (double)(float)c;
}

// The limits of an exposure or entropy cutoff: the lower limit a plain, the
// upper one a compactified percentage, as both options are documented.  The
// reference's exposure functor instantiates its upper limit through the
// plain base class (src/enfuse.h:659-661), which agrees for every
// non-negative limit; negative limits and a lower limit above the upper one
// are errors there (exit(1), src/enfuse.h:667-685, 1154-1172) and here.
enb_status cutoff_limits(enb_ctx* ctx, const char* what, double lower, int lower_pct, double upper, int upper_pct,
                         double maxv, bool integral, bool& active, double& lo, double& hi)
{
    active = cutoff_effective(lower, lower_pct, maxv, false) || cutoff_effective(upper, upper_pct, maxv, true);
    if (!active) {
        return ENB_OK;
    }
    lo = cutoff_value(lower, lower_pct, maxv, integral, false);
    hi = cutoff_value(upper, upper_pct, maxv, integral, true);
    ENB_CHECK(ctx, lo >= 0.0, std::string("negative lower ") + what + " cutoff");
    ENB_CHECK(ctx, hi >= 0.0, std::string("negative upper ") + what + " cutoff");
    ENB_CHECK(ctx, lo <= hi, std::string("lower ") + what + " cutoff exceeds upper cutoff");
    return ENB_OK;
}

// The cutoffs of integer samples with maximum maxv in WeightParams: limits
// outside [0, maxv] act as the nearest value outside that range.
enb_status int_cutoffs(enb_ctx* ctx, const enb_enfuse_params* prm, uint32_t maxv, WeightParams& wp)
{
    const auto clampi = [&](double v) { return (int32_t)std::min(std::max(v, -1.0), (double)maxv + 1.0); };
    bool on = false;
    double lo = 0.0, hi = 0.0;
    if (prm->w_exposure > 0.0) {
        ENB_TRY(cutoff_limits(ctx, "exposure", prm->exp_cutoff_lower, prm->exp_cutoff_lower_pct, prm->exp_cutoff_upper,
                              prm->exp_cutoff_upper_pct, (double)maxv, true, on, lo, hi));
        wp.exp_cut = on;
        wp.cut_proj[0] = prm->exp_cutoff_lower_projector;
        wp.cut_proj[1] = prm->exp_cutoff_upper_projector;
        wp.cut_lo = clampi(lo);
        wp.cut_hi = clampi(hi);
    }
    if (prm->w_entropy > 0.0) {
        ENB_TRY(cutoff_limits(ctx, "entropy", prm->ent_cutoff_lower, prm->ent_cutoff_lower_pct, prm->ent_cutoff_upper,
                              prm->ent_cutoff_upper_pct, (double)maxv, true, on, lo, hi));
        wp.ent_cut = on;
        wp.ent_lo = clampi(lo);
        wp.ent_hi = clampi(hi);
    }
    return ENB_OK;
}

// The cutoffs of float samples (limits relative to float_range's scale).
enb_status float_cutoffs(enb_ctx* ctx, const enb_enfuse_params* prm, double range, FloatWeightParams& wp)
{
    bool on = false;
    double lo = 0.0, hi = 0.0;
    if (prm->w_exposure > 0.0) {
        ENB_TRY(cutoff_limits(ctx, "exposure", prm->exp_cutoff_lower, prm->exp_cutoff_lower_pct, prm->exp_cutoff_upper,
                              prm->exp_cutoff_upper_pct, range, false, on, lo, hi));
        wp.exp_cut = on;
        wp.cut_proj[0] = prm->exp_cutoff_lower_projector;
        wp.cut_proj[1] = prm->exp_cutoff_upper_projector;
        wp.cut_lo = (float)lo;
        wp.cut_hi = (float)hi;
    }
    if (prm->w_entropy > 0.0) {
        ENB_TRY(cutoff_limits(ctx, "entropy", prm->ent_cutoff_lower, prm->ent_cutoff_lower_pct, prm->ent_cutoff_upper,
                              prm->ent_cutoff_upper_pct, range, false, on, lo, hi));
        wp.ent_cut = on;
        wp.ent_lo = (float)lo;
        wp.ent_hi = (float)hi;
    }
    return ENB_OK;
}

enb_status alpha_plane(enb_ctx* ctx, const enb_image* img, const enb_image* alpha, DevBuf& buf, BytePlane& out);

enb_status enfuse_mask_float(enb_ctx* ctx, const enb_enfuse_params* prm, const enb_image* src,
                             const enb_image* alpha, const FloatPlane& out)
{
    ENB_TRY(build_tables(ctx, prm, 1u));  // p log p tables of the entropy
    FloatWeightParams wp{};
    wp.use_exposure = prm->w_exposure > 0.0;
    wp.use_contrast = prm->w_contrast > 0.0;
    wp.use_saturation = prm->w_saturation > 0.0;
    wp.use_entropy = prm->w_entropy > 0.0;
    wp.contrast_window = prm->contrast_window;
    wp.entropy_window = prm->entropy_window;
    wp.gray_projector = prm->gray_projector;
    wp.exp_function = prm->exp_function;
    if (prm->gray_projector == ENB_GRAY_MIXER) {
        const double sm = prm->mixer[0] + prm->mixer[1] + prm->mixer[2];
        for (int i = 0; i < 3; ++i) {
            wp.mixer[i] = prm->mixer[i] / sm;
        }
    }
    wp.w_exposure = (float)prm->w_exposure;
    wp.w_contrast = (float)prm->w_contrast;
    wp.w_saturation = (float)prm->w_saturation;
    wp.w_entropy = (float)prm->w_entropy;
    const double range = float_range_of(prm);
    wp.range = (float)range;
    wp.opt_hi = (float)prm->exp_optimum;
    wp.opt_lo = (float)(prm->exp_optimum - (double)wp.opt_hi);
    const double inv_width = 1.0 / exposure_effective_width(prm->exp_function, prm->exp_width);
    wp.inv_hi = (float)inv_width;
    wp.inv_lo = (float)(inv_width - (double)wp.inv_hi);
    ENB_TRY(float_cutoffs(ctx, prm, range, wp));
    const PixelView pv = pixel_view(src);
    DevBuf abuf;
    BytePlane ap;
    ENB_TRY(alpha_plane(ctx, src, alpha, abuf, ap));
    ENB_LAUNCH(ctx, launch_f_enfuse_mask(FloatPixelView{(const float*)pv.p, pv.pitch, pv.w, pv.h, pv.C, pv.stride}, ap,
                                         wp, ctx->tables, out, ctx->stream));
    return ENB_OK;
}

enb_status enfuse_mask_impl(enb_ctx* ctx, const enb_enfuse_params* prm, const enb_image* src,
                            const enb_image* alpha, const FloatPlane& out)
{
    if (src->dtype == ENB_F32) {
        return enfuse_mask_float(ctx, prm, src, alpha, out);
    }
    const uint32_t maxv = src->dtype == ENB_U8 ? 255u : 65535u;
    ENB_TRY(build_tables(ctx, prm, maxv));
    WeightParams wp{};
    wp.use_exposure = prm->w_exposure > 0.0;
    wp.use_contrast = prm->w_contrast > 0.0;
    wp.use_saturation = prm->w_saturation > 0.0;
    wp.use_entropy = prm->w_entropy > 0.0;
    wp.contrast_window = prm->contrast_window;
    wp.entropy_window = prm->entropy_window;
    wp.gray_projector = prm->gray_projector;
    if (prm->gray_projector == ENB_GRAY_MIXER) {
        const double s = prm->mixer[0] + prm->mixer[1] + prm->mixer[2];
        wp.mixer[0] = prm->mixer[0] / s;
        wp.mixer[1] = prm->mixer[1] / s;
        wp.mixer[2] = prm->mixer[2] / s;
    }
    wp.w_saturation = prm->w_saturation;
    wp.w_sat_hi = (float)prm->w_saturation;
    wp.w_sat_lo = (float)(prm->w_saturation - (double)wp.w_sat_hi);
    wp.maxv = maxv;
    ENB_TRY(int_cutoffs(ctx, prm, maxv, wp));
    ENB_LAUNCH(ctx, launch_enfuse_mask(pixel_view(src), alpha_source(src, alpha), wp, ctx->tables, out, ctx->stream));
    return ENB_OK;
}

// Pyramid types of EnblendNumericTraits (src/numerictraits.h:168-185): u8
// Int16 9.7 image and mask pyramids; u16 Int32 17.7 image, Int32 9.15 mask;
// float: FP32 image pyramid (the reference's double), Int32 9.15 mask.
int fixed_bits_image(int dt) { return dt == ENB_U8 ? ENB_I16 : (dt == ENB_F32 ? ENB_F32 : ENB_I32); }
int fixed_bits_mask(int dt) { return dt == ENB_U8 ? ENB_I16 : ENB_I32; }
int mask_frac(int dt) { return dt == ENB_U8 ? 7 : 15; }
constexpr int kImageFrac = 7;

// Materialise the alpha of an interleaved image as a U8 plane.
enb_status alpha_plane(enb_ctx* ctx, const enb_image* img, const enb_image* alpha, DevBuf& buf, BytePlane& out)
{
    if (alpha && alpha->data) {
        ENB_CHECK(ctx, bytes_ok(alpha, img->width, img->height), "alpha plane: must be U8 of the image size");
        out = byte_plane(alpha);
        return ENB_OK;
    }
    const int64_t pitch = round_up(img->width, 128);
    ENB_CUDA(ctx, buf.alloc((size_t)(pitch * img->height), ctx->stream));
    out = BytePlane{(uint8_t*)buf.p, pitch, img->width, img->height};
    ENB_LAUNCH(ctx, launch_alpha_extract(alpha_source(img, nullptr), out, ctx->stream));
    return ENB_OK;
}

// ---- host-buffer staging ---------------------------------------------------

struct Staged {
    DevBuf buf;
    enb_image dev{};
};

enb_status stage_in(enb_ctx* ctx, const enb_image* host, Staged& s, bool copy)
{
    s.dev = *host;
    const int stride = host->planar ? 1 : (host->pix_stride > 0 ? host->pix_stride : host->channels);
    const int64_t row = (int64_t)host->width * stride * (int64_t)dtype_size(host->dtype);
    // a dense host image keeps its pitch on the device (one contiguous copy)
    // when its rows start on 16-byte boundaries; otherwise the device rows
    // are 128-byte aligned, so that the level-0 passes can move the staged
    // images and masks in 2-D TMA boxes
    const int64_t pitch = (host->pitch == row && row % 16 == 0) ? row : round_up(row, 128);
    ENB_CUDA(ctx, s.buf.alloc((size_t)(pitch * host->height), ctx->stream));
    s.dev.data = s.buf.p;
    s.dev.pitch = pitch;
    if (copy) {
        ENB_CUDA(ctx, cudaMemcpy2DAsync(s.buf.p, pitch, host->data, host->pitch, row, host->height,
                                        cudaMemcpyHostToDevice, ctx->stream));
    }
    return ENB_OK;
}

enb_status stage_out(enb_ctx* ctx, const enb_image* host, const Staged& s)
{
    const int stride = host->planar ? 1 : (host->pix_stride > 0 ? host->pix_stride : host->channels);
    const int64_t row = (int64_t)host->width * stride * (int64_t)dtype_size(host->dtype);
    ENB_CUDA(ctx, cudaMemcpy2DAsync(host->data, host->pitch, s.dev.data, s.dev.pitch, row, host->height,
                                    cudaMemcpyDeviceToHost, ctx->stream));
    return ENB_OK;
}

// ---- drivers ----------------------------------------------------------------

// enblend with the reference's pass structure: every level of the mask,
// white and black pyramids materialised, one kernel per reference operation.
enb_status enblend_plain(enb_ctx* ctx, const enb_image* white, const enb_image* white_alpha, const enb_image* black,
                         const enb_image* black_alpha, const enb_image* mask, const enb_image* out,
                         const enb_image* out_alpha, const enb_fuse_options& o, int32_t* level0)
{
    const int w = black->width, h = black->height, C = black->channels, dt = black->dtype;
    const int L = enb_num_levels(w, h, 1, o.levels);
    const int pdt = fixed_bits_image(dt), mdt = fixed_bits_mask(dt), mf = mask_frac(dt);
    const int wrap = o.wrap != 0;

    // Mask Gaussian pyramid without alpha (src/enblend.h:384-388).
    PyrHolder mg(ctx), wl(ctx), bl(ctx);
    ENB_TRY(pyramid_alloc(ctx, L, w, h, 1, mdt, &mg.p));
    ENB_LAUNCH(ctx, launch_bytes_to_fixed(byte_plane(mask), level_view(mg.p, 0), mf, ctx->stream));
    ENB_TRY(gaussian_levels(ctx, wrap, mg.p, nullptr));

    // White and black Laplacian pyramids (src/enblend.h:418-446).
    DevBuf wa_buf, ba_buf;
    BytePlane wa, ba;
    ENB_TRY(alpha_plane(ctx, white, white_alpha, wa_buf, wa));
    ENB_TRY(alpha_plane(ctx, black, black_alpha, ba_buf, ba));
    ENB_TRY(pyramid_alloc(ctx, L, w, h, C, pdt, &wl.p));
    ENB_TRY(pyramid_alloc(ctx, L, w, h, C, pdt, &bl.p));
    ENB_LAUNCH(ctx, launch_to_fixed(pixel_view(white), level_view(wl.p, 0), kImageFrac, ctx->stream));
    ENB_TRY(gaussian_levels(ctx, wrap, wl.p, &wa));
    ENB_TRY(laplacian_levels(ctx, wrap, wl.p));
    ENB_LAUNCH(ctx, launch_to_fixed(pixel_view(black), level_view(bl.p, 0), kImageFrac, ctx->stream));
    ENB_TRY(gaussian_levels(ctx, wrap, bl.p, &ba));
    ENB_TRY(laplacian_levels(ctx, wrap, bl.p));

    // Union alpha: black alpha where white is transparent, else opaque
    // (src/enblend.h:461-464).
    DevBuf ua_buf;
    BytePlane ua;
    if (out_alpha && out_alpha->data) {
        ENB_CHECK(ctx, bytes_ok(out_alpha, w, h), "out_alpha: must be U8 of the image size");
        ua = byte_plane(out_alpha);
    } else {
        const int64_t pitch = round_up(w, 128);
        ENB_CUDA(ctx, ua_buf.alloc((size_t)(pitch * h), ctx->stream));
        ua = BytePlane{(uint8_t*)ua_buf.p, pitch, w, h};
    }
    ENB_LAUNCH(ctx, launch_union_alpha(ba, ua, 1, ctx->stream));
    ENB_LAUNCH(ctx, launch_union_alpha(wa, ua, 0, ctx->stream));

    // Blend, collapse, copy out (src/enblend.h:468-510).
    for (int l = 0; l < L; ++l) {
        ENB_LAUNCH(ctx, launch_blend(level_view(mg.p, l), level_view(wl.p, l), level_view(bl.p, l), 255 << mf,
                                     ctx->stream));
    }
    ENB_TRY(collapse_levels(ctx, wrap, bl.p));
    if (level0) {
        ENB_LAUNCH(ctx, launch_copy_level0(level_view(bl.p, 0), level0, ctx->stream));
    }
    const PixelView ov = pixel_view(out);
    if (out->data != black->data) {
        ENB_LAUNCH(ctx, launch_copy_pixels(pixel_view(black), out->data, ov.pitch, ctx->stream));
    }
    ENB_LAUNCH(ctx, launch_from_fixed(level_view(bl.p, 0), ua, out->data, ov.pitch, out->dtype, ov.stride, kImageFrac,
                                      o.dither, o.seed, ctx->stream));
    if (ov.stride == 4) {
        ENB_LAUNCH(ctx, launch_alpha_component(ua, out->data, ov.pitch, out->dtype, ctx->stream));
    }
    return ENB_OK;
}

// enblend with fused level passes (enb_fused.cu): level 0 is only read (the
// first reduce converts on the fly, the last pass writes the output pixels);
// levels 1..L-1 of the white, black and mask Gaussian pyramids are built by
// the reduce chain, then one pass per level forms the Laplacians, blends and
// collapses into the result pyramid R.
// Host transfers of a host-buffer call overlapped with the level-0 passes:
// the inputs arrive on the copy stream in row bands, and the level-1 reduces
// of the rows a band completes run as soon as it lands; the output leaves in
// row bands as the level-0 pass finishes them.
struct BandIO {
    std::vector<int> in_end;           // input rows present after band b
    std::vector<cudaEvent_t> in_done;  // recorded on the copy stream after band b
    int out_rows = 0;                  // output rows per band (a multiple of 16)
    std::function<enb_status(int, int)> out_ready;  // rows [r0, r1) of the output are queued
};

enb_status enblend_fused(enb_ctx* ctx, const enb_image* white, const enb_image* white_alpha, const enb_image* black,
                         const enb_image* black_alpha, const enb_image* mask, const enb_image* out,
                         const enb_image* out_alpha, const enb_fuse_options& o, int32_t* level0,
                         BandIO* io = nullptr)
{
    const int w = black->width, h = black->height, C = black->channels, dt = black->dtype;
    const int L = enb_num_levels(w, h, 1, o.levels);
    const int pdt = fixed_bits_image(dt), mdt = fixed_bits_mask(dt), mf = mask_frac(dt);
    const int wrap = o.wrap != 0;
    const int32_t white_value = 255 << mf;

    // Both images' alpha must come from the same kind of source; otherwise
    // materialise both as planes.
    AlphaSrc wa = alpha_source(white, white_alpha), ba = alpha_source(black, black_alpha);
    DevBuf wa_buf, ba_buf;
    if (wa.mode != ba.mode) {
        BytePlane wp, bp;
        ENB_TRY(alpha_plane(ctx, white, white_alpha, wa_buf, wp));
        ENB_TRY(alpha_plane(ctx, black, black_alpha, ba_buf, bp));
        wa = AlphaSrc{};
        wa.mode = kAlphaPlane;
        wa.plane = wp;
        ba = AlphaSrc{};
        ba.mode = kAlphaPlane;
        ba.plane = bp;
    }
    if (out_alpha && out_alpha->data) {
        ENB_CHECK(ctx, bytes_ok(out_alpha, w, h), "out_alpha: must be U8 of the image size");
    }

    PyrHolder gw(ctx), gb(ctx), mg(ctx), rr(ctx);
    AlphaChain awc, abc;
    const int NL = L - 1;  // stored levels 1..L-1 as local levels 0..NL-1
    if (NL >= 1) {
        const int w1 = (w + 1) >> 1, h1 = (h + 1) >> 1;
        ENB_TRY(pyramid_alloc(ctx, NL, w1, h1, C, pdt, &gw.p));
        ENB_TRY(pyramid_alloc(ctx, NL, w1, h1, C, pdt, &gb.p));
        ENB_TRY(pyramid_alloc(ctx, NL, w1, h1, C, pdt, &rr.p));
        ENB_TRY(pyramid_alloc(ctx, NL, w1, h1, 1, mdt, &mg.p));
        ENB_CUDA(ctx, awc.alloc(NL, w1, h1, ctx->stream));
        ENB_CUDA(ctx, abc.alloc(NL, w1, h1, ctx->stream));
        // Down sweep (src/enblend.h:384-446: the three Gaussian pyramids).
        if (io) {
            // level-1 tile rows as their source rows arrive
            int done = 0;
            for (size_t b = 0; b < io->in_end.size(); ++b) {
                ENB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, io->in_done[b], 0));
                const int ready = reduce_tile_rows_ready(h, h1, io->in_end[b]);
                if (ready > done) {
                    ENB_LAUNCH(ctx, launch_reduce0_alpha2(pixel_view(white), wa, level_view(gw.p, 0), awc.level(0),
                                                          pixel_view(black), ba, level_view(gb.p, 0), abc.level(0),
                                                          kImageFrac, wrap, ctx->stream, done, ready - done));
                    ENB_LAUNCH(ctx, launch_reduce0_bytes(byte_plane(mask), mf, level_view(mg.p, 0), wrap, ctx->stream,
                                                         done, ready - done));
                    done = ready;
                }
            }
        } else {
            ENB_LAUNCH(ctx, launch_reduce0_alpha2(pixel_view(white), wa, level_view(gw.p, 0), awc.level(0),
                                                  pixel_view(black), ba, level_view(gb.p, 0), abc.level(0), kImageFrac,
                                                  wrap, ctx->stream));
            ENB_LAUNCH(ctx, launch_reduce0_bytes(byte_plane(mask), mf, level_view(mg.p, 0), wrap, ctx->stream));
        }
        for (int j = 1; j < NL; ++j) {
            ENB_CHECK(ctx, gw.p->w[j - 1] > 1 && gw.p->h[j - 1] > 1, "reduce: src image too small in reduce");
        }
        // Levels first..NL-1 (all at most coarse_pixels pixels) go to the one
        // coarse launch, which also blends the top and collapses down to first.
        const int64_t cpx = o.coarse_pixels == 0 ? kCoarsePixels : (int64_t)o.coarse_pixels;
        int first = NL;
        if (cpx > 0) {
            for (int j = 1; j < NL; ++j) {
                if ((int64_t)gw.p->w[j] * gw.p->h[j] <= cpx) {
                    first = j;
                    break;
                }
            }
        }
        for (int j = 1; j < first; ++j) {
            const BytePlane sa = awc.level(j - 1), da = awc.level(j), sb = abc.level(j - 1), db = abc.level(j);
            ENB_LAUNCH(ctx, launch_reduce_img2_mask(wrap, level_view(gw.p, j - 1), sa, level_view(gw.p, j), da,
                                                    level_view(gb.p, j - 1), sb, level_view(gb.p, j), db,
                                                    level_view(mg.p, j - 1), level_view(mg.p, j), ctx->stream));
        }
        int up_from = NL - 2;
        if (first < NL) {
            CoarseHost ch{};
            ch.n = NL - first + 1;
            for (int s = 0; s < ch.n; ++s) {
                const int j = first - 1 + s;
                ch.gw[s] = level_view(gw.p, j);
                ch.gb[s] = level_view(gb.p, j);
                ch.rr[s] = level_view(rr.p, j);
                ch.mg[s] = level_view(mg.p, j);
                ch.aw[s] = awc.level(j);
                ch.ab[s] = abc.level(j);
            }
            ch.white_value = white_value;
            ch.wrap = wrap;
            ENB_LAUNCH(ctx, launch_coarse(ch, ctx->stream));
            up_from = first - 1;
        } else {
            // Up sweep: top level blend, then Laplacian + blend + collapse per
            // level (src/blend.h:81-121, src/pyramid.h:1758-1784).
            ENB_LAUNCH(ctx, launch_blend_into(level_view(mg.p, NL - 1), level_view(gw.p, NL - 1),
                                              level_view(gb.p, NL - 1), level_view(rr.p, NL - 1), white_value,
                                              ctx->stream));
        }
        for (int j = up_from; j >= 0; --j) {
            ENB_LAUNCH(ctx, launch_up_level(level_view(gw.p, j + 1), level_view(gb.p, j + 1), level_view(rr.p, j + 1),
                                            level_view(mg.p, j), level_view(gw.p, j), level_view(gb.p, j),
                                            level_view(rr.p, j), white_value, wrap, ctx->stream));
        }
    }
    // Level 0 straight to the output pixels (src/enblend.h:468-510).
    Out0Host h0{};
    h0.white = pixel_view(white);
    h0.black = pixel_view(black);
    h0.white_alpha = wa;
    h0.black_alpha = ba;
    h0.mask = byte_plane(mask);
    h0.mfrac = mf;
    h0.white_value = white_value;
    h0.out = out->data;
    h0.opitch = pixel_view(out).pitch;
    h0.out_alpha = (out_alpha && out_alpha->data) ? byte_plane(out_alpha) : BytePlane{nullptr, 0, w, h};
    h0.level0 = level0;
    h0.frac = kImageFrac;
    h0.dither = o.dither;
    h0.wrap = wrap;
    h0.seed = o.seed;
    h0.err = device_error_word(ctx);
    h0.tx_extra = ctx->tx_extra;
    PlanarView g0{}, b0{}, r0{};
    if (NL >= 1) {
        g0 = level_view(gw.p, 0);
        b0 = level_view(gb.p, 0);
        r0 = level_view(rr.p, 0);
    }
    const PlanarView* pg = NL >= 1 ? &g0 : nullptr;
    const PlanarView* pb = NL >= 1 ? &b0 : nullptr;
    const PlanarView* pr = NL >= 1 ? &r0 : nullptr;
    if (io) {
        // every input row is needed here (a single level reads them only now)
        if (!io->in_done.empty()) {
            ENB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, io->in_done.back(), 0));
        }
        // output rows in bands, each copied out as soon as it is written
        for (int y0 = 0; y0 < h; y0 += io->out_rows) {
            const int y1 = std::min(h, y0 + io->out_rows);
            ENB_LAUNCH(ctx, launch_out0(pg, pb, pr, h0, ctx->stream, y0 / 16, (y1 - y0 + 15) / 16));
            ENB_TRY(io->out_ready(y0, y1));
        }
    } else {
        ENB_LAUNCH(ctx, launch_out0(pg, pb, pr, h0, ctx->stream));
    }
    return ENB_OK;
}

// enfuseMain's pyramid section for 8/16-bit images as fused level passes
// (enb_efuse.cu): weights of all exposures per tile with the normalised
// masks as level 0 of the mask pyramids, K-job reduces, one up pass per
// level, level 0 straight to the output pixels.  The integers are the
// per-operation path's (and the reference's).
enb_status enfuse_fused(enb_ctx* ctx, const enb_enfuse_params* prm, int K, const enb_image* images,
                        const enb_image* alphas, const enb_image* masks_in, const enb_image* out,
                        const enb_image* out_alpha, const enb_fuse_options& o, int32_t* level0, int L)
{
    const int w = images[0].width, h = images[0].height, C = images[0].channels, dt = images[0].dtype;
    const size_t ps = dt == ENB_U8 ? 2 : 4;  // Int16 / Int32 pyramids and masks
    EfuseHost eh{};
    eh.K = K;
    eh.L = L;
    eh.w = w;
    eh.h = h;
    eh.C = C;
    eh.S = pixel_view(&images[0]).stride;
    eh.dtype = dt;
    eh.hard = o.hard_mask != 0;
    eh.wrap = o.wrap != 0;
    eh.dither = o.dither;
    eh.seed = o.seed;
    eh.level0 = level0;
    const uint32_t maxv = dt == ENB_U8 ? 255u : 65535u;
    if (!masks_in) {
        ENB_TRY(build_tables(ctx, prm, maxv));
        WeightParams& wp = eh.wp;
        wp.use_exposure = prm->w_exposure > 0.0;
        wp.use_contrast = prm->w_contrast > 0.0;
        wp.use_saturation = prm->w_saturation > 0.0;
        wp.use_entropy = prm->w_entropy > 0.0;
        wp.contrast_window = prm->contrast_window;
        wp.entropy_window = prm->entropy_window;
        wp.gray_projector = prm->gray_projector;
        if (prm->gray_projector == ENB_GRAY_MIXER) {
            const double sm = prm->mixer[0] + prm->mixer[1] + prm->mixer[2];
            for (int i = 0; i < 3; ++i) {
                wp.mixer[i] = prm->mixer[i] / sm;
            }
        }
        wp.w_saturation = prm->w_saturation;
        wp.w_sat_hi = (float)prm->w_saturation;
        wp.w_sat_lo = (float)(prm->w_saturation - (double)wp.w_sat_hi);
        wp.maxv = maxv;
        ENB_TRY(int_cutoffs(ctx, prm, maxv, wp));
        eh.tab = ctx->tables;
    } else {
        eh.wp.maxv = maxv;
    }
    for (int k = 0; k < K; ++k) {
        eh.img[k] = pixel_view(&images[k]);
        eh.alpha[k] = alpha_source(&images[k], alphas ? &alphas[k] : nullptr);
        if (masks_in) {
            ENB_CHECK(ctx, floats_ok(&masks_in[k], w, h), "masks_in: F32 planes of the image size expected");
            eh.masks_in[k] = (const float*)masks_in[k].data;
            eh.mipitch[k] = masks_in[k].pitch / 4;
        }
    }
    // level geometry and one allocation for every plane
    int64_t total = 0;
    int64_t off_m[kMaxLevels] = {}, off_g[kMaxLevels] = {}, off_a[kMaxLevels] = {}, off_u[kMaxLevels] = {},
            off_r[kMaxLevels] = {};
    for (int l = 0; l < L; ++l) {
        eh.lw[l] = l == 0 ? w : (eh.lw[l - 1] + 1) >> 1;
        eh.lh[l] = l == 0 ? h : (eh.lh[l - 1] + 1) >> 1;
        eh.pitch[l] = round_up(eh.lw[l], 64);
        eh.apitch[l] = round_up(eh.lw[l], 128);
        const int64_t plane = eh.pitch[l] * eh.lh[l] * (int64_t)ps, aplane = eh.apitch[l] * eh.lh[l];
        off_m[l] = total;
        total += K * plane;
        if (l >= 1) {
            off_g[l] = total;
            total += K * C * plane;
            off_a[l] = total;
            total += round_up(K * aplane, 256);
            off_u[l] = total;
            total += round_up(aplane, 256);
            off_r[l] = total;
            total += C * plane;
        }
    }
    BytePlane ua;
    DevBuf ua_buf;
    if (out_alpha && out_alpha->data) {
        ENB_CHECK(ctx, bytes_ok(out_alpha, w, h), "out_alpha: must be U8 of the image size");
        ua = byte_plane(out_alpha);
    } else {
        const int64_t pitch = round_up(w, 128);
        ENB_CUDA(ctx, ua_buf.alloc((size_t)(pitch * h), ctx->stream));
        ua = BytePlane{(uint8_t*)ua_buf.p, pitch, w, h};
    }
    DevBuf mem;
    ENB_CUDA(ctx, mem.alloc((size_t)total, ctx->stream));
    uint8_t* base = (uint8_t*)mem.p;
    for (int l = 0; l < L; ++l) {
        const int64_t plane = eh.pitch[l] * eh.lh[l] * (int64_t)ps, aplane = eh.apitch[l] * eh.lh[l];
        for (int k = 0; k < K; ++k) {
            eh.m[k][l] = base + off_m[l] + k * plane;
            if (l >= 1) {
                eh.g[k][l] = base + off_g[l] + (int64_t)k * C * plane;
                eh.a[k][l] = base + off_a[l] + k * aplane;
            }
        }
        if (l >= 1) {
            eh.u[l] = base + off_u[l];
            eh.r[l] = base + off_r[l];
        }
    }
    eh.u[0] = ua.p;
    eh.upitch0 = ua.pitch;
    eh.out = out->data;
    eh.opitch = pixel_view(out).pitch;

    ENB_LAUNCH(ctx, launch_ef_weights(eh, ctx->stream));
    for (int l = 0; l + 1 < L; ++l) {
        ENB_LAUNCH(ctx, launch_ef_reduce(eh, l, 0, ctx->stream));
        ENB_LAUNCH(ctx, launch_ef_reduce(eh, l, 1, ctx->stream));
    }
    ENB_LAUNCH(ctx, launch_ef_top(eh, ctx->stream));
    for (int l = L - 2; l >= 1; --l) {
        ENB_LAUNCH(ctx, launch_ef_up(eh, l, ctx->stream));
    }
    ENB_LAUNCH(ctx, launch_ef_out0(eh, ctx->stream));
    return ENB_OK;
}

enb_status enfuse_device(enb_ctx* ctx, const enb_enfuse_params* prm, int K, const enb_image* images,
                         const enb_image* alphas, const enb_image* masks_in, const enb_image* out,
                         const enb_image* out_alpha, const enb_fuse_options& o, int32_t* level0)
{
    const int w = images[0].width, h = images[0].height, C = images[0].channels, dt = images[0].dtype;
    const int L = enb_num_levels(w, h, 1, o.levels);
    if (!o.plain && dt != ENB_F32 && K <= kEfuseMaxK && L >= 2 && pixel_view(out).stride == pixel_view(&images[0]).stride) {
        // one alpha mode for all exposures (the level-1 reduce is compiled per mode)
        bool uniform = true;
        const int m0 = alpha_source(&images[0], alphas ? &alphas[0] : nullptr).mode;
        for (int k = 1; k < K; ++k) {
            uniform = uniform && alpha_source(&images[k], alphas ? &alphas[k] : nullptr).mode == m0;
        }
        if (uniform) {
            return enfuse_fused(ctx, prm, K, images, alphas, masks_in, out, out_alpha, o, level0, L);
        }
    }
    const int pdt = fixed_bits_image(dt), mdt = fixed_bits_mask(dt), mf = mask_frac(dt);
    const int wrap = o.wrap != 0;
    const int64_t fpitch = round_up(w, 32);

    // Weight masks (enfuseMask or --load-masks), their sum and the union alpha
    // (src/enfuse.h:1281-1391).
    DevBuf mask_mem, norm_mem;
    ENB_CUDA(ctx, mask_mem.alloc((size_t)(fpitch * h * 4) * K, ctx->stream));
    ENB_CUDA(ctx, norm_mem.alloc((size_t)(fpitch * h * 4), ctx->stream));
    std::vector<FloatPlane> masks(K);
    const FloatPlane norm{(float*)norm_mem.p, fpitch, w, h};
    std::vector<DevBuf> abufs(K);
    std::vector<BytePlane> aplanes(K);
    DevBuf ua_buf;
    BytePlane ua;
    if (out_alpha && out_alpha->data) {
        ENB_CHECK(ctx, bytes_ok(out_alpha, w, h), "out_alpha: must be U8 of the image size");
        ua = byte_plane(out_alpha);
    } else {
        const int64_t pitch = round_up(w, 128);
        ENB_CUDA(ctx, ua_buf.alloc((size_t)(pitch * h), ctx->stream));
        ua = BytePlane{(uint8_t*)ua_buf.p, pitch, w, h};
    }
    for (int k = 0; k < K; ++k) {
        masks[k] = FloatPlane{(float*)mask_mem.p + (size_t)k * fpitch * h, fpitch, w, h};
        ENB_TRY(alpha_plane(ctx, &images[k], alphas ? &alphas[k] : nullptr, abufs[k], aplanes[k]));
        if (masks_in) {
            ENB_CHECK(ctx, floats_ok(&masks_in[k], w, h), "masks_in: F32 planes of the image size expected");
            ENB_CUDA(ctx, cudaMemcpy2DAsync(masks[k].p, fpitch * 4, masks_in[k].data, masks_in[k].pitch, (size_t)w * 4, h,
                                            cudaMemcpyDeviceToDevice, ctx->stream));
        } else {
            enb_image ai{};
            ai.data = aplanes[k].p;
            ai.pitch = aplanes[k].pitch;
            ai.width = w;
            ai.height = h;
            ai.channels = 1;
            ai.pix_stride = 1;
            ai.dtype = ENB_U8;
            ENB_TRY(enfuse_mask_impl(ctx, prm, &images[k], &ai, masks[k]));
        }
        ENB_LAUNCH(ctx, launch_union_alpha(aplanes[k], ua, k == 0, ctx->stream));
        ENB_LAUNCH(ctx, launch_norm_accumulate(masks[k], norm, k == 0, ctx->stream));
    }
    if (o.hard_mask) {
        ENB_CHECK(ctx, K <= 64, "hard mask: at most 64 images");
        ENB_LAUNCH(ctx, launch_hard_mask(masks.data(), K, ctx->stream));
    }

    // Pyramids, merge and accumulation (src/enfuse.h:1501-1595).
    PyrHolder result(ctx), lp(ctx), mg(ctx);
    ENB_TRY(pyramid_alloc(ctx, L, w, h, C, pdt, &result.p));
    ENB_TRY(pyramid_alloc(ctx, L, w, h, C, pdt, &lp.p));
    ENB_TRY(pyramid_alloc(ctx, L, w, h, 1, mdt, &mg.p));
    for (int k = 0; k < K; ++k) {
        ENB_LAUNCH(ctx, launch_to_fixed(pixel_view(&images[k]), level_view(lp.p, 0), kImageFrac, ctx->stream));
        ENB_TRY(gaussian_levels(ctx, wrap, lp.p, &aplanes[k]));
        ENB_TRY(laplacian_levels(ctx, wrap, lp.p));
        if (o.hard_mask) {
            ENB_LAUNCH(ctx, launch_float_to_fixed(masks[k], level_view(mg.p, 0), mf, ctx->stream));
        } else {
            ENB_LAUNCH(ctx, launch_soft_mask_to_fixed(masks[k], norm, K, level_view(mg.p, 0), mf, ctx->stream));
        }
        ENB_TRY(gaussian_levels(ctx, wrap, mg.p, &ua));
        for (int l = 0; l < L; ++l) {
            ENB_LAUNCH(ctx, launch_mask_mul_acc(level_view(lp.p, l), level_view(mg.p, l), 255 << mf,
                                                level_view(result.p, l), k > 0, ctx->stream));
        }
    }
    ENB_TRY(collapse_levels(ctx, wrap, result.p));
    if (level0) {
        ENB_LAUNCH(ctx, launch_copy_level0(level_view(result.p, 0), level0, ctx->stream));
    }
    const PixelView ov = pixel_view(out);
    ENB_CUDA(ctx, cudaMemset2DAsync(out->data, out->pitch, 0, (size_t)w * ov.stride * dtype_size(dt), h, ctx->stream));
    ENB_LAUNCH(ctx, launch_from_fixed(level_view(result.p, 0), ua, out->data, ov.pitch, out->dtype, ov.stride,
                                      kImageFrac, o.dither, o.seed, ctx->stream));
    if (ov.stride == 4) {
        ENB_LAUNCH(ctx, launch_alpha_component(ua, out->data, ov.pitch, out->dtype, ctx->stream));
    }
    return ENB_OK;
}

bool same_geometry(const enb_image* a, const enb_image* b)
{
    return a->width == b->width && a->height == b->height && a->channels == b->channels && a->dtype == b->dtype;
}

// Device address of g_noalloc_scratch on the context's device, looked up on
// every call with that device current (cheap once the module is loaded, and
// still right after the host application reset the device).
std::mutex g_noalloc_mu;

enb_status noalloc_scratch(enb_ctx* ctx, void** out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    int cur = -1;
    ENB_CUDA(ctx, cudaGetDevice(&cur));
    if (cur != ctx->device) {
        ENB_CUDA(ctx, cudaSetDevice(ctx->device));
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != ctx->device) {
        cudaSetDevice(cur);
    }
    if (e != cudaSuccess || !p) {
        return cuda_fail(ctx, e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress(noalloc scratch)");
    }
    *out = p;
    return ENB_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================

// Rows of the input bands of the banded host path (a multiple of the 32
// source rows of a level-1 tile row) and of its output bands.
constexpr int kInBandRows = 256;
constexpr int kOutBandRows = 512;

static cudaError_t ensure_io(enb_ctx* ctx, size_t events)
{
    if (!ctx->copy_stream) {
        const cudaError_t e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            return e;
        }
    }
    while (ctx->io_events.size() < events) {
        cudaEvent_t ev;
        const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            return e;
        }
        ctx->io_events.push_back(ev);
    }
    return cudaSuccess;
}

static cudaError_t copy_rows(const enb_image* host, const enb_image& dev, int r0, int r1, cudaMemcpyKind kind,
                             cudaStream_t st)
{
    const int stride = host->planar ? 1 : (host->pix_stride > 0 ? host->pix_stride : host->channels);
    const size_t row = (size_t)host->width * stride * dtype_size(host->dtype);
    const char* hp = (const char*)host->data + (int64_t)r0 * host->pitch;
    const char* dp = (const char*)dev.data + (int64_t)r0 * dev.pitch;
    if (kind == cudaMemcpyHostToDevice) {
        return cudaMemcpy2DAsync((void*)dp, dev.pitch, hp, host->pitch, row, r1 - r0, kind, st);
    }
    return cudaMemcpy2DAsync((void*)hp, host->pitch, dp, dev.pitch, row, r1 - r0, kind, st);
}

// enblend on host buffers with the transfers overlapped: input row bands go
// to the device on the copy stream while the level-1 reduces consume the
// bands that have landed, and output row bands come back while the level-0
// pass writes the next ones.  The call returns once the output is in host
// memory, like the unbanded path.
enb_status enblend_host_banded(enb_ctx* ctx, const enb_image* white, const enb_image* white_alpha,
                               const enb_image* black, const enb_image* black_alpha, const enb_image* mask,
                               const enb_image* out, const enb_image* out_alpha, const enb_fuse_options& o)
{
    const int w = black->width, h = black->height, C = black->channels;
    const int nin = (h + kInBandRows - 1) / kInBandRows;
    const int nout = (h + kOutBandRows - 1) / kOutBandRows;
    ENB_CUDA(ctx, ensure_io(ctx, (size_t)(nin + nout + 2)));
    cudaStream_t cs = ctx->copy_stream;
    cudaEvent_t* ev = ctx->io_events.data();

    Staged sw, sb, swa, sba, sm, soa;
    ENB_TRY(stage_in(ctx, white, sw, false));
    ENB_TRY(stage_in(ctx, black, sb, false));
    ENB_TRY(stage_in(ctx, mask, sm, false));
    const bool has_wa = white_alpha && white_alpha->data, has_ba = black_alpha && black_alpha->data;
    if (has_wa) {
        ENB_TRY(stage_in(ctx, white_alpha, swa, false));
    }
    if (has_ba) {
        ENB_TRY(stage_in(ctx, black_alpha, sba, false));
    }
    const bool want_alpha = out_alpha && out_alpha->data;
    if (want_alpha) {
        ENB_TRY(stage_in(ctx, out_alpha, soa, false));
    }
    DevBuf l0;
    if (o.level0_out) {
        ENB_CUDA(ctx, l0.alloc((size_t)w * h * C * 4, ctx->stream));
    }
    // the staging buffers come from the stream-ordered pool of the main stream
    ENB_CUDA(ctx, cudaEventRecord(ev[nin + nout], ctx->stream));
    ENB_CUDA(ctx, cudaStreamWaitEvent(cs, ev[nin + nout], 0));

    BandIO io;
    for (int b = 0; b < nin; ++b) {
        const int r0 = b * kInBandRows, r1 = std::min(h, r0 + kInBandRows);
        ENB_CUDA(ctx, copy_rows(white, sw.dev, r0, r1, cudaMemcpyHostToDevice, cs));
        ENB_CUDA(ctx, copy_rows(black, sb.dev, r0, r1, cudaMemcpyHostToDevice, cs));
        ENB_CUDA(ctx, copy_rows(mask, sm.dev, r0, r1, cudaMemcpyHostToDevice, cs));
        if (has_wa) {
            ENB_CUDA(ctx, copy_rows(white_alpha, swa.dev, r0, r1, cudaMemcpyHostToDevice, cs));
        }
        if (has_ba) {
            ENB_CUDA(ctx, copy_rows(black_alpha, sba.dev, r0, r1, cudaMemcpyHostToDevice, cs));
        }
        ENB_CUDA(ctx, cudaEventRecord(ev[b], cs));
        io.in_end.push_back(r1);
        io.in_done.push_back(ev[b]);
    }
    int next_out = 0;
    io.out_rows = kOutBandRows;
    io.out_ready = [&](int y0, int y1) -> enb_status {
        cudaEvent_t e = ev[nin + next_out++];
        ENB_CUDA(ctx, cudaEventRecord(e, ctx->stream));
        ENB_CUDA(ctx, cudaStreamWaitEvent(cs, e, 0));
        ENB_CUDA(ctx, copy_rows(out, sb.dev, y0, y1, cudaMemcpyDeviceToHost, cs));
        if (want_alpha) {
            ENB_CUDA(ctx, copy_rows(out_alpha, soa.dev, y0, y1, cudaMemcpyDeviceToHost, cs));
        }
        return ENB_OK;
    };
    const enb_status st = enblend_fused(ctx, &sw.dev, has_wa ? &swa.dev : nullptr, &sb.dev, has_ba ? &sba.dev : nullptr,
                                        &sm.dev, &sb.dev, want_alpha ? &soa.dev : nullptr, o, (int32_t*)l0.p, &io);
    if (st != ENB_OK) {
        cudaStreamSynchronize(cs);
        cudaStreamSynchronize(ctx->stream);
        return st;
    }
    if (o.level0_out) {
        ENB_CUDA(ctx, cudaMemcpyAsync(o.level0_out, l0.p, (size_t)w * h * C * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    // the main stream (and with it the frees of the staging buffers) waits
    // for the last output band
    ENB_CUDA(ctx, cudaEventRecord(ev[nin + nout + 1], cs));
    ENB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev[nin + nout + 1], 0));
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

extern "C" {

int enb_abi_version(void) { return ENBGPU_ABI_VERSION; }

enb_status enb_create(int device, enb_ctx** out)
{
    if (!out) {
        return ENB_ERR_INVALID;
    }
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0 || device < 0 || device >= n) {
        cudaGetLastError();
        return ENB_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        return ENB_ERR_CUDA;
    }
    // Keep freed pyramid memory in the stream-ordered pool across
    // synchronisations instead of returning it to the driver after each call.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    enb_ctx* ctx = new enb_ctx();
    ctx->device = device;
    *out = ctx;
    return ENB_OK;
}

enb_status enb_destroy(enb_ctx* ctx)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    if (ctx->table_mem) {
        cudaFreeAsync(ctx->table_mem, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
    }
    prof_resolve(ctx);
    for (cudaEvent_t e : ctx->pool) {
        cudaEventDestroy(e);
    }
    for (cudaEvent_t e : ctx->io_events) {
        cudaEventDestroy(e);
    }
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->batch) {
        cudaDeviceSynchronize();
        ctx->batch.reset();
    }
    if (ctx->dev_err) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->dev_err);
    }
    delete ctx;
    return ENB_OK;
}

enb_status enb_profile_enable(enb_ctx* ctx, int enable)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    prof_resolve(ctx);
    ctx->kernels.clear();
    ctx->prof = enable != 0;
    return ENB_OK;
}

int enb_profile_count(enb_ctx* ctx) { return ctx ? (int)ctx->kernels.size() : 0; }

enb_status enb_profile_entry(enb_ctx* ctx, int i, const char** name, uint64_t* launches, double* total_ms,
                             double* bytes)
{
    if (!ctx || i < 0 || i >= (int)ctx->kernels.size()) {
        return ENB_ERR_INVALID;
    }
    prof_resolve(ctx);
    const auto& k = ctx->kernels[(size_t)i];
    if (name) {
        *name = k.name.c_str();
    }
    if (launches) {
        *launches = k.launches;
    }
    if (total_ms) {
        *total_ms = k.ms;
    }
    if (bytes) {
        *bytes = k.bytes;
    }
    return ENB_OK;
}

enb_status enb_set_stream(enb_ctx* ctx, void* stream)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ctx->stream = (cudaStream_t)stream;
    return ENB_OK;
}

enb_status enb_synchronize(enb_ctx* ctx)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_error(ctx);
}

const char* enb_last_error(const enb_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

enb_status enb_debug_overarm_tile_waits(enb_ctx* ctx, uint32_t extra_bytes)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, extra_bytes <= 4096, "debug_overarm_tile_waits: at most 4096 extra bytes");
    ctx->tx_extra = extra_bytes;
    return ENB_OK;
}

uint64_t enb_launch_count(const enb_ctx* ctx) { return ctx ? ctx->launches : 0; }

void enb_default_enfuse_params(enb_enfuse_params* p)
{
    if (!p) {
        return;
    }
    memset(p, 0, sizeof *p);
    p->w_exposure = 1.0;
    p->w_saturation = 0.0;
    p->w_contrast = 0.0;
    p->w_entropy = 0.0;
    p->exp_optimum = 0.5;
    p->exp_width = 0.2;
    p->exp_function = ENB_EXP_GAUSSIAN;
    p->contrast_window = 5;
    p->entropy_window = 3;
    p->gray_projector = ENB_GRAY_AVERAGE;
    // --exposure-cutoff 0%:100%:anti-value:value, --entropy-cutoff 0%:100%
    // (src/enfuse.cc:124-127, 141-142)
    p->exp_cutoff_lower = 0.0;
    p->exp_cutoff_lower_pct = 1;
    p->exp_cutoff_upper = 100.0;
    p->exp_cutoff_upper_pct = 1;
    p->exp_cutoff_lower_projector = ENB_GRAY_ANTI_VALUE;
    p->exp_cutoff_upper_projector = ENB_GRAY_VALUE;
    p->ent_cutoff_lower = 0.0;
    p->ent_cutoff_lower_pct = 1;
    p->ent_cutoff_upper = 100.0;
    p->ent_cutoff_upper_pct = 1;
}

void enb_default_fuse_options(enb_fuse_options* o)
{
    if (!o) {
        return;
    }
    memset(o, 0, sizeof *o);
    o->dither = ENB_DITHER_HASH;
    o->seed = 0x5eed;
    o->graph = 1;
}

int enb_num_levels(int w, int h, int min_levels, int exact_levels)
{
    unsigned int shortdim = (unsigned int)std::min(w, h);
    int allowable = min_levels;
    while (allowable <= kMaxLevels) {
        if (shortdim <= 8u) {
            break;
        }
        shortdim = (shortdim + 1u) >> 1;
        ++allowable;
    }
    if (allowable > min_levels) {
        if (exact_levels >= 1) {
            allowable = std::min(allowable, exact_levels);
        } else if (exact_levels < 0) {
            allowable = allowable + exact_levels >= min_levels ? allowable + exact_levels : min_levels;
        }
    }
    return allowable;
}

enb_status enb_pyramid_create(enb_ctx* ctx, int levels, int width, int height, int channels, int dtype,
                              enb_pyramid** out)
{
    if (!ctx || !out) {
        return ENB_ERR_INVALID;
    }
    return pyramid_alloc(ctx, levels, width, height, channels, dtype, out);
}

enb_status enb_pyramid_free(enb_ctx* ctx, enb_pyramid* pyr)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    pyramid_release(ctx, pyr);
    return ENB_OK;
}

int enb_pyramid_levels(const enb_pyramid* pyr) { return pyr ? pyr->levels : 0; }

enb_status enb_pyramid_level(const enb_pyramid* p, int l, enb_image* out)
{
    if (!p || !out || l < 0 || l >= p->levels) {
        return ENB_ERR_INVALID;
    }
    const int64_t es = (int64_t)dtype_size(p->dtype);
    memset(out, 0, sizeof *out);
    out->data = (char*)p->base + p->offset[l];
    out->pitch = p->pitch[l] * es;
    out->plane_pitch = p->pitch[l] * p->h[l] * es;
    out->width = p->w[l];
    out->height = p->h[l];
    out->channels = p->C;
    out->pix_stride = 1;
    out->dtype = p->dtype;
    out->planar = 1;
    return ENB_OK;
}

static enb_status level_copy(enb_ctx* ctx, const enb_pyramid* p, int l, void* host, bool to_host)
{
    if (!ctx || !p || !host || l < 0 || l >= p->levels) {
        return fail(ctx, ENB_ERR_INVALID, "pyramid level copy: bad arguments");
    }
    const size_t es = dtype_size(p->dtype);
    const size_t row = (size_t)p->w[l] * es;
    char* dev = (char*)p->base + p->offset[l];
    const size_t dpitch = (size_t)p->pitch[l] * es;
    for (int c = 0; c < p->C; ++c) {
        char* dplane = dev + (size_t)c * dpitch * p->h[l];
        char* hplane = (char*)host + (size_t)c * row * p->h[l];
        if (to_host) {
            ENB_CUDA(ctx, cudaMemcpy2DAsync(hplane, row, dplane, dpitch, row, p->h[l], cudaMemcpyDeviceToHost, ctx->stream));
        } else {
            ENB_CUDA(ctx, cudaMemcpy2DAsync(dplane, dpitch, hplane, row, row, p->h[l], cudaMemcpyHostToDevice, ctx->stream));
        }
    }
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return ENB_OK;
}

enb_status enb_pyramid_read_level(enb_ctx* ctx, const enb_pyramid* p, int l, void* host_dst)
{
    return level_copy(ctx, p, l, host_dst, true);
}

enb_status enb_pyramid_write_level(enb_ctx* ctx, enb_pyramid* p, int l, const void* host_src)
{
    return level_copy(ctx, p, l, const_cast<void*>(host_src), false);
}

enb_status enb_to_pyramid(enb_ctx* ctx, const enb_image* src, const enb_image* dst, int frac)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, planar_ok(dst), "to_pyramid: dst must be a planar I16/I32/F32 level");
    ENB_CHECK(ctx, frac >= 0 && frac <= 24, "to_pyramid: frac_bits outside 0..24");
    ENB_CHECK(ctx, src && src->width == dst->width && src->height == dst->height, "to_pyramid: size mismatch");
    if (dst->dtype == ENB_F32) {
        ENB_CHECK(ctx, pixels_ok(src) && src->dtype == ENB_F32 && src->channels == dst->channels,
                  "to_pyramid: an F32 level takes an interleaved F32 image of its channel count");
        ENB_LAUNCH(ctx, launch_to_fixed(pixel_view(src), planar_view(dst), frac, ctx->stream));
        return ENB_OK;
    }
    if (src->dtype == ENB_F32) {
        ENB_CHECK(ctx, src->channels == 1 && dst->channels == 1 && floats_ok(src, src->width, src->height),
                  "to_pyramid: F32 sources are single-channel planes");
        ENB_LAUNCH(ctx, launch_float_to_fixed(float_plane(src), planar_view(dst), frac, ctx->stream));
        return ENB_OK;
    }
    ENB_CHECK(ctx, pixels_ok(src) && src->dtype != ENB_F32, "to_pyramid: src must be interleaved U8/U16");
    ENB_CHECK(ctx, src->channels == dst->channels, "to_pyramid: channel mismatch");
    ENB_LAUNCH(ctx, launch_to_fixed(pixel_view(src), planar_view(dst), frac, ctx->stream));
    return ENB_OK;
}

enb_status enb_reduce(enb_ctx* ctx, int wrap, const enb_image* src, const enb_image* src_alpha, const enb_image* dst,
                      const enb_image* dst_alpha)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, planar_ok(src) && planar_ok(dst), "reduce: planar I16/I32 levels expected");
    ENB_CHECK(ctx, src->dtype == dst->dtype && src->channels == dst->channels && (src->channels == 1 || src->channels == 3),
              "reduce: dtype/channel mismatch");
    ENB_CHECK(ctx, src->width > 1 && src->height > 1, "reduce: src image too small in reduce");
    ENB_CHECK(ctx, dst->width == (src->width + 1) >> 1 && dst->height == (src->height + 1) >> 1,
              "reduce: dst must be ((w+1)>>1, (h+1)>>1)");
    if (src_alpha) {
        ENB_CHECK(ctx, bytes_ok(src_alpha, src->width, src->height) && bytes_ok(dst_alpha, dst->width, dst->height),
                  "reduce: alpha planes must be U8 of the level sizes");
        const BytePlane sa = byte_plane(src_alpha), da = byte_plane(dst_alpha);
        ENB_LAUNCH(ctx, launch_reduce(wrap != 0, planar_view(src), &sa, planar_view(dst), &da, ctx->stream));
    } else {
        ENB_LAUNCH(ctx, launch_reduce(wrap != 0, planar_view(src), nullptr, planar_view(dst), nullptr, ctx->stream));
    }
    return ENB_OK;
}

enb_status enb_expand(enb_ctx* ctx, int add, int wrap, const enb_image* src, const enb_image* dst)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, planar_ok(src) && planar_ok(dst), "expand: planar I16/I32 levels expected");
    ENB_CHECK(ctx, src->dtype == dst->dtype && src->channels == dst->channels && (src->channels == 1 || src->channels == 3),
              "expand: dtype/channel mismatch");
    ENB_CHECK(ctx, src->width == (dst->width + 1) >> 1 && src->height == (dst->height + 1) >> 1,
              "expand: src must be ((w+1)>>1, (h+1)>>1) of dst");
    ENB_LAUNCH(ctx, launch_expand(add != 0, wrap != 0, planar_view(src), planar_view(dst), ctx->stream));
    return ENB_OK;
}

enb_status enb_blend(enb_ctx* ctx, const enb_image* mask, const enb_image* white, const enb_image* black,
                     int32_t white_value)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, planar_ok(mask) && planar_ok(white) && planar_ok(black), "blend: planar levels expected");
    ENB_CHECK(ctx, mask->channels == 1 && same_geometry(white, black) && mask->width == black->width &&
                       mask->height == black->height && (black->channels == 1 || black->channels == 3),
              "blend: size/channel mismatch");
    ENB_CHECK(ctx, white_value > 0, "blend: white value must be positive");
    ENB_LAUNCH(ctx, launch_blend(planar_view(mask), planar_view(white), planar_view(black), white_value, ctx->stream));
    return ENB_OK;
}

enb_status enb_mask_multiply_accumulate(enb_ctx* ctx, const enb_image* lp, const enb_image* mask, int32_t divisor,
                                        const enb_image* result, int accumulate)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, planar_ok(lp) && planar_ok(mask) && planar_ok(result), "mask_multiply: planar levels expected");
    ENB_CHECK(ctx, mask->channels == 1 && same_geometry(lp, result) && mask->width == lp->width &&
                       mask->height == lp->height && (lp->channels == 1 || lp->channels == 3),
              "mask_multiply: size/channel mismatch");
    ENB_CHECK(ctx, divisor > 0, "mask_multiply: divisor must be positive");
    ENB_LAUNCH(ctx, launch_mask_mul_acc(planar_view(lp), planar_view(mask), divisor, planar_view(result),
                                        accumulate != 0, ctx->stream));
    return ENB_OK;
}

enb_status enb_from_pyramid(enb_ctx* ctx, const enb_image* src, const enb_image* alpha, const enb_image* dst,
                            int frac, int dither, uint64_t seed)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, planar_ok(src), "from_pyramid: planar source level expected");
    ENB_CHECK(ctx, pixels_ok(dst) && dst->width == src->width && dst->height == src->height &&
                       dst->channels == src->channels,
              "from_pyramid: dst must be an interleaved U8/U16/F32 image of the level size");
    ENB_CHECK(ctx, bytes_ok(alpha, src->width, src->height), "from_pyramid: alpha must be U8 of the level size");
    ENB_CHECK(ctx, (src->dtype == ENB_F32) == (dst->dtype == ENB_F32),
              "from_pyramid: F32 levels convert to F32 pixels, fixed point to U8/U16");
    if (src->dtype == ENB_F32) {
        const PixelView fv = pixel_view(dst);
        ENB_LAUNCH(ctx, launch_from_fixed(planar_view(src), byte_plane(alpha), dst->data, fv.pitch, dst->dtype,
                                          fv.stride, 0, 0, 0, ctx->stream));
        return ENB_OK;
    }
    ENB_CHECK(ctx, frac >= 2 && frac <= 24, "from_pyramid: frac_bits must be 2..24");
    ENB_CHECK(ctx, dither == ENB_DITHER_HASH || dither == ENB_DITHER_NEAREST, "from_pyramid: unknown dither mode");
    const PixelView dv = pixel_view(dst);
    ENB_LAUNCH(ctx, launch_from_fixed(planar_view(src), byte_plane(alpha), dst->data, dv.pitch, dst->dtype, dv.stride,
                                      frac, dither, seed, ctx->stream));
    return ENB_OK;
}

enb_status enb_gaussian_pyramid(enb_ctx* ctx, int wrap, const enb_image* src, const enb_image* alpha, int frac,
                                enb_pyramid* pyr)
{
    if (!ctx || !pyr) {
        return ENB_ERR_INVALID;
    }
    enb_image l0;
    enb_pyramid_level(pyr, 0, &l0);
    ENB_TRY(enb_to_pyramid(ctx, src, &l0, frac));
    if (alpha) {
        ENB_CHECK(ctx, bytes_ok(alpha, src->width, src->height), "gaussian_pyramid: alpha must be U8 of the image size");
        const BytePlane a = byte_plane(alpha);
        return gaussian_levels(ctx, wrap != 0, pyr, &a);
    }
    return gaussian_levels(ctx, wrap != 0, pyr, nullptr);
}

// Allocation-free variant of enb_gaussian_pyramid: the reduced alpha planes
// go to g_noalloc_scratch instead of a stream-ordered allocation.  Launches
// bypass the profiler (which creates CUDA events on demand).
enb_status enb_gaussian_pyramid_noalloc(enb_ctx* ctx, int wrap, const enb_image* src, const enb_image* alpha,
                                        int frac, enb_pyramid* p)
{
    if (!ctx || !p) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, src && src->width == p->w[0] && src->height == p->h[0], "noalloc: src size differs from level 0");
    ENB_CHECK(ctx, frac >= 0 && frac <= 24, "noalloc: frac_bits outside 0..24");
    const PlanarView l0 = level_view(p, 0);
    // Level 0 takes the conversions of enb_to_pyramid, with its checks: an
    // F32 pyramid the logarithmic mapping of an interleaved F32 image, a
    // fixed-point pyramid either fromRealPromote(v * 2^frac) of an F32 plane
    // (one channel) or v << frac of interleaved U8/U16 pixels.
    const bool f32_plane = p->dtype != ENB_F32 && src->dtype == ENB_F32;
    if (p->dtype == ENB_F32) {
        ENB_CHECK(ctx, pixels_ok(src) && src->dtype == ENB_F32 && src->channels == p->C,
                  "noalloc: an F32 pyramid takes an interleaved F32 image of its channel count");
    } else if (f32_plane) {
        ENB_CHECK(ctx, src->channels == 1 && p->C == 1 && floats_ok(src, src->width, src->height),
                  "noalloc: F32 sources of a fixed-point pyramid are single-channel planes");
    } else {
        ENB_CHECK(ctx, pixels_ok(src) && src->dtype != ENB_F32 && src->channels == p->C,
                  "noalloc: src must be interleaved U8/U16 of the pyramid's channels");
    }
    if (alpha) {
        ENB_CHECK(ctx, bytes_ok(alpha, src->width, src->height), "noalloc: alpha must be U8 of the image size");
    }
    // Layout of the alpha planes of levels 1..L-1 in the scratch array.
    int64_t off[kMaxLevels + 1] = {}, pitch[kMaxLevels + 1] = {};
    int64_t total = 0;
    for (int l = 1; l < p->levels; ++l) {
        pitch[l] = round_up(p->w[l], 128);
        off[l] = total;
        total += round_up(pitch[l] * p->h[l], 256);
    }
    if (alpha && total > (int64_t)ENB_NOALLOC_SCRATCH_BYTES) {
        return fail(ctx, ENB_ERR_INVALID,
                    "noalloc: the reduced alpha planes need " + std::to_string(total) + " bytes, more than the " +
                        std::to_string((unsigned)ENB_NOALLOC_SCRATCH_BYTES) + "-byte scratch (about 48 Mpx at level 0)");
    }
    for (int l = 1; l < p->levels; ++l) {
        ENB_CHECK(ctx, p->w[l - 1] > 1 && p->h[l - 1] > 1, "reduce: src image too small in reduce");
    }
    uint8_t* scratch = nullptr;
    if (alpha) {
        void* s = nullptr;
        ENB_TRY(noalloc_scratch(ctx, &s));
        scratch = (uint8_t*)s;
    }
    cudaError_t e = f32_plane ? launch_float_to_fixed(float_plane(src), l0, frac, ctx->stream)
                              : launch_to_fixed(pixel_view(src), l0, frac, ctx->stream);
    ctx->launches++;
    if (e != cudaSuccess) {
        return cuda_fail(ctx, e, "noalloc: conversion to fixed point");
    }
    for (int l = 1; l < p->levels; ++l) {
        if (alpha) {
            const BytePlane sa = l == 1 ? byte_plane(alpha)
                                        : BytePlane{scratch + off[l - 1], pitch[l - 1], p->w[l - 1], p->h[l - 1]};
            const BytePlane da{scratch + off[l], pitch[l], p->w[l], p->h[l]};
            e = launch_reduce(wrap != 0, level_view(p, l - 1), &sa, level_view(p, l), &da, ctx->stream);
        } else {
            e = launch_reduce(wrap != 0, level_view(p, l - 1), nullptr, level_view(p, l), nullptr, ctx->stream);
        }
        ctx->launches++;
        if (e != cudaSuccess) {
            return cuda_fail(ctx, e, "noalloc: reduce");
        }
    }
    return ENB_OK;
}

enb_status enb_laplacian_pyramid(enb_ctx* ctx, int wrap, const enb_image* src, const enb_image* alpha, int frac,
                                 enb_pyramid* pyr)
{
    ENB_TRY(enb_gaussian_pyramid(ctx, wrap, src, alpha, frac, pyr));
    return laplacian_levels(ctx, wrap != 0, pyr);
}

enb_status enb_collapse_pyramid(enb_ctx* ctx, int wrap, enb_pyramid* pyr)
{
    if (!ctx || !pyr) {
        return ENB_ERR_INVALID;
    }
    return collapse_levels(ctx, wrap != 0, pyr);
}

enb_status enb_blend_pyramids(enb_ctx* ctx, const enb_pyramid* mask_gp, const enb_pyramid* white_lp,
                              enb_pyramid* black_lp, int32_t white_value)
{
    if (!ctx || !mask_gp || !white_lp || !black_lp) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, mask_gp->levels == black_lp->levels && white_lp->levels == black_lp->levels,
              "blend_pyramids: level count mismatch");
    for (int l = 0; l < black_lp->levels; ++l) {
        ENB_CHECK(ctx, mask_gp->w[l] == black_lp->w[l] && mask_gp->h[l] == black_lp->h[l], "blend_pyramids: size mismatch");
        ENB_LAUNCH(ctx, launch_blend(level_view(mask_gp, l), level_view(white_lp, l), level_view(black_lp, l),
                                     white_value, ctx->stream));
    }
    return ENB_OK;
}

enb_status enb_enfuse_mask(enb_ctx* ctx, const enb_enfuse_params* prm, const enb_image* src, const enb_image* alpha,
                           const enb_image* mask_out)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    ENB_CHECK(ctx, pixels_ok(src), "enfuse_mask: src must be interleaved U8/U16/F32 (1 or 3 channels)");
    ENB_TRY(check_params(ctx, prm, src->width, src->height));
    ENB_CHECK(ctx, floats_ok(mask_out, src->width, src->height), "enfuse_mask: mask_out must be F32 of the image size");
    if (alpha && alpha->data) {
        ENB_CHECK(ctx, bytes_ok(alpha, src->width, src->height), "enfuse_mask: alpha must be U8 of the image size");
    }
    return enfuse_mask_impl(ctx, prm, src, alpha, float_plane(mask_out));
}

enb_status enb_enfuse(enb_ctx* ctx, const enb_enfuse_params* prm, int K, const enb_image* images,
                      const enb_image* alphas, const enb_image* masks_in, const enb_image* out,
                      const enb_image* out_alpha, const enb_fuse_options* opt)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    enb_fuse_options o;
    enb_default_fuse_options(&o);
    if (opt) {
        o = *opt;
    }
    ENB_CHECK(ctx, K >= 1 && images, "enfuse: need at least one image");
    for (int k = 0; k < K; ++k) {
        ENB_CHECK(ctx, pixels_ok(&images[k]), "enfuse: images must be interleaved U8/U16/F32 with 1 or 3 channels");
        ENB_CHECK(ctx, same_geometry(&images[k], &images[0]), "enfuse: images differ in size, channels or type");
    }
    ENB_CHECK(ctx, out && pixels_ok(out) && same_geometry(out, &images[0]), "enfuse: out must match the inputs");
    ENB_CHECK(ctx, o.dither == ENB_DITHER_HASH || o.dither == ENB_DITHER_NEAREST, "enfuse: unknown dither mode");
    if (!masks_in) {
        ENB_TRY(check_params(ctx, prm, images[0].width, images[0].height));
    }
    const int w = images[0].width, h = images[0].height, C = images[0].channels;
    if (!o.host_buffers) {
        return enfuse_device(ctx, prm, K, images, alphas, masks_in, out, out_alpha, o, (int32_t*)o.level0_out);
    }
    // Host buffers: stage in, run, stage out (copies on the context stream).
    std::vector<Staged> si(K), sa(alphas ? K : 0), sm(masks_in ? K : 0);
    std::vector<enb_image> di(K), da(alphas ? K : 0), dm(masks_in ? K : 0);
    for (int k = 0; k < K; ++k) {
        ENB_TRY(stage_in(ctx, &images[k], si[k], true));
        di[k] = si[k].dev;
        if (alphas) {
            ENB_TRY(stage_in(ctx, &alphas[k], sa[k], alphas[k].data != nullptr));
            da[k] = sa[k].dev;
            if (!alphas[k].data) {
                da[k].data = nullptr;
            }
        }
        if (masks_in) {
            ENB_TRY(stage_in(ctx, &masks_in[k], sm[k], true));
            dm[k] = sm[k].dev;
        }
    }
    Staged so, soa;
    ENB_TRY(stage_in(ctx, out, so, false));
    const bool want_alpha = out_alpha && out_alpha->data;
    if (want_alpha) {
        ENB_TRY(stage_in(ctx, out_alpha, soa, false));
    }
    DevBuf l0;
    if (o.level0_out) {
        ENB_CUDA(ctx, l0.alloc((size_t)w * h * C * 4, ctx->stream));
    }
    ENB_TRY(enfuse_device(ctx, prm, K, di.data(), alphas ? da.data() : nullptr, masks_in ? dm.data() : nullptr,
                          &so.dev, want_alpha ? &soa.dev : nullptr, o, (int32_t*)l0.p));
    ENB_TRY(stage_out(ctx, out, so));
    if (want_alpha) {
        ENB_TRY(stage_out(ctx, out_alpha, soa));
    }
    if (o.level0_out) {
        ENB_CUDA(ctx, cudaMemcpyAsync(o.level0_out, l0.p, (size_t)w * h * C * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return ENB_OK;
}

enb_status enb_enblend(enb_ctx* ctx, const enb_image* white, const enb_image* white_alpha, const enb_image* black,
                       const enb_image* black_alpha, const enb_image* mask, const enb_image* out,
                       const enb_image* out_alpha, const enb_fuse_options* opt)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    enb_fuse_options o;
    enb_default_fuse_options(&o);
    if (opt) {
        o = *opt;
    }
    ENB_CHECK(ctx, pixels_ok(white) && pixels_ok(black) && same_geometry(white, black),
              "enblend: white/black must be interleaved U8/U16/F32 images of one geometry");
    if (black->dtype == ENB_F32) {
        o.plain = 1;  // the fused level passes are fixed point
    }
    ENB_CHECK(ctx, out && pixels_ok(out) && same_geometry(out, black), "enblend: out must match the inputs");
    ENB_CHECK(ctx, mask && bytes_ok(mask, black->width, black->height), "enblend: mask must be U8 of the image size");
    ENB_CHECK(ctx, black->width > 1 && black->height > 1, "enblend: image too small");
    ENB_CHECK(ctx, o.dither == ENB_DITHER_HASH || o.dither == ENB_DITHER_NEAREST, "enblend: unknown dither mode");
    const int w = black->width, h = black->height, C = black->channels;
    auto run = [&](const enb_image* wi, const enb_image* wai, const enb_image* bi, const enb_image* bai,
                   const enb_image* mi, const enb_image* oi, const enb_image* oai, int32_t* l0) {
        return o.plain ? enblend_plain(ctx, wi, wai, bi, bai, mi, oi, oai, o, l0)
                       : enblend_fused(ctx, wi, wai, bi, bai, mi, oi, oai, o, l0);
    };
    if (!o.host_buffers) {
        return run(white, white_alpha, black, black_alpha, mask, out, out_alpha, (int32_t*)o.level0_out);
    }
    if (!o.plain && alpha_source(white, white_alpha).mode == alpha_source(black, black_alpha).mode) {
        return enblend_host_banded(ctx, white, white_alpha, black, black_alpha, mask, out, out_alpha, o);
    }
    // Host buffers: the result is formed in place in the device copy of the
    // black image and copied back from there.
    Staged sw, sb, swa, sba, sm, soa;
    ENB_TRY(stage_in(ctx, white, sw, true));
    ENB_TRY(stage_in(ctx, black, sb, true));
    ENB_TRY(stage_in(ctx, mask, sm, true));
    const bool has_wa = white_alpha && white_alpha->data, has_ba = black_alpha && black_alpha->data;
    if (has_wa) {
        ENB_TRY(stage_in(ctx, white_alpha, swa, true));
    }
    if (has_ba) {
        ENB_TRY(stage_in(ctx, black_alpha, sba, true));
    }
    const bool want_alpha = out_alpha && out_alpha->data;
    if (want_alpha) {
        ENB_TRY(stage_in(ctx, out_alpha, soa, false));
    }
    DevBuf l0;
    if (o.level0_out) {
        ENB_CUDA(ctx, l0.alloc((size_t)w * h * C * 4, ctx->stream));
    }
    ENB_TRY(run(&sw.dev, has_wa ? &swa.dev : nullptr, &sb.dev, has_ba ? &sba.dev : nullptr, &sm.dev, &sb.dev,
                want_alpha ? &soa.dev : nullptr, (int32_t*)l0.p));
    ENB_TRY(stage_out(ctx, out, sb));
    if (want_alpha) {
        ENB_TRY(stage_out(ctx, out_alpha, soa));
    }
    if (o.level0_out) {
        ENB_CUDA(ctx, cudaMemcpyAsync(o.level0_out, l0.p, (size_t)w * h * C * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return ENB_OK;
}

// ---- batched stacks ---------------------------------------------------------

static enb_status float_weight_params(enb_ctx* ctx, const enb_enfuse_params* prm, FloatWeightParams& wp)
{
    ENB_TRY(build_tables(ctx, prm, 1u));
    wp = FloatWeightParams{};
    wp.use_exposure = prm->w_exposure > 0.0;
    wp.use_contrast = prm->w_contrast > 0.0;
    wp.use_saturation = prm->w_saturation > 0.0;
    wp.use_entropy = prm->w_entropy > 0.0;
    wp.contrast_window = prm->contrast_window;
    wp.entropy_window = prm->entropy_window;
    wp.gray_projector = prm->gray_projector;
    wp.exp_function = prm->exp_function;
    if (prm->gray_projector == ENB_GRAY_MIXER) {
        const double sm = prm->mixer[0] + prm->mixer[1] + prm->mixer[2];
        for (int i = 0; i < 3; ++i) {
            wp.mixer[i] = prm->mixer[i] / sm;
        }
    }
    wp.w_exposure = (float)prm->w_exposure;
    wp.w_contrast = (float)prm->w_contrast;
    wp.w_saturation = (float)prm->w_saturation;
    wp.w_entropy = (float)prm->w_entropy;
    const double range = float_range_of(prm);
    wp.range = (float)range;
    wp.opt_hi = (float)prm->exp_optimum;
    wp.opt_lo = (float)(prm->exp_optimum - (double)wp.opt_hi);
    const double inv_width = 1.0 / exposure_effective_width(prm->exp_function, prm->exp_width);
    wp.inv_hi = (float)inv_width;
    wp.inv_lo = (float)(inv_width - (double)wp.inv_hi);
    return float_cutoffs(ctx, prm, range, wp);
}

// What the batched fuse's work depends on: the stacks' sizes, exposure
// counts and channels, the parameters and the options (not the buffers).
static std::string batch_geometry_key(const enb_enfuse_params* prm, int n, const enb_stack* stacks,
                                      const enb_fuse_options& o)
{
    std::string key;
    const auto put = [&key](const void* p, size_t b) { key.append((const char*)p, b); };
    put(&n, sizeof n);
    put(prm, sizeof *prm);
    put(&o.levels, sizeof o.levels);
    put(&o.wrap, sizeof o.wrap);
    put(&o.hard_mask, sizeof o.hard_mask);
    for (int i = 0; i < n; ++i) {
        const enb_image& im = stacks[i].images[0];
        const int32_t g[4] = {stacks[i].K, im.width, im.height, im.channels};
        put(g, sizeof g);
        const int32_t a = stacks[i].alphas ? 1 : 0;
        put(&a, sizeof a);
    }
    return key;
}

enb_status enb_fuse_stacks(enb_ctx* ctx, const enb_enfuse_params* prm, int n, const enb_stack* stacks,
                           const enb_fuse_options* opt)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    enb_fuse_options o;
    enb_default_fuse_options(&o);
    if (opt) {
        o = *opt;
    }
    ENB_CHECK(ctx, n >= 1 && stacks, "fuse_stacks: need at least one stack");
    int C = -1;
    for (int i = 0; i < n; ++i) {
        const enb_stack& st = stacks[i];
        ENB_CHECK(ctx, st.K >= 1 && st.K <= ENB_BATCH_MAX_K && st.images && st.out,
                  "fuse_stacks: each stack needs 1..16 images and an output");
        for (int k = 0; k < st.K; ++k) {
            ENB_CHECK(ctx, pixels_ok(&st.images[k]) && st.images[k].dtype == ENB_F32,
                      "fuse_stacks: images must be interleaved F32 with 1 or 3 channels");
            ENB_CHECK(ctx, same_geometry(&st.images[k], &st.images[0]), "fuse_stacks: a stack's images differ");
            if (st.alphas && st.alphas[k].data) {
                ENB_CHECK(ctx, bytes_ok(&st.alphas[k], st.images[0].width, st.images[0].height),
                          "fuse_stacks: alpha planes must be U8 of the image size");
            }
        }
        ENB_CHECK(ctx, pixels_ok(st.out) && same_geometry(st.out, &st.images[0]),
                  "fuse_stacks: out must match the stack's images");
        if (st.out_alpha && st.out_alpha->data) {
            ENB_CHECK(ctx, bytes_ok(st.out_alpha, st.images[0].width, st.images[0].height),
                      "fuse_stacks: out_alpha must be U8 of the image size");
        }
        ENB_CHECK(ctx, C < 0 || st.images[0].channels == C, "fuse_stacks: all stacks need the same channel count");
        C = st.images[0].channels;
        ENB_TRY(check_params(ctx, prm, st.images[0].width, st.images[0].height));
    }
    if (o.plain) {
        // the plain per-stack path: enb_enfuse stack by stack
        for (int i = 0; i < n; ++i) {
            enb_fuse_options so = o;
            so.plain = 0;
            so.level0_out = nullptr;
            ENB_TRY(enb_enfuse(ctx, prm, stacks[i].K, stacks[i].images, stacks[i].alphas, nullptr, stacks[i].out,
                               stacks[i].out_alpha, &so));
        }
        return ENB_OK;
    }
    FloatWeightParams wp;
    ENB_TRY(float_weight_params(ctx, prm, wp));
    int32_t cp = o.coarse_pixels;
    if (cp == 0) {
        const auto it = ctx->tuned.find(batch_geometry_key(prm, n, stacks, o));
        cp = it != ctx->tuned.end() ? it->second : 4096;
    }
    const int64_t coarse = cp < 0 ? 0 : cp;
    // cache key: every descriptor, the parameters and the options
    std::string key;
    auto put = [&key](const void* p, size_t b) { key.append((const char*)p, b); };
    put(&n, sizeof n);
    put(prm, sizeof *prm);
    put(&coarse, sizeof coarse);
    put(&o.levels, sizeof o.levels);
    put(&o.wrap, sizeof o.wrap);
    put(&o.hard_mask, sizeof o.hard_mask);
    put(&o.host_buffers, sizeof o.host_buffers);
    put(&ctx->tables.plogp_fx, sizeof(void*));
    for (int i = 0; i < n; ++i) {
        const enb_stack& st = stacks[i];
        put(&st.K, sizeof st.K);
        for (int k = 0; k < st.K; ++k) {
            put(&st.images[k], sizeof(enb_image));
            const void* ap = st.alphas ? st.alphas[k].data : nullptr;
            put(&ap, sizeof ap);
            if (ap) {
                put(&st.alphas[k].pitch, sizeof(int64_t));
            }
        }
        put(st.out, sizeof(enb_image));
        const void* oa = st.out_alpha ? st.out_alpha->data : nullptr;
        put(&oa, sizeof oa);
        if (oa) {
            put(&st.out_alpha->pitch, sizeof(int64_t));
        }
    }
    if (!ctx->batch) {
        ctx->batch.reset(new enb_ctx::BatchCache());
        ENB_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->batch->gs, cudaStreamNonBlocking));
        ENB_CUDA(ctx, cudaEventCreateWithFlags(&ctx->batch->ev[0], cudaEventDisableTiming));
        ENB_CUDA(ctx, cudaEventCreateWithFlags(&ctx->batch->ev[1], cudaEventDisableTiming));
    }
    enb_ctx::BatchCache& bc = *ctx->batch;
    // host buffers: device copies of every image (kept with the plan)
    std::vector<size_t> in_off, out_off, oa_off;
    size_t stage_bytes = 0;
    auto img_bytes = [](const enb_image& im) {
        const int stride = im.pix_stride > 0 ? im.pix_stride : im.channels;
        return (size_t)im.width * stride * 4 * (size_t)im.height;
    };
    auto up256 = [](size_t v) { return (v + 255) & ~(size_t)255; };
    if (o.host_buffers) {
        for (int i = 0; i < n; ++i) {
            for (int k = 0; k < stacks[i].K; ++k) {
                in_off.push_back(stage_bytes);
                stage_bytes += up256(img_bytes(stacks[i].images[k]));
                in_off.push_back(stage_bytes);  // alpha plane slot
                if (stacks[i].alphas && stacks[i].alphas[k].data) {
                    stage_bytes += up256((size_t)stacks[i].images[k].width * stacks[i].images[k].height);
                }
            }
            out_off.push_back(stage_bytes);
            stage_bytes += up256(img_bytes(*stacks[i].out));
            oa_off.push_back(stage_bytes);
            if (stacks[i].out_alpha && stacks[i].out_alpha->data) {
                stage_bytes += up256((size_t)stacks[i].out->width * stacks[i].out->height);
            }
        }
    }
    if (bc.key != key || !bc.plan) {
        if (bc.exec) {
            cudaGraphExecDestroy(bc.exec);
            bc.exec = nullptr;
        }
        ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        ENB_CUDA(ctx, cudaStreamSynchronize(bc.gs));
        batch_plan_destroy(bc.plan);
        bc.plan = nullptr;
        cudaFree(bc.stage);
        bc.stage = nullptr;
        bc.key.clear();
        if (stage_bytes) {
            ENB_CUDA(ctx, cudaMalloc(&bc.stage, stage_bytes));
        }
        std::vector<BatchStackHost> hs((size_t)n);
        size_t j = 0;
        for (int i = 0; i < n; ++i) {
            const enb_stack& st = stacks[i];
            BatchStackHost& h = hs[(size_t)i];
            memset(&h, 0, sizeof h);
            h.K = st.K;
            h.w = st.images[0].width;
            h.h = st.images[0].height;
            h.C = C;
            for (int k = 0; k < st.K; ++k) {
                const enb_image& im = st.images[k];
                const int stride = im.pix_stride > 0 ? im.pix_stride : im.channels;
                h.istride[k] = stride;
                const bool has_a = st.alphas && st.alphas[k].data;
                ENB_CHECK(ctx, has_a || stride != 4, "fuse_stacks: RGBA images need alpha planes");
                if (o.host_buffers) {
                    h.img[k] = (const float*)((char*)bc.stage + in_off[j]);
                    h.ipitch[k] = (int64_t)im.width * stride;
                    h.alpha[k] = has_a ? (const uint8_t*)((char*)bc.stage + in_off[j + 1]) : nullptr;
                    h.apitch[k] = im.width;
                    j += 2;
                } else {
                    h.img[k] = (const float*)im.data;
                    h.ipitch[k] = im.pitch / 4;
                    h.alpha[k] = has_a ? (const uint8_t*)st.alphas[k].data : nullptr;
                    h.apitch[k] = has_a ? st.alphas[k].pitch : 0;
                }
            }
            const int ostride = st.out->pix_stride > 0 ? st.out->pix_stride : st.out->channels;
            h.ostride = ostride;
            const bool has_oa = st.out_alpha && st.out_alpha->data;
            if (o.host_buffers) {
                h.out = (float*)((char*)bc.stage + out_off[(size_t)i]);
                h.opitch = (int64_t)st.out->width * ostride;
                h.oalpha = has_oa ? (uint8_t*)((char*)bc.stage + oa_off[(size_t)i]) : nullptr;
                h.oapitch = st.out->width;
            } else {
                h.out = (float*)st.out->data;
                h.opitch = st.out->pitch / 4;
                h.oalpha = has_oa ? (uint8_t*)st.out_alpha->data : nullptr;
                h.oapitch = has_oa ? st.out_alpha->pitch : 0;
            }
        }
        unsigned int* err = device_error_word(ctx);
        if (!err) {
            return fail(ctx, ENB_ERR_NOMEM, "fuse_stacks: the device error word");
        }
        cudaError_t e = batch_plan_create(hs, wp, ctx->tables, o.levels, o.wrap != 0, o.hard_mask != 0, coarse, err,
                                          ctx->stream, &bc.plan);
        if (e != cudaSuccess) {
            return fail(ctx, e == cudaErrorMemoryAllocation ? ENB_ERR_NOMEM : ENB_ERR_CUDA,
                        std::string("fuse_stacks: ") + cudaGetErrorString(e));
        }
        bc.key = key;
    }
    if (o.host_buffers) {
        size_t j = 0;
        for (int i = 0; i < n; ++i) {
            for (int k = 0; k < stacks[i].K; ++k) {
                const enb_image& im = stacks[i].images[k];
                const int stride = im.pix_stride > 0 ? im.pix_stride : im.channels;
                const size_t row = (size_t)im.width * stride * 4;
                ENB_CUDA(ctx, cudaMemcpy2DAsync((char*)bc.stage + in_off[j], row, im.data, im.pitch, row, im.height,
                                                cudaMemcpyHostToDevice, ctx->stream));
                if (stacks[i].alphas && stacks[i].alphas[k].data) {
                    ENB_CUDA(ctx, cudaMemcpy2DAsync((char*)bc.stage + in_off[j + 1], im.width, stacks[i].alphas[k].data,
                                                    stacks[i].alphas[k].pitch, im.width, im.height,
                                                    cudaMemcpyHostToDevice, ctx->stream));
                }
                j += 2;
            }
        }
    }
    const int nsteps = batch_plan_steps(bc.plan);
    if (o.graph && !ctx->prof) {
        if (!bc.exec) {
            cudaGraph_t g = nullptr;
            ENB_CUDA(ctx, cudaStreamBeginCapture(bc.gs, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            for (int i = 0; i < nsteps && e == cudaSuccess; ++i) {
                e = batch_plan_launch(bc.plan, i, bc.gs);
            }
            const cudaError_t e2 = cudaStreamEndCapture(bc.gs, &g);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (g) {
                    cudaGraphDestroy(g);
                }
                return cuda_fail(ctx, e != cudaSuccess ? e : e2, "fuse_stacks: graph capture");
            }
            e = cudaGraphInstantiate(&bc.exec, g, 0);
            cudaGraphDestroy(g);
            ENB_CUDA(ctx, e);
        }
        ENB_CUDA(ctx, cudaEventRecord(bc.ev[0], ctx->stream));
        ENB_CUDA(ctx, cudaStreamWaitEvent(bc.gs, bc.ev[0], 0));
        ENB_CUDA(ctx, cudaGraphLaunch(bc.exec, bc.gs));
        ENB_CUDA(ctx, cudaEventRecord(bc.ev[1], bc.gs));
        ENB_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, bc.ev[1], 0));
        ctx->launches += (uint64_t)nsteps;
    } else {
        for (int i = 0; i < nsteps; ++i) {
            ENB_LAUNCH(ctx, batch_plan_launch(bc.plan, i, ctx->stream));
        }
    }
    if (o.host_buffers) {
        for (int i = 0; i < n; ++i) {
            const enb_image& oi = *stacks[i].out;
            const int stride = oi.pix_stride > 0 ? oi.pix_stride : oi.channels;
            const size_t row = (size_t)oi.width * stride * 4;
            ENB_CUDA(ctx, cudaMemcpy2DAsync(oi.data, oi.pitch, (char*)bc.stage + out_off[(size_t)i], row, row,
                                            oi.height, cudaMemcpyDeviceToHost, ctx->stream));
            if (stacks[i].out_alpha && stacks[i].out_alpha->data) {
                ENB_CUDA(ctx, cudaMemcpy2DAsync(stacks[i].out_alpha->data, stacks[i].out_alpha->pitch,
                                                (char*)bc.stage + oa_off[(size_t)i], oi.width, oi.width, oi.height,
                                                cudaMemcpyDeviceToHost, ctx->stream));
            }
        }
        ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return ENB_OK;
}

// ---- adjoint ----------------------------------------------------------------

enb_status enb_fuse_stacks_tune(enb_ctx* ctx, const enb_enfuse_params* prm, int n, const enb_stack* stacks,
                                const enb_fuse_options* opt, const int32_t* candidates, int n_candidates, int reps,
                                float* times_ms, int32_t* best)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    static const int32_t kDefault[] = {-1, 1024, 4096, 16384, 65536};
    if (!candidates) {
        candidates = kDefault;
        n_candidates = (int)(sizeof kDefault / sizeof kDefault[0]);
    }
    ENB_CHECK(ctx, n_candidates >= 1 && reps >= 1, "fuse_stacks_tune: need candidates and reps >= 1");
    enb_fuse_options o;
    enb_default_fuse_options(&o);
    if (opt) {
        o = *opt;
    }
    ENB_CHECK(ctx, !o.plain && !o.host_buffers, "fuse_stacks_tune: tunes the batched device path");
    for (int c = 0; c < n_candidates; ++c) {
        ENB_CHECK(ctx, candidates[c] != 0, "fuse_stacks_tune: a candidate of 0 pixels means 'tuned'");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ENB_CUDA(ctx, cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return cuda_fail(ctx, cudaGetLastError(), "cudaEventCreate");
    }
    enb_status st = ENB_OK;
    float best_ms = 0.0f;
    int32_t best_cp = candidates[0];
    for (int c = 0; c < n_candidates && st == ENB_OK; ++c) {
        enb_fuse_options co = o;
        co.coarse_pixels = candidates[c];
        st = enb_fuse_stacks(ctx, prm, n, stacks, &co);  // builds the plan and graph
        cudaEventRecord(e0, ctx->stream);
        for (int r = 0; st == ENB_OK && r < reps; ++r) {
            st = enb_fuse_stacks(ctx, prm, n, stacks, &co);
        }
        if (st != ENB_OK) {
            break;
        }
        cudaEventRecord(e1, ctx->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = cuda_fail(ctx, cudaGetLastError(), "cudaEventSynchronize");
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)reps;
        if (times_ms) {
            times_ms[c] = ms;
        }
        if (c == 0 || ms < best_ms) {
            best_ms = ms;
            best_cp = candidates[c];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != ENB_OK) {
        return st;
    }
    ctx->tuned[batch_geometry_key(prm, n, stacks, o)] = best_cp;
    if (best) {
        *best = best_cp;
    }
    return check_device_error(ctx);
}

enb_status enb_fuse_grad(enb_ctx* ctx, const enb_enfuse_params* prm, int K, const enb_image* images,
                         const enb_image* logits, const enb_image* target, const enb_image* out,
                         const enb_image* grad_logits, enb_fuse_grad_result* res, const enb_fuse_options* opt)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    enb_fuse_options o;
    enb_default_fuse_options(&o);
    if (opt) {
        o = *opt;
    }
    ENB_CHECK(ctx, K >= 1 && images && target && res, "fuse_grad: images, target and result required");
    for (int k = 0; k < K; ++k) {
        ENB_CHECK(ctx, pixels_ok(&images[k]) && images[k].dtype == ENB_F32 && images[k].channels == 3,
                  "fuse_grad: images must be interleaved F32 RGB");
        ENB_CHECK(ctx, same_geometry(&images[k], &images[0]), "fuse_grad: images differ in size");
    }
    const int w = images[0].width, h = images[0].height;
    ENB_CHECK(ctx, pixels_ok(target) && target->dtype == ENB_F32 && target->channels == 3 && target->width == w &&
                       target->height == h,
              "fuse_grad: target must be an F32 RGB image of the inputs' size");
    if (out) {
        ENB_CHECK(ctx, pixels_ok(out) && out->dtype == ENB_F32 && out->width == w && out->height == h,
                  "fuse_grad: out must be an F32 image of the inputs' size");
    }
    for (int k = 0; k < K; ++k) {
        if (logits) {
            ENB_CHECK(ctx, floats_ok(&logits[k], w, h), "fuse_grad: logits must be F32 planes of the image size");
        }
        if (grad_logits) {
            ENB_CHECK(ctx, floats_ok(&grad_logits[k], w, h), "fuse_grad: grad_logits must be F32 planes");
        }
    }
    ENB_CHECK(ctx, !o.wrap && !o.hard_mask, "fuse_grad: wrap-around and hard masks are not differentiated");
    if (prm->w_entropy > 0.0) {
        return fail(ctx, ENB_ERR_UNSUPPORTED, "fuse_grad: the entropy weight is not differentiated");
    }
    {
        bool cut = false;
        double lo = 0.0, hi = 0.0;
        ENB_TRY(cutoff_limits(ctx, "exposure", prm->exp_cutoff_lower, prm->exp_cutoff_lower_pct, prm->exp_cutoff_upper,
                              prm->exp_cutoff_upper_pct, float_range_of(prm), false, cut, lo, hi));
        if (cut && prm->w_exposure > 0.0) {
            return fail(ctx, ENB_ERR_UNSUPPORTED, "fuse_grad: the exposure cutoff is not differentiated");
        }
    }
    ENB_TRY(check_params(ctx, prm, w, h));
    const int L = enb_num_levels(w, h, 1, o.levels);
    const int64_t fp = round_up(w, 32), plane = fp * h;
    DevBuf planes, a255;
    ENB_CUDA(ctx, planes.alloc((size_t)plane * 4 * K * 6 + 64, ctx->stream));
    float* wk = (float*)planes.p;
    float* ak = wk + plane * K;
    float* mk = ak + plane * K;
    float* gm = mk + plane * K;
    float* gw = gm + plane * K;
    float* ga = gw + plane * K;
    double* dsc = (double*)(ga + plane * K);
    const int64_t apitch = round_up(w, 128);
    ENB_CUDA(ctx, a255.alloc((size_t)(apitch * h), ctx->stream));
    ENB_CUDA(ctx, cudaMemsetAsync(a255.p, 255, (size_t)(apitch * h), ctx->stream));
    ENB_CUDA(ctx, cudaMemsetAsync(dsc, 0, 6 * sizeof(double), ctx->stream));
    const BytePlane alpha{(uint8_t*)a255.p, apitch, w, h};
    enb_image aimg{};
    aimg.data = a255.p;
    aimg.pitch = apitch;
    aimg.width = w;
    aimg.height = h;
    aimg.channels = 1;
    aimg.pix_stride = 1;
    aimg.dtype = ENB_U8;

    // forward: weights, logits, masks
    for (int k = 0; k < K; ++k) {
        ENB_TRY(enfuse_mask_impl(ctx, prm, &images[k], &aimg, FloatPlane{wk + plane * k, fp, w, h}));
        if (logits) {
            ENB_CUDA(ctx, cudaMemcpy2DAsync(ak + plane * k, fp * 4, logits[k].data, logits[k].pitch, (size_t)w * 4, h,
                                            cudaMemcpyDeviceToDevice, ctx->stream));
        }
    }
    ENB_LAUNCH(ctx, launch_adj_norm(K, wk, logits ? ak : nullptr, mk, fp, plane, w, h, ctx->stream));
    PyrHolder R(ctx), LP(ctx), M(ctx), GR(ctx), ACC(ctx);
    ENB_TRY(pyramid_alloc(ctx, L, w, h, 3, ENB_F32, &R.p));
    ENB_TRY(pyramid_alloc(ctx, L, w, h, 3, ENB_F32, &LP.p));
    ENB_TRY(pyramid_alloc(ctx, L, w, h, 1, ENB_F32, &M.p));
    auto build_lp = [&](int k) -> enb_status {
        const PixelView iv = pixel_view(&images[k]);
        ENB_LAUNCH(ctx, launch_adj_to_pyramid(FloatPixelView{(const float*)iv.p, iv.pitch, iv.w, iv.h, 3, iv.stride},
                                              level_view(LP.p, 0), ctx->stream));
        ENB_TRY(gaussian_levels(ctx, 0, LP.p, &alpha));
        ENB_TRY(laplacian_levels(ctx, 0, LP.p));
        return ENB_OK;
    };
    for (int k = 0; k < K; ++k) {
        ENB_TRY(build_lp(k));
        const PlanarView m0 = level_view(M.p, 0);
        ENB_CUDA(ctx, cudaMemcpy2DAsync(m0.p, m0.pitch * 4, mk + plane * k, fp * 4, (size_t)w * 4, h,
                                        cudaMemcpyDeviceToDevice, ctx->stream));
        ENB_TRY(gaussian_levels(ctx, 0, M.p, &alpha));
        for (int l = 0; l < L; ++l) {
            ENB_LAUNCH(ctx, launch_adj_merge(level_view(LP.p, l), level_view(M.p, l), level_view(R.p, l), k == 0,
                                             ctx->stream));
        }
    }
    ENB_TRY(collapse_levels(ctx, 0, R.p));
    ENB_TRY(pyramid_alloc(ctx, L, w, h, 3, ENB_F32, &GR.p));
    const PixelView tv = pixel_view(target);
    float* outp = nullptr;
    int64_t opitch = 0;
    int ostride = 3;
    if (out) {
        const PixelView ov = pixel_view(out);
        outp = (float*)out->data;
        opitch = ov.pitch;
        ostride = ov.stride;
        if (ov.stride == 4) {
            ENB_LAUNCH(ctx, launch_alpha_component(alpha, out->data, ov.pitch, ENB_F32, ctx->stream));
        }
    }
    ENB_LAUNCH(ctx, launch_adj_loss(level_view(R.p, 0), (const float*)target->data, tv.pitch, tv.stride, outp, opitch,
                                    ostride, level_view(GR.p, 0), dsc, ctx->stream));

    // backward: collapse, merge and mask pyramids per exposure
    for (int l = 0; l + 1 < L; ++l) {
        ENB_LAUNCH(ctx, launch_expand_T(level_view(GR.p, l), level_view(GR.p, l + 1), ctx->stream));
    }
    ENB_TRY(pyramid_alloc(ctx, L, w, h, 1, ENB_F32, &ACC.p));
    for (int k = 0; k < K; ++k) {
        ENB_TRY(build_lp(k));
        for (int l = L - 1; l >= 0; --l) {
            const PlanarView nxt = l + 1 < L ? level_view(ACC.p, l + 1) : PlanarView{};
            ENB_LAUNCH(ctx, launch_adj_mask_level(level_view(GR.p, l), level_view(LP.p, l), l + 1 < L ? &nxt : nullptr,
                                                  level_view(ACC.p, l), ctx->stream));
        }
        const PlanarView a0 = level_view(ACC.p, 0);
        ENB_CUDA(ctx, cudaMemcpy2DAsync(gm + plane * k, fp * 4, a0.p, a0.pitch * 4, (size_t)w * 4, h,
                                        cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ENB_LAUNCH(ctx, launch_adj_norm_bw(K, wk, logits ? ak : nullptr, gm, gw, ga, fp, plane, w, h, ctx->stream));
    FloatWeightParams wp;
    ENB_TRY(float_weight_params(ctx, prm, wp));
    const float inv_width = (float)(1.0 / exposure_effective_width(prm->exp_function, prm->exp_width));
    for (int k = 0; k < K; ++k) {
        const PixelView iv = pixel_view(&images[k]);
        ENB_LAUNCH(ctx, launch_adj_weights_bw(FloatPixelView{(const float*)iv.p, iv.pitch, iv.w, iv.h, 3, iv.stride},
                                              gw + plane * k, fp, wp, inv_width, (float)prm->exp_width,
                                              (float)prm->w_exposure, prm->contrast_window, dsc + 1, ctx->stream));
    }
    if (grad_logits) {
        for (int k = 0; k < K; ++k) {
            ENB_CUDA(ctx, cudaMemcpy2DAsync(grad_logits[k].data, grad_logits[k].pitch, ga + plane * k, fp * 4,
                                            (size_t)w * 4, h, cudaMemcpyDeviceToDevice, ctx->stream));
        }
    }
    double hs[6];
    ENB_CUDA(ctx, cudaMemcpyAsync(hs, dsc, sizeof hs, cudaMemcpyDeviceToHost, ctx->stream));
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    res->loss = hs[0] / (3.0 * (double)w * (double)h);
    res->d_exp_optimum = hs[1];
    res->d_exp_width = hs[2];
    res->d_w_exposure = hs[3];
    res->d_w_saturation = hs[4];
    res->d_w_contrast = hs[5];
    return ENB_OK;
}

// enblend's seam mask by the nearest-feature transform (src/nearest.h:427-553,
// src/mask.h:1101-1180 for --fine-mask --no-optimize).
enb_status enb_nft_mask(enb_ctx* ctx, const enb_image* white_alpha, const enb_image* black_alpha,
                        const enb_image* mask, const enb_fuse_options* opt)
{
    if (!ctx) {
        return ENB_ERR_INVALID;
    }
    enb_fuse_options o;
    enb_default_fuse_options(&o);
    if (opt) {
        o = *opt;
    }
    ENB_CHECK(ctx, white_alpha && black_alpha && mask, "nft_mask: white_alpha, black_alpha and mask required");
    const int w = white_alpha->width, h = white_alpha->height;
    ENB_CHECK(ctx, w >= 1 && h >= 1 && bytes_ok(white_alpha, w, h) && bytes_ok(black_alpha, w, h) && bytes_ok(mask, w, h),
              "nft_mask: white_alpha, black_alpha and mask must be U8 planes of one size");
    const int wrap = o.wrap != 0;
    Staged sw, sb, sm;
    const enb_image *wi = white_alpha, *bi = black_alpha, *mi = mask;
    if (o.host_buffers) {
        ENB_TRY(stage_in(ctx, white_alpha, sw, true));
        ENB_TRY(stage_in(ctx, black_alpha, sb, true));
        ENB_TRY(stage_in(ctx, mask, sm, false));
        wi = &sw.dev;
        bi = &sb.dev;
        mi = &sm.dev;
    }
    DevBuf scratch, tally;
    ENB_CUDA(ctx, scratch.alloc(nft_scratch_bytes(w, h, wrap), ctx->stream));
    ENB_CUDA(ctx, tally.alloc(2 * sizeof(unsigned int), ctx->stream));
    ENB_CUDA(ctx, cudaMemsetAsync(tally.p, 0, 2 * sizeof(unsigned int), ctx->stream));
    const BytePlane wp = byte_plane(wi), bp = byte_plane(bi), mp = byte_plane(mi);
    for (int stage = 0; stage < 3; ++stage) {
        ENB_LAUNCH(ctx, launch_nft_stage(stage, wp, bp, mp, wrap, scratch.p, (unsigned int*)tally.p, ctx->stream));
    }
    unsigned int t[2] = {0u, 0u};
    ENB_CUDA(ctx, cudaMemcpyAsync(t, tally.p, sizeof t, cudaMemcpyDeviceToHost, ctx->stream));
    if (o.host_buffers) {
        ENB_TRY(stage_out(ctx, mask, sm));
    }
    ENB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // quick_tally's overlap check (src/nearest.h:465-470, 531-545): fewer than
    // 4 (w + h) pixels covered by one image only, in both directions
    const uint64_t threshold = 4ull * ((uint64_t)w + (uint64_t)h);
    if (t[0] < threshold && t[1] < threshold) {
        return fail(ctx, ENB_ERR_INVALID, "nft_mask: excessive image overlap; too high risk of defective seam line");
    }
    return ENB_OK;
}

}  // extern "C"

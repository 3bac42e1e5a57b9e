/*
 * enbgpu.hpp -- header-only C++ adaptor over the C ABI (enbgpu.h) with the
 * shape of the reference's internal pyramid / blend / weight templates, so
 * that C++ code written against them can call the GB300 path:
 *
 *   gaussianPyramid   src/pyramid.h:1471 (numLevels, wraparound, src, alpha)
 *   laplacianPyramid  src/pyramid.h:1650 (exportName, numLevels, wraparound, src, alpha)
 *   collapsePyramid   src/pyramid.h:1759 (wraparound, pyramid)
 *   blend             src/blend.h:82-86  (maskGP, whiteLP, blackLP, maskPyramidWhiteValue)
 *   enfuseMask        src/enfuse.h:963   (src, alpha, result) with the weighting options
 *   copyToPyramidImage / copyFromPyramidImageIf  src/fixmath.h:2121-2147, 2259-2294
 *
 * The reference's templates take VIGRA iterator/accessor triples and return
 * `new`-ed std::vector<PyramidImageType*>*; here images are device buffers
 * (ImageRef) and pyramids are owning handles (Pyramid, freed on
 * destruction), and a failed call throws enbgpu::Error as the reference's
 * vigra_precondition throws.  The pixel type is the template parameter, as in
 * the reference: it selects the pyramid's fixed-point format
 * (EnblendNumericTraits, src/numerictraits.h:159-185).
 */
#ifndef ENBGPU_HPP
#define ENBGPU_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>

#include "enbgpu.h"

namespace enbgpu {

struct Error : std::runtime_error {
    enb_status status;
    Error(enb_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

class Context {
  public:
    explicit Context(int device = 0)
    {
        const enb_status s = enb_create(device, &ctx_);
        if (s != ENB_OK) {
            throw Error(s, "enb_create failed (no usable CUDA device)");
        }
    }
    ~Context() { enb_destroy(ctx_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    enb_ctx* get() const { return ctx_; }
    void check(enb_status s) const
    {
        if (s != ENB_OK) {
            throw Error(s, enb_last_error(ctx_));
        }
    }
    void synchronize() const { check(enb_synchronize(ctx_)); }

  private:
    enb_ctx* ctx_ = nullptr;
};

// Sample type traits: the C ABI dtype and the pyramid of that pixel type.
template <typename T> struct Sample;
template <> struct Sample<uint8_t> {
    static constexpr int dtype = ENB_U8, pyramid = ENB_I16, frac = 7, mask_pyramid = ENB_I16, mask_frac = 7;
};
template <> struct Sample<uint16_t> {
    static constexpr int dtype = ENB_U16, pyramid = ENB_I32, frac = 7, mask_pyramid = ENB_I32, mask_frac = 15;
};
template <> struct Sample<float> {
    static constexpr int dtype = ENB_F32, pyramid = ENB_F32, frac = 0, mask_pyramid = ENB_I32, mask_frac = 15;
};

// A device image: interleaved pixels (channels colour samples out of
// stride), or an 8-bit plane (alpha, seam mask), or a float weight plane.
struct ImageRef {
    enb_image d{};
    template <typename T>
    static ImageRef pixels(const T* data, int width, int height, int channels, int stride, int64_t pitch_bytes = 0)
    {
        ImageRef r;
        r.d.data = const_cast<T*>(data);
        r.d.width = width;
        r.d.height = height;
        r.d.channels = channels;
        r.d.pix_stride = stride;
        r.d.pitch = pitch_bytes ? pitch_bytes : (int64_t)width * stride * (int64_t)sizeof(T);
        r.d.dtype = Sample<T>::dtype;
        return r;
    }
    template <typename T>
    static ImageRef plane(const T* data, int width, int height, int64_t pitch_bytes = 0)
    {
        return pixels<T>(data, width, height, 1, 1, pitch_bytes);
    }
    const enb_image* get() const { return &d; }
};

// std::vector<PyramidImageType*> of the reference as an owning handle.
class Pyramid {
  public:
    Pyramid(const Context& ctx, int levels, int width, int height, int channels, int dtype) : ctx_(&ctx)
    {
        ctx.check(enb_pyramid_create(ctx.get(), levels, width, height, channels, dtype, &p_));
    }
    ~Pyramid()
    {
        if (p_) {
            enb_pyramid_free(ctx_->get(), p_);
        }
    }
    Pyramid(Pyramid&& o) noexcept : ctx_(o.ctx_), p_(std::exchange(o.p_, nullptr)) {}
    Pyramid& operator=(Pyramid&& o) noexcept
    {
        std::swap(p_, o.p_);
        ctx_ = o.ctx_;
        return *this;
    }
    Pyramid(const Pyramid&) = delete;
    Pyramid& operator=(const Pyramid&) = delete;
    int size() const { return enb_pyramid_levels(p_); }
    enb_image level(int l) const
    {
        enb_image e{};
        ctx_->check(enb_pyramid_level(p_, l, &e));
        return e;
    }
    enb_pyramid* get() const { return p_; }

  private:
    const Context* ctx_;
    enb_pyramid* p_ = nullptr;
};

// gaussianPyramid<ImagePixelType>(numLevels, wraparound, src, alpha)
// (src/pyramid.h:1471-1478); alpha nullptr: the alpha-free reduce.
template <typename PixelComponent>
Pyramid gaussianPyramid(const Context& ctx, unsigned numLevels, bool wraparound, const ImageRef& src,
                        const ImageRef* alpha = nullptr)
{
    const bool weights = src.d.dtype == ENB_F32 && src.d.pix_stride == 1 && !std::is_same<PixelComponent, float>::value;
    Pyramid p(ctx, (int)numLevels, src.d.width, src.d.height, src.d.channels,
              weights ? Sample<PixelComponent>::mask_pyramid : Sample<PixelComponent>::pyramid);
    ctx.check(enb_gaussian_pyramid(ctx.get(), wraparound, src.get(), alpha ? alpha->get() : nullptr,
                                   weights ? Sample<PixelComponent>::mask_frac : Sample<PixelComponent>::frac, p.get()));
    return p;
}

// laplacianPyramid<ImagePixelType>(exportName, numLevels, wraparound, src,
// alpha) (src/pyramid.h:1650-1657); exportName (the debug export) is unused.
template <typename PixelComponent>
Pyramid laplacianPyramid(const Context& ctx, const char* /*exportName*/, unsigned numLevels, bool wraparound,
                         const ImageRef& src, const ImageRef* alpha = nullptr)
{
    Pyramid p(ctx, (int)numLevels, src.d.width, src.d.height, src.d.channels, Sample<PixelComponent>::pyramid);
    ctx.check(enb_laplacian_pyramid(ctx.get(), wraparound, src.get(), alpha ? alpha->get() : nullptr,
                                    Sample<PixelComponent>::frac, p.get()));
    return p;
}

// collapsePyramid(wraparound, pyramid) (src/pyramid.h:1759-1760): level 0
// receives the result.
inline void collapsePyramid(const Context& ctx, bool wraparound, Pyramid& p)
{
    ctx.check(enb_collapse_pyramid(ctx.get(), wraparound, p.get()));
}

// blend(maskGP, whiteLP, blackLP, maskPyramidWhiteValue) (src/blend.h:82-86):
// blackLP := the per-level CartesianBlend of whiteLP into blackLP.
inline void blend(const Context& ctx, const Pyramid& maskGP, const Pyramid& whiteLP, Pyramid& blackLP,
                  int32_t maskPyramidWhiteValue)
{
    ctx.check(enb_blend_pyramids(ctx.get(), maskGP.get(), whiteLP.get(), blackLP.get(), maskPyramidWhiteValue));
}

// enfuseMask(src, alpha, result) (src/enfuse.h:963-965) with the weighting
// options the reference reads from its globals (src/enfuse.cc:117-160).
inline void enfuseMask(const Context& ctx, const enb_enfuse_params& options, const ImageRef& src,
                       const ImageRef* alpha, const ImageRef& result)
{
    ctx.check(enb_enfuse_mask(ctx.get(), &options, src.get(), alpha ? alpha->get() : nullptr, result.get()));
}

// copyToPyramidImage (src/fixmath.h:2121-2147) into level 0 of p.
template <typename PixelComponent>
void copyToPyramidImage(const Context& ctx, const ImageRef& src, Pyramid& p)
{
    const enb_image l0 = p.level(0);
    ctx.check(enb_to_pyramid(ctx.get(), src.get(), &l0, Sample<PixelComponent>::frac));
}

// copyFromPyramidImageIf (src/fixmath.h:2259-2294): level 0 of p into the
// pixels where alpha is set, with the dither rule.
template <typename PixelComponent>
void copyFromPyramidImageIf(const Context& ctx, const Pyramid& p, const ImageRef& alpha, const ImageRef& dst,
                            int dither = ENB_DITHER_HASH, uint64_t seed = 0x5eed)
{
    const enb_image l0 = p.level(0);
    ctx.check(enb_from_pyramid(ctx.get(), &l0, alpha.get(), dst.get(), Sample<PixelComponent>::frac, dither, seed));
}

// Default weighting options of enfuse (src/enfuse.cc:117-160).
inline enb_enfuse_params defaultEnfuseOptions()
{
    enb_enfuse_params p;
    enb_default_enfuse_params(&p);
    return p;
}

}  // namespace enbgpu

#endif /* ENBGPU_HPP */

// vigra_shim_io.hxx -- the rest of the VIGRA interface that the reference's
// src/enfuse.h, src/assemble.h and src/mga.h instantiate (test oracle only),
// restated from VIGRA's documented semantics:
//   * functor expressions (vigra::functor::Arg1/Arg2/Arg3, Param, ifThenElse
//     and the arithmetic / comparison operators): each node evaluates its
//     operands and combines them with the C++ operator; a binary node's
//     result is PromoteTraits<R1, R2>::Promote of its operands' results and
//     ifThenElse's that of its two branches;
//   * Threshold<S, D>(lower, upper, no, yes): s < lower or upper < s gives
//     `no`, else `yes`;
//   * FindMinMax, FindBoundingRectangle: the inspection functors;
//   * image import / export through an in-memory file table instead of
//     files: ImageImportInfo(name) describes a table entry registered with
//     memfile_put, importImage / importImageAlpha copy its samples through
//     the destination accessors, exportImage / exportImageAlpha store the
//     samples they read under the export name (memfile_get).
// It is not VIGRA: the convolution filters of enfuse's optional edge-scale
// contrast mode (laplacianOfGaussian, gaussianSharpening) are declared but
// fail when called.
#ifndef ENB_REFSHIM_VIGRA_SHIM_IO_HXX
#define ENB_REFSHIM_VIGRA_SHIM_IO_HXX

#include <map>
#include <memory>
#include <mutex>
#include <type_traits>

namespace vigra {

// ---- functor expressions -------------------------------------------------------------
namespace functor {

template <class E>
struct UnaryFunctor {
    E e;
    UnaryFunctor() : e() {}
    explicit UnaryFunctor(const E& x) : e(x) {}
    template <class... A>
    auto operator()(const A&... a) const -> decltype(e(a...))
    {
        return e(a...);
    }
};

struct ArgumentFunctor1 {
    template <class T1, class... R>
    const T1& operator()(const T1& v1, const R&...) const
    {
        return v1;
    }
};
struct ArgumentFunctor2 {
    template <class T1, class T2, class... R>
    const T2& operator()(const T1&, const T2& v2, const R&...) const
    {
        return v2;
    }
};
struct ArgumentFunctor3 {
    template <class T1, class T2, class T3>
    const T3& operator()(const T1&, const T2&, const T3& v3) const
    {
        return v3;
    }
};

template <class T>
struct ParameterFunctor {
    T v;
    template <class... A>
    T operator()(const A&...) const
    {
        return v;
    }
};

inline UnaryFunctor<ArgumentFunctor1> Arg1() { return UnaryFunctor<ArgumentFunctor1>(); }
inline UnaryFunctor<ArgumentFunctor2> Arg2() { return UnaryFunctor<ArgumentFunctor2>(); }
inline UnaryFunctor<ArgumentFunctor3> Arg3() { return UnaryFunctor<ArgumentFunctor3>(); }

template <class T>
inline UnaryFunctor<ParameterFunctor<T>> Param(const T& v)
{
    return UnaryFunctor<ParameterFunctor<T>>(ParameterFunctor<T>{v});
}

// Binary node: PromoteTraits of the operands' results.
#define ENB_SHIM_FUNCTOR_BINARY(NAME, OP)                                                                  \
    template <class E1, class E2>                                                                          \
    struct NAME {                                                                                          \
        E1 a;                                                                                              \
        E2 b;                                                                                              \
        template <class... A>                                                                              \
        typename PromoteTraits<typename std::decay<decltype(std::declval<const E1&>()(std::declval<const A&>()...))>::type, \
                               typename std::decay<decltype(std::declval<const E2&>()(std::declval<const A&>()...))>::type>::Promote \
        operator()(const A&... x) const                                                                    \
        {                                                                                                  \
            return a(x...) OP b(x...);                                                                     \
        }                                                                                                  \
    };                                                                                                     \
    template <class E1, class E2>                                                                          \
    inline UnaryFunctor<NAME<UnaryFunctor<E1>, UnaryFunctor<E2>>> operator OP(const UnaryFunctor<E1>& a,   \
                                                                              const UnaryFunctor<E2>& b)   \
    {                                                                                                      \
        return UnaryFunctor<NAME<UnaryFunctor<E1>, UnaryFunctor<E2>>>(                                     \
            NAME<UnaryFunctor<E1>, UnaryFunctor<E2>>{a, b});                                               \
    }
ENB_SHIM_FUNCTOR_BINARY(Functor_add, +)
ENB_SHIM_FUNCTOR_BINARY(Functor_subtract, -)
ENB_SHIM_FUNCTOR_BINARY(Functor_multiply, *)
ENB_SHIM_FUNCTOR_BINARY(Functor_divide, /)
#undef ENB_SHIM_FUNCTOR_BINARY

// Comparison node: bool.
#define ENB_SHIM_FUNCTOR_COMPARE(NAME, OP)                                                                 \
    template <class E1, class E2>                                                                          \
    struct NAME {                                                                                          \
        E1 a;                                                                                              \
        E2 b;                                                                                              \
        template <class... A>                                                                              \
        bool operator()(const A&... x) const                                                               \
        {                                                                                                  \
            return a(x...) OP b(x...);                                                                     \
        }                                                                                                  \
    };                                                                                                     \
    template <class E1, class E2>                                                                          \
    inline UnaryFunctor<NAME<UnaryFunctor<E1>, UnaryFunctor<E2>>> operator OP(const UnaryFunctor<E1>& a,   \
                                                                              const UnaryFunctor<E2>& b)   \
    {                                                                                                      \
        return UnaryFunctor<NAME<UnaryFunctor<E1>, UnaryFunctor<E2>>>(                                     \
            NAME<UnaryFunctor<E1>, UnaryFunctor<E2>>{a, b});                                               \
    }
ENB_SHIM_FUNCTOR_COMPARE(Functor_greater, >)
ENB_SHIM_FUNCTOR_COMPARE(Functor_less, <)
ENB_SHIM_FUNCTOR_COMPARE(Functor_greater_equal, >=)
ENB_SHIM_FUNCTOR_COMPARE(Functor_less_equal, <=)
ENB_SHIM_FUNCTOR_COMPARE(Functor_equals, ==)
ENB_SHIM_FUNCTOR_COMPARE(Functor_differs, !=)
#undef ENB_SHIM_FUNCTOR_COMPARE

// ifThenElse: the branch's value converted to PromoteTraits of both branches.
template <class C, class E1, class E2>
struct IfThenElseFunctor {
    C c;
    E1 a;
    E2 b;
    template <class... A>
    typename PromoteTraits<typename std::decay<decltype(std::declval<const E1&>()(std::declval<const A&>()...))>::type,
                           typename std::decay<decltype(std::declval<const E2&>()(std::declval<const A&>()...))>::type>::Promote
    operator()(const A&... x) const
    {
        typedef typename PromoteTraits<
            typename std::decay<decltype(std::declval<const E1&>()(std::declval<const A&>()...))>::type,
            typename std::decay<decltype(std::declval<const E2&>()(std::declval<const A&>()...))>::type>::Promote R;
        return c(x...) ? static_cast<R>(a(x...)) : static_cast<R>(b(x...));
    }
};

template <class C, class E1, class E2>
inline UnaryFunctor<IfThenElseFunctor<UnaryFunctor<C>, UnaryFunctor<E1>, UnaryFunctor<E2>>>
ifThenElse(const UnaryFunctor<C>& c, const UnaryFunctor<E1>& a, const UnaryFunctor<E2>& b)
{
    return UnaryFunctor<IfThenElseFunctor<UnaryFunctor<C>, UnaryFunctor<E1>, UnaryFunctor<E2>>>(
        IfThenElseFunctor<UnaryFunctor<C>, UnaryFunctor<E1>, UnaryFunctor<E2>>{c, a, b});
}

}  // namespace functor

// ---- point functors ---------------------------------------------------------------------
template <class SrcValueType, class DestValueType>
class Threshold {
  public:
    typedef SrcValueType argument_type;
    typedef DestValueType result_type;
    Threshold(argument_type lower, argument_type higher, result_type noresult, result_type yesresult)
        : lower_(lower), higher_(higher), no_(noresult), yes_(yesresult)
    {
    }
    result_type operator()(argument_type s) const { return (s < lower_ || higher_ < s) ? no_ : yes_; }

  private:
    argument_type lower_, higher_;
    result_type no_, yes_;
};

template <class VALUETYPE>
class FindMinMax {
  public:
    typedef VALUETYPE argument_type;
    typedef VALUETYPE result_type;
    typedef VALUETYPE value_type;
    FindMinMax() : min(NumericTraits<value_type>::max()), max(NumericTraits<value_type>::min()), count(0) {}
    void reset()
    {
        count = 0;
        min = NumericTraits<value_type>::max();
        max = NumericTraits<value_type>::min();
    }
    void operator()(const argument_type& v)
    {
        if (count) {
            if (v < min) {
                min = v;
            }
            if (max < v) {
                max = v;
            }
        } else {
            min = v;
            max = v;
        }
        ++count;
    }
    VALUETYPE min, max;
    unsigned int count;
};

class FindBoundingRectangle {
  public:
    Point2D upperLeft, lowerRight;
    bool valid;
    FindBoundingRectangle() : valid(false) {}
    void operator()(const Diff2D& c)
    {
        if (!valid) {
            upperLeft = Point2D(c);
            lowerRight = Point2D(c.x + 1, c.y + 1);
            valid = true;
        } else {
            upperLeft.x = std::min(upperLeft.x, c.x);
            upperLeft.y = std::min(upperLeft.y, c.y);
            lowerRight.x = std::max(lowerRight.x, c.x + 1);
            lowerRight.y = std::max(lowerRight.y, c.y + 1);
        }
    }
    Rect2D operator()() const { return Rect2D(upperLeft, lowerRight); }
};

// ---- convolution filters of the edge-scale contrast mode (not provided) -------------
template <class SI, class SA, class DI, class DA>
void laplacianOfGaussian(SI, SI, SA, DI, DA, double)
{
    vigra_fail("laplacianOfGaussian: not available in the oracle shim");
}

template <class SI, class SA, class DI, class DA>
void gaussianSharpening(SI, SI, SA, DI, DA, double, double)
{
    vigra_fail("gaussianSharpening: not available in the oracle shim");
}

// ---- default accessors, coordinate iteration -----------------------------------------------
template <class T>
inline pair<ImageIter<T>, StandardValueAccessor<typename std::remove_const<T>::type>> destIter(ImageIter<T> ul)
{
    return pair<ImageIter<T>, StandardValueAccessor<typename std::remove_const<T>::type>>(
        ul, StandardValueAccessor<typename std::remove_const<T>::type>());
}

// A Diff2D used as an iterator over image coordinates: its accessor yields
// the coordinate itself.
struct CoordinateAccessor {
    typedef Diff2D value_type;
    Diff2D operator()(const Diff2D& i) const { return i; }
    Diff2D operator()(const Diff2D& i, const Diff2D& d) const { return i + d; }
};

inline triple<Diff2D, Diff2D, CoordinateAccessor> srcIterRange(const Diff2D& ul, const Diff2D& lr)
{
    return triple<Diff2D, Diff2D, CoordinateAccessor>(ul, lr, CoordinateAccessor());
}

template <class SI, class SA, class MI, class MA, class F>
inline void inspectImageIf(const triple<SI, SI, SA>& s, const pair<MI, MA>& m, F& f)
{
    inspectImageIf(s.first, s.second, s.third, m.first, m.second, f);
}

// ---- in-memory image files ---------------------------------------------------------------
// One "file": width x height pixels of `bands` samples (colour bands first,
// then the extra band, i.e. alpha), stored as doubles (exact for the 8/16-bit
// integer and float pixel types), with VIGRA's pixel-type name.
struct MemFile {
    int width = 0, height = 0, bands = 0, extra = 0;
    std::string pixel_type;  // "UINT8", "UINT16", "FLOAT", ...
    Diff2D position;
    std::vector<double> samples;
};

inline std::map<std::string, MemFile>& memfile_table()
{
    static std::map<std::string, MemFile> t;
    return t;
}

inline std::mutex& memfile_mutex()
{
    static std::mutex m;
    return m;
}

inline void memfile_put(const std::string& name, const MemFile& f)
{
    std::lock_guard<std::mutex> l(memfile_mutex());
    memfile_table()[name] = f;
}

inline bool memfile_get(const std::string& name, MemFile& f)
{
    std::lock_guard<std::mutex> l(memfile_mutex());
    auto it = memfile_table().find(name);
    if (it == memfile_table().end()) {
        return false;
    }
    f = it->second;
    return true;
}

inline void memfile_clear()
{
    std::lock_guard<std::mutex> l(memfile_mutex());
    memfile_table().clear();
}

class ImageImportInfo {
  public:
    enum PixelType { UINT8, INT16, UINT16, INT32, UINT32, FLOAT, DOUBLE };
    explicit ImageImportInfo(const char* filename, unsigned int imageIndex = 0) : name_(filename), index_(imageIndex)
    {
        if (!memfile_get(name_, f_)) {
            vigra_fail((std::string("ImageImportInfo: no in-memory image \"") + name_ + "\"").c_str());
        }
    }
    const char* getFileName() const { return name_.c_str(); }
    int width() const { return f_.width; }
    int height() const { return f_.height; }
    Size2D size() const { return Size2D(f_.width, f_.height); }
    int numBands() const { return f_.bands; }
    int numExtraBands() const { return f_.extra; }
    bool isGrayscale() const { return f_.bands - f_.extra == 1; }
    bool isColor() const { return f_.bands - f_.extra == 3; }
    const char* getPixelType() const { return f_.pixel_type.c_str(); }
    Diff2D getPosition() const { return f_.position; }
    Size2D getCanvasSize() const { return Size2D(f_.position.x + f_.width, f_.position.y + f_.height); }
    PixelType pixelType() const
    {
        const std::string& t = f_.pixel_type;
        return t == "UINT8" ? UINT8 : t == "INT16" ? INT16 : t == "UINT16" ? UINT16 : t == "INT32" ? INT32
             : t == "UINT32" ? UINT32 : t == "DOUBLE" ? DOUBLE : FLOAT;
    }
    float getXResolution() const { return 0.0f; }
    float getYResolution() const { return 0.0f; }
    int numImages() const { return 1; }
    int getImageIndex() const { return (int)index_; }
    void setImageIndex(int i) { index_ = (unsigned)i; }
    const MemFile& file() const { return f_; }

  private:
    std::string name_;
    unsigned index_;
    MemFile f_;
};

class ImageExportInfo {
  public:
    explicit ImageExportInfo(const char* filename, const char* = "w") : name_(filename) {}
    ImageExportInfo& setPixelType(const char* t)
    {
        pixel_type_ = t ? t : "";
        return *this;
    }
    const char* getPixelType() const { return pixel_type_.c_str(); }
    ImageExportInfo& setCompression(const char*) { return *this; }
    ImageExportInfo& setXResolution(float) { return *this; }
    ImageExportInfo& setYResolution(float) { return *this; }
    ImageExportInfo& setPosition(const Diff2D& p)
    {
        position_ = p;
        return *this;
    }
    Diff2D getPosition() const { return position_; }
    ImageExportInfo& setCanvasSize(const Size2D&) { return *this; }
    const char* getFileName() const { return name_.c_str(); }
    ImageExportInfo& setFileName(const char* n)
    {
        name_ = n;
        return *this;
    }
    ImageExportInfo& setFileType(const char*) { return *this; }

  private:
    std::string name_;
    std::string pixel_type_;
    Diff2D position_;
};

namespace detail {

// Number of samples of a pixel value and sample access.
template <class T>
struct MemPixel {
    enum { n = 1 };
    static double get(const T& v, int) { return (double)v; }
    static T make(const double* s) { return RequiresExplicitCast<T>::cast(s[0]); }
};

template <class V, unsigned R, unsigned G, unsigned B>
struct MemPixel<RGBValue<V, R, G, B>> {
    enum { n = 3 };
    static double get(const RGBValue<V, R, G, B>& v, int i) { return (double)v[i]; }
    static RGBValue<V, R, G, B> make(const double* s)
    {
        return RGBValue<V, R, G, B>(RequiresExplicitCast<V>::cast(s[0]), RequiresExplicitCast<V>::cast(s[1]),
                                    RequiresExplicitCast<V>::cast(s[2]));
    }
};

}  // namespace detail

template <class DI, class DA>
void importImage(const ImageImportInfo& info, DI ul, DA da)
{
    typedef typename std::decay<typename DA::value_type>::type V;
    const MemFile& f = info.file();
    vigra_precondition(f.bands - f.extra == detail::MemPixel<V>::n, "importImage: band count mismatch");
    for (int y = 0; y < f.height; ++y) {
        for (int x = 0; x < f.width; ++x) {
            const double* s = &f.samples[((size_t)y * f.width + x) * f.bands];
            da.set(detail::MemPixel<V>::make(s), ul, Diff2D(x, y));
        }
    }
}

template <class DI, class DA>
void importImage(const ImageImportInfo& info, const pair<DI, DA>& d)
{
    importImage(info, d.first, d.second);
}

// The colour bands into the image; the extra band, as a sample of the
// image's component type, through the alpha accessor.
template <class DI, class DA, class AI, class AA>
void importImageAlpha(const ImageImportInfo& info, const pair<DI, DA>& img, const pair<AI, AA>& alpha)
{
    typedef typename std::decay<typename DA::value_type>::type V;
    typedef typename NumericTraits<V>::ValueType Component;
    const MemFile& f = info.file();
    vigra_precondition(f.extra == 1 && f.bands - 1 == detail::MemPixel<V>::n, "importImageAlpha: band count mismatch");
    for (int y = 0; y < f.height; ++y) {
        for (int x = 0; x < f.width; ++x) {
            const double* s = &f.samples[((size_t)y * f.width + x) * f.bands];
            img.second.set(detail::MemPixel<V>::make(s), img.first, Diff2D(x, y));
            alpha.second.set(detail::RequiresExplicitCast<Component>::cast(s[f.bands - 1]), alpha.first, Diff2D(x, y));
        }
    }
}

inline std::string memfile_pixel_type_of(const char* requested, const char* fallback)
{
    return (requested && *requested) ? std::string(requested) : std::string(fallback);
}

template <class T>
inline const char* memfile_type_name()
{
    typedef typename NumericTraits<T>::ValueType C;
    return std::is_same<C, UInt8>::value    ? "UINT8"
           : std::is_same<C, UInt16>::value ? "UINT16"
           : std::is_same<C, Int16>::value  ? "INT16"
           : std::is_same<C, Int32>::value  ? "INT32"
           : std::is_same<C, UInt32>::value ? "UINT32"
           : std::is_same<C, double>::value ? "DOUBLE"
                                            : "FLOAT";
}

template <class SI, class SA>
void exportImage(SI ul, SI lr, SA sa, const ImageExportInfo& info)
{
    typedef typename std::decay<typename SA::value_type>::type V;
    MemFile f;
    const Diff2D s = lr - ul;
    f.width = s.x;
    f.height = s.y;
    f.bands = detail::MemPixel<V>::n;
    f.extra = 0;
    f.pixel_type = memfile_pixel_type_of(info.getPixelType(), memfile_type_name<V>());
    f.position = info.getPosition();
    f.samples.resize((size_t)f.width * f.height * f.bands);
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            const V v = sa(ul, Diff2D(x, y));
            for (int b = 0; b < f.bands; ++b) {
                f.samples[((size_t)y * f.width + x) * f.bands + b] = detail::MemPixel<V>::get(v, b);
            }
        }
    }
    memfile_put(info.getFileName(), f);
}

template <class SI, class SA>
void exportImage(const triple<SI, SI, SA>& s, const ImageExportInfo& info)
{
    exportImage(s.first, s.second, s.third, info);
}

template <class SI, class SA, class AI, class AA>
void exportImageAlpha(const triple<SI, SI, SA>& img, const pair<AI, AA>& alpha, const ImageExportInfo& info)
{
    typedef typename std::decay<typename SA::value_type>::type V;
    MemFile f;
    const Diff2D s = img.second - img.first;
    f.width = s.x;
    f.height = s.y;
    f.bands = detail::MemPixel<V>::n + 1;
    f.extra = 1;
    f.pixel_type = memfile_pixel_type_of(info.getPixelType(), memfile_type_name<V>());
    f.position = info.getPosition();
    f.samples.resize((size_t)f.width * f.height * f.bands);
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            const V v = img.third(img.first, Diff2D(x, y));
            double* d = &f.samples[((size_t)y * f.width + x) * f.bands];
            for (int b = 0; b + 1 < f.bands; ++b) {
                d[b] = detail::MemPixel<V>::get(v, b);
            }
            d[f.bands - 1] = (double)alpha.second(alpha.first, Diff2D(x, y));
        }
    }
    memfile_put(info.getFileName(), f);
}

}  // namespace vigra

#endif

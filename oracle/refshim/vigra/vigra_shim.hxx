// vigra_shim.hxx -- a small restatement of the parts of VIGRA (>= 1.9) that
// the reference's pyramid.h, blend.h, fixmath.h, numerictraits.h and
// openmp_vigra.h use, written for this project's test oracle only.  It
// follows VIGRA's documented semantics where results depend on them:
//   * NumericTraits<T>::Promote: int for the integer types narrower than int,
//     the type itself otherwise; RealPromote: double for integers;
//   * fromPromote saturates to the type's range (identity for int and wider);
//   * fromRealPromote of an integer type rounds half away from zero
//     ((int)(v + 0.5) / (int)(v - 0.5)) and saturates;
//   * storing a float/double through an accessor or converting an RGBValue
//     into an integer RGBValue uses fromRealPromote; storing an integer of
//     another integer type uses static_cast (RequiresExplicitCast);
//   * RGBValue arithmetic is componentwise; RGBValue op RGBValue promotes
//     with PromoteTraits; RGBValue * or / a double yields the real-promoted
//     RGBValue.
// It is not VIGRA: only the interfaces the reference headers instantiate.
// vigra_shim_io.hxx adds what src/enfuse.h, src/assemble.h and src/mga.h use.
#ifndef ENB_REFSHIM_VIGRA_SHIM_HXX
#define ENB_REFSHIM_VIGRA_SHIM_HXX

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <ostream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace vigra {

// ---- sized integers -------------------------------------------------------
typedef int8_t Int8;
typedef int16_t Int16;
typedef int32_t Int32;
typedef int64_t Int64;
typedef uint8_t UInt8;
typedef uint16_t UInt16;
typedef uint32_t UInt32;
typedef uint64_t UInt64;

// ---- errors -----------------------------------------------------------------
struct PreconditionViolation : public std::runtime_error {
    explicit PreconditionViolation(const std::string& m) : std::runtime_error(m) {}
};

inline void vigra_precondition(bool cond, const char* msg)
{
    if (!cond) {
        throw PreconditionViolation(msg);
    }
}

inline void vigra_precondition(bool cond, const std::string& msg) { vigra_precondition(cond, msg.c_str()); }

inline void vigra_postcondition(bool cond, const char* msg) { vigra_precondition(cond, msg); }

inline void vigra_fail(const char* msg) { throw std::runtime_error(msg); }

enum SkipInitializationTag { SkipInitialization };

// ---- type flags ---------------------------------------------------------------
struct VigraTrueType {
    static const bool asBool = true;
};
struct VigraFalseType {
    static const bool asBool = false;
};

// ---- 2D geometry ---------------------------------------------------------------
class Diff2D {
  public:
    int x, y;
    Diff2D() : x(0), y(0) {}
    Diff2D(int ax, int ay) : x(ax), y(ay) {}
    Diff2D operator-() const { return Diff2D(-x, -y); }
    Diff2D& operator+=(const Diff2D& o) { x += o.x; y += o.y; return *this; }
    Diff2D& operator-=(const Diff2D& o) { x -= o.x; y -= o.y; return *this; }
    Diff2D operator+(const Diff2D& o) const { return Diff2D(x + o.x, y + o.y); }
    Diff2D operator-(const Diff2D& o) const { return Diff2D(x - o.x, y - o.y); }
    // VIGRA divides both coordinates (truncating toward zero for ints)
    Diff2D operator/(int s) const { return Diff2D(x / s, y / s); }
    bool operator==(const Diff2D& o) const { return x == o.x && y == o.y; }
    bool operator!=(const Diff2D& o) const { return !(*this == o); }
    int width() const { return x; }
    int height() const { return y; }
    int area() const { return x * y; }
};

class Size2D : public Diff2D {
  public:
    Size2D() {}
    Size2D(int w, int h) : Diff2D(w, h) {}
    Size2D(const Diff2D& d) : Diff2D(d) {}
};

class Point2D : public Diff2D {
  public:
    Point2D() {}
    Point2D(int px, int py) : Diff2D(px, py) {}
    Point2D(const Diff2D& d) : Diff2D(d) {}
};

inline std::ostream& operator<<(std::ostream& o, const Diff2D& d) { return o << "(" << d.x << ", " << d.y << ")"; }

class Rect2D {
  public:
    Rect2D() {}
    Rect2D(const Point2D& ul, const Point2D& lr) : ul_(ul), lr_(lr) {}
    Rect2D(const Size2D& s) : ul_(0, 0), lr_(s) {}
    int left() const { return ul_.x; }
    int top() const { return ul_.y; }
    int right() const { return lr_.x; }
    int bottom() const { return lr_.y; }
    int width() const { return lr_.x - ul_.x; }
    int height() const { return lr_.y - ul_.y; }
    int area() const { return width() * height(); }
    Size2D size() const { return Size2D(width(), height()); }
    Point2D upperLeft() const { return ul_; }
    Point2D lowerRight() const { return lr_; }
    void setUpperLeft(const Point2D& p) { ul_ = p; }
    void setLowerRight(const Point2D& p) { lr_ = p; }
    void moveBy(const Diff2D& d) { ul_ += d; lr_ += d; }
    void addBorder(int b) { ul_ -= Diff2D(b, b); lr_ += Diff2D(b, b); }
    bool isEmpty() const { return width() <= 0 || height() <= 0; }
    Rect2D& operator&=(const Rect2D& r)
    {
        ul_.x = std::max(ul_.x, r.ul_.x);
        ul_.y = std::max(ul_.y, r.ul_.y);
        lr_.x = std::min(lr_.x, r.lr_.x);
        lr_.y = std::min(lr_.y, r.lr_.y);
        return *this;
    }

  private:
    Point2D ul_, lr_;
};

inline std::ostream& operator<<(std::ostream& o, const Rect2D& r)
{
    return o << "[" << r.upperLeft() << " to " << r.lowerRight() << "]";
}

// ---- tuples -----------------------------------------------------------------------
template <class T1, class T2, class T3>
struct triple {
    T1 first;
    T2 second;
    T3 third;
    triple() {}
    triple(const T1& a, const T2& b, const T3& c) : first(a), second(b), third(c) {}
};

template <class T1, class T2, class T3>
inline triple<T1, T2, T3> make_triple(T1 a, T2 b, T3 c)
{
    return triple<T1, T2, T3>(a, b, c);
}

using std::pair;

// ---- numeric traits ------------------------------------------------------------------
template <class T>
struct NumericTraits;

namespace detail {

template <class T>
struct IntTraitsBase {
    typedef T Type;
    typedef VigraTrueType isIntegral;
    typedef VigraTrueType isScalar;
    typedef VigraTrueType isOrdered;
    typedef VigraFalseType isComplex;
    typedef double RealPromote;
    typedef T ValueType;
    static T zero() { return T(0); }
    static T one() { return T(1); }
    static T nonZero() { return T(1); }
    static T min() { return std::numeric_limits<T>::min(); }
    static T max() { return std::numeric_limits<T>::max(); }
    static double toRealPromote(T v) { return (double)v; }
    static T fromRealPromote(double v)
    {
        return v < 0.0 ? (v <= (double)min() ? min() : (T)(v - 0.5))
                       : (v >= (double)max() ? max() : (T)(v + 0.5));
    }
};

}  // namespace detail

#define ENB_SHIM_SMALL_INT(T, SIGNED)                                                     \
    template <>                                                                            \
    struct NumericTraits<T> : detail::IntTraitsBase<T> {                                  \
        typedef int Promote;                                                               \
        typedef SIGNED isSigned;                                                           \
        static int toPromote(T v) { return (int)v; }                                       \
        static T fromPromote(int v) { return v <= (int)min() ? min() : (v >= (int)max() ? max() : (T)v); } \
    };
ENB_SHIM_SMALL_INT(signed char, VigraTrueType)
ENB_SHIM_SMALL_INT(unsigned char, VigraFalseType)
ENB_SHIM_SMALL_INT(short, VigraTrueType)
ENB_SHIM_SMALL_INT(unsigned short, VigraFalseType)
#undef ENB_SHIM_SMALL_INT

template <>
struct NumericTraits<char> : NumericTraits<signed char> {
    typedef char Type;
};

#define ENB_SHIM_WIDE_INT(T, SIGNED)                           \
    template <>                                                 \
    struct NumericTraits<T> : detail::IntTraitsBase<T> {       \
        typedef T Promote;                                      \
        typedef SIGNED isSigned;                                \
        static T toPromote(T v) { return v; }                   \
        static T fromPromote(T v) { return v; }                 \
    };
ENB_SHIM_WIDE_INT(int, VigraTrueType)
ENB_SHIM_WIDE_INT(unsigned int, VigraFalseType)
ENB_SHIM_WIDE_INT(long, VigraTrueType)
ENB_SHIM_WIDE_INT(unsigned long, VigraFalseType)
ENB_SHIM_WIDE_INT(long long, VigraTrueType)
ENB_SHIM_WIDE_INT(unsigned long long, VigraFalseType)
#undef ENB_SHIM_WIDE_INT

#define ENB_SHIM_REAL(T)                                          \
    template <>                                                    \
    struct NumericTraits<T> {                                      \
        typedef T Type;                                            \
        typedef T Promote;                                         \
        typedef T RealPromote;                                     \
        typedef T ValueType;                                       \
        typedef VigraFalseType isIntegral;                         \
        typedef VigraTrueType isScalar;                            \
        typedef VigraTrueType isSigned;                            \
        typedef VigraTrueType isOrdered;                           \
        typedef VigraFalseType isComplex;                          \
        static T zero() { return static_cast<T>(0); }              \
        static T one() { return static_cast<T>(1); }               \
        static T nonZero() { return static_cast<T>(1); }           \
        static T min() { return -std::numeric_limits<T>::max(); } \
        static T max() { return std::numeric_limits<T>::max(); }   \
        static T smallestPositive() { return std::numeric_limits<T>::min(); } \
        static T toPromote(T v) { return v; }                      \
        static T toRealPromote(T v) { return v; }                  \
        static T fromPromote(T v) { return v; }                    \
        static T fromRealPromote(T v) { return v; }                \
    };
ENB_SHIM_REAL(float)
ENB_SHIM_REAL(double)
ENB_SHIM_REAL(long double)
#undef ENB_SHIM_REAL

template <class A, class B>
struct PromoteTraits {
    typedef decltype(A() + B()) Promote;
};

template <class T>
struct SquareRootTraits {
    typedef double SquareRootResult;
    typedef T SquareRootArgument;
};

namespace detail {

// How a value is converted when stored into a pixel of type T.
template <class T>
struct RequiresExplicitCast {
    template <class U>
    static const U& cast(const U& v)
    {
        return v;
    }
};

#define ENB_SHIM_CAST(T)                                                  \
    template <>                                                            \
    struct RequiresExplicitCast<T> {                                       \
        static T cast(float v) { return NumericTraits<T>::fromRealPromote(v); }  \
        static T cast(double v) { return NumericTraits<T>::fromRealPromote(v); } \
        static T cast(T v) { return v; }                                   \
        template <class U>                                                 \
        static T cast(U v)                                                 \
        {                                                                  \
            return static_cast<T>(v);                                      \
        }                                                                  \
    };
ENB_SHIM_CAST(signed char)
ENB_SHIM_CAST(unsigned char)
ENB_SHIM_CAST(short)
ENB_SHIM_CAST(unsigned short)
ENB_SHIM_CAST(int)
ENB_SHIM_CAST(unsigned int)
ENB_SHIM_CAST(long)
ENB_SHIM_CAST(unsigned long)
ENB_SHIM_CAST(long long)
ENB_SHIM_CAST(unsigned long long)
#undef ENB_SHIM_CAST

}  // namespace detail

// ---- RGBValue ------------------------------------------------------------------------
template <class V, unsigned R = 0, unsigned G = 1, unsigned B = 2>
class RGBValue {
  public:
    typedef V value_type;
    typedef V* iterator;
    typedef const V* const_iterator;
    enum { static_size = 3 };

    RGBValue() { d_[0] = d_[1] = d_[2] = V(); }
    explicit RGBValue(V v) { d_[0] = d_[1] = d_[2] = v; }
    RGBValue(V r, V g, V b)
    {
        d_[R] = r;
        d_[G] = g;
        d_[B] = b;
    }
    template <class U, unsigned R2, unsigned G2, unsigned B2>
    RGBValue(const RGBValue<U, R2, G2, B2>& o)
    {
        d_[R] = detail::RequiresExplicitCast<V>::cast(o.red());
        d_[G] = detail::RequiresExplicitCast<V>::cast(o.green());
        d_[B] = detail::RequiresExplicitCast<V>::cast(o.blue());
    }
    template <class U, unsigned R2, unsigned G2, unsigned B2>
    RGBValue& operator=(const RGBValue<U, R2, G2, B2>& o)
    {
        d_[R] = detail::RequiresExplicitCast<V>::cast(o.red());
        d_[G] = detail::RequiresExplicitCast<V>::cast(o.green());
        d_[B] = detail::RequiresExplicitCast<V>::cast(o.blue());
        return *this;
    }

    V& operator[](int i) { return d_[i]; }
    const V& operator[](int i) const { return d_[i]; }
    const V& red() const { return d_[R]; }
    const V& green() const { return d_[G]; }
    const V& blue() const { return d_[B]; }
    void setRed(V v) { d_[R] = v; }
    void setGreen(V v) { d_[G] = v; }
    void setBlue(V v) { d_[B] = v; }
    // 0.3 R + 0.59 G + 0.11 B in double, stored as the component type
    // (rounded and saturated for integer components)
    V luminance() const { return detail::RequiresExplicitCast<V>::cast(0.3 * red() + 0.59 * green() + 0.11 * blue()); }
    iterator begin() { return d_; }
    iterator end() { return d_ + 3; }
    const_iterator begin() const { return d_; }
    const_iterator end() const { return d_ + 3; }
    static unsigned size() { return 3; }

    template <class U, unsigned R2, unsigned G2, unsigned B2>
    RGBValue& operator+=(const RGBValue<U, R2, G2, B2>& o)
    {
        for (int i = 0; i < 3; ++i) d_[i] += o[i];
        return *this;
    }
    template <class U, unsigned R2, unsigned G2, unsigned B2>
    RGBValue& operator-=(const RGBValue<U, R2, G2, B2>& o)
    {
        for (int i = 0; i < 3; ++i) d_[i] -= o[i];
        return *this;
    }
    template <class U, unsigned R2, unsigned G2, unsigned B2>
    RGBValue& operator*=(const RGBValue<U, R2, G2, B2>& o)
    {
        for (int i = 0; i < 3; ++i) d_[i] *= o[i];
        return *this;
    }
    template <class U, unsigned R2, unsigned G2, unsigned B2>
    RGBValue& operator/=(const RGBValue<U, R2, G2, B2>& o)
    {
        for (int i = 0; i < 3; ++i) d_[i] /= o[i];
        return *this;
    }
    RGBValue& operator*=(double v)
    {
        for (int i = 0; i < 3; ++i) d_[i] = detail::RequiresExplicitCast<V>::cast(d_[i] * v);
        return *this;
    }
    RGBValue& operator/=(double v)
    {
        for (int i = 0; i < 3; ++i) d_[i] = detail::RequiresExplicitCast<V>::cast(d_[i] / v);
        return *this;
    }
    RGBValue operator-() const { return RGBValue(-d_[R], -d_[G], -d_[B]); }

  private:
    V d_[3];
};

template <class V1, unsigned R, unsigned G, unsigned B, class V2, unsigned R2, unsigned G2, unsigned B2>
inline bool operator==(const RGBValue<V1, R, G, B>& a, const RGBValue<V2, R2, G2, B2>& b)
{
    return a.red() == b.red() && a.green() == b.green() && a.blue() == b.blue();
}

template <class V1, unsigned R, unsigned G, unsigned B, class V2, unsigned R2, unsigned G2, unsigned B2>
inline bool operator!=(const RGBValue<V1, R, G, B>& a, const RGBValue<V2, R2, G2, B2>& b)
{
    return !(a == b);
}

template <class V, unsigned R, unsigned G, unsigned B>
struct NumericTraits<RGBValue<V, R, G, B>> {
    typedef RGBValue<V, R, G, B> Type;
    typedef RGBValue<typename NumericTraits<V>::Promote, R, G, B> Promote;
    typedef RGBValue<typename NumericTraits<V>::RealPromote, R, G, B> RealPromote;
    typedef V ValueType;
    typedef typename NumericTraits<V>::isIntegral isIntegral;
    typedef VigraFalseType isScalar;
    typedef typename NumericTraits<V>::isSigned isSigned;
    typedef VigraFalseType isOrdered;
    typedef VigraFalseType isComplex;
    static Type zero() { return Type(NumericTraits<V>::zero()); }
    static Type one() { return Type(NumericTraits<V>::one()); }
    static Type nonZero() { return Type(NumericTraits<V>::nonZero()); }
    static Type min() { return Type(NumericTraits<V>::min()); }
    static Type max() { return Type(NumericTraits<V>::max()); }
    static Promote toPromote(const Type& v)
    {
        return Promote(NumericTraits<V>::toPromote(v.red()), NumericTraits<V>::toPromote(v.green()),
                       NumericTraits<V>::toPromote(v.blue()));
    }
    static RealPromote toRealPromote(const Type& v)
    {
        return RealPromote(NumericTraits<V>::toRealPromote(v.red()), NumericTraits<V>::toRealPromote(v.green()),
                           NumericTraits<V>::toRealPromote(v.blue()));
    }
    template <class U>
    static Type fromPromote(const RGBValue<U, R, G, B>& v)
    {
        return Type(NumericTraits<V>::fromPromote(v.red()), NumericTraits<V>::fromPromote(v.green()),
                    NumericTraits<V>::fromPromote(v.blue()));
    }
    template <class U>
    static Type fromRealPromote(const RGBValue<U, R, G, B>& v)
    {
        return Type(NumericTraits<V>::fromRealPromote(v.red()), NumericTraits<V>::fromRealPromote(v.green()),
                    NumericTraits<V>::fromRealPromote(v.blue()));
    }
};

template <class V1, unsigned R, unsigned G, unsigned B, class V2, unsigned R2, unsigned G2, unsigned B2>
struct PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>> {
    typedef RGBValue<typename PromoteTraits<V1, V2>::Promote, R, G, B> Promote;
};

template <class V1, unsigned R, unsigned G, unsigned B, class V2, unsigned R2, unsigned G2, unsigned B2>
inline typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote
operator+(const RGBValue<V1, R, G, B>& a, const RGBValue<V2, R2, G2, B2>& b)
{
    typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote r(a);
    r += b;
    return r;
}

template <class V1, unsigned R, unsigned G, unsigned B, class V2, unsigned R2, unsigned G2, unsigned B2>
inline typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote
operator-(const RGBValue<V1, R, G, B>& a, const RGBValue<V2, R2, G2, B2>& b)
{
    typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote r(a);
    r -= b;
    return r;
}

template <class V1, unsigned R, unsigned G, unsigned B, class V2, unsigned R2, unsigned G2, unsigned B2>
inline typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote
operator*(const RGBValue<V1, R, G, B>& a, const RGBValue<V2, R2, G2, B2>& b)
{
    typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote r(a);
    r *= b;
    return r;
}

template <class V1, unsigned R, unsigned G, unsigned B, class V2, unsigned R2, unsigned G2, unsigned B2>
inline typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote
operator/(const RGBValue<V1, R, G, B>& a, const RGBValue<V2, R2, G2, B2>& b)
{
    typename PromoteTraits<RGBValue<V1, R, G, B>, RGBValue<V2, R2, G2, B2>>::Promote r(a);
    r /= b;
    return r;
}

template <class V, unsigned R, unsigned G, unsigned B>
inline typename NumericTraits<RGBValue<V, R, G, B>>::RealPromote operator*(double v, const RGBValue<V, R, G, B>& a)
{
    typename NumericTraits<RGBValue<V, R, G, B>>::RealPromote r(a);
    r *= v;
    return r;
}

template <class V, unsigned R, unsigned G, unsigned B>
inline typename NumericTraits<RGBValue<V, R, G, B>>::RealPromote operator*(const RGBValue<V, R, G, B>& a, double v)
{
    typename NumericTraits<RGBValue<V, R, G, B>>::RealPromote r(a);
    r *= v;
    return r;
}

template <class V, unsigned R, unsigned G, unsigned B>
inline typename NumericTraits<RGBValue<V, R, G, B>>::RealPromote operator/(const RGBValue<V, R, G, B>& a, double v)
{
    typename NumericTraits<RGBValue<V, R, G, B>>::RealPromote r(a);
    r /= v;
    return r;
}

template <class V, unsigned R, unsigned G, unsigned B>
inline std::ostream& operator<<(std::ostream& o, const RGBValue<V, R, G, B>& v)
{
    return o << "(" << v.red() << ", " << v.green() << ", " << v.blue() << ")";
}

// ---- image iterators ------------------------------------------------------------------
template <class T>
class ImageIter {
  public:
    typedef typename std::remove_const<T>::type value_type;
    typedef value_type PixelType;
    typedef T& reference;
    typedef T& index_reference;
    typedef T* pointer;
    typedef Diff2D difference_type;
    typedef T* row_iterator;
    typedef int MoveX;
    typedef int MoveY;

    // x and y are the column and row of the current position; they
    // compare, step and subtract like VIGRA's MoveX/MoveY members.
    struct Coord {
        int v;
        Coord& operator++() { ++v; return *this; }
        Coord operator++(int) { Coord c = *this; ++v; return c; }
        Coord& operator--() { --v; return *this; }
        Coord operator--(int) { Coord c = *this; --v; return c; }
        Coord& operator+=(int d) { v += d; return *this; }
        Coord& operator-=(int d) { v -= d; return *this; }
        int operator-(const Coord& o) const { return v - o.v; }
        bool operator==(const Coord& o) const { return v == o.v; }
        bool operator!=(const Coord& o) const { return v != o.v; }
        bool operator<(const Coord& o) const { return v < o.v; }
        bool operator<=(const Coord& o) const { return v <= o.v; }
        bool operator>(const Coord& o) const { return v > o.v; }
        bool operator>=(const Coord& o) const { return v >= o.v; }
    };

    Coord x, y;

    ImageIter() : base_(nullptr), stride_(0) { x.v = y.v = 0; }
    ImageIter(T* base, std::ptrdiff_t stride, int px = 0, int py = 0) : base_(base), stride_(stride)
    {
        x.v = px;
        y.v = py;
    }
    template <class U>
    ImageIter(const ImageIter<U>& o) : base_(o.base()), stride_(o.stride())
    {
        x.v = o.x.v;
        y.v = o.y.v;
    }

    T* base() const { return base_; }
    std::ptrdiff_t stride() const { return stride_; }

    T& operator*() const { return base_[(std::ptrdiff_t)y.v * stride_ + x.v]; }
    T* operator->() const { return &**this; }
    T& operator[](const Diff2D& d) const { return base_[(std::ptrdiff_t)(y.v + d.y) * stride_ + x.v + d.x]; }
    T& operator()(int dx, int dy) const { return base_[(std::ptrdiff_t)(y.v + dy) * stride_ + x.v + dx]; }
    T* operator[](int dy) const { return base_ + (std::ptrdiff_t)(y.v + dy) * stride_ + x.v; }
    row_iterator rowIterator() const { return &**this; }

    ImageIter& operator+=(const Diff2D& d) { x.v += d.x; y.v += d.y; return *this; }
    ImageIter& operator-=(const Diff2D& d) { x.v -= d.x; y.v -= d.y; return *this; }
    ImageIter operator+(const Diff2D& d) const { ImageIter r = *this; r += d; return r; }
    ImageIter operator-(const Diff2D& d) const { ImageIter r = *this; r -= d; return r; }
    Diff2D operator-(const ImageIter& o) const { return Diff2D(x.v - o.x.v, y.v - o.y.v); }
    bool operator==(const ImageIter& o) const { return base_ == o.base_ && x.v == o.x.v && y.v == o.y.v; }
    bool operator!=(const ImageIter& o) const { return !(*this == o); }

  private:
    T* base_;
    std::ptrdiff_t stride_;
};

// ---- accessors ----------------------------------------------------------------------
template <class T>
class StandardValueAccessor {
  public:
    typedef T value_type;
    template <class I>
    T operator()(const I& i) const
    {
        return *i;
    }
    template <class I, class D>
    T operator()(const I& i, const D& d) const
    {
        return i[d];
    }
    template <class V, class I>
    void set(const V& v, const I& i) const
    {
        *i = detail::RequiresExplicitCast<T>::cast(v);
    }
    template <class V, class I, class D>
    void set(const V& v, const I& i, const D& d) const
    {
        i[d] = detail::RequiresExplicitCast<T>::cast(v);
    }
};

template <class T>
class StandardConstValueAccessor {
  public:
    typedef T value_type;
    template <class I>
    T operator()(const I& i) const
    {
        return *i;
    }
    template <class I, class D>
    T operator()(const I& i, const D& d) const
    {
        return i[d];
    }
};

template <class T>
using StandardAccessor = StandardValueAccessor<T>;
template <class T>
using StandardConstAccessor = StandardConstValueAccessor<T>;

// ---- BasicImage ----------------------------------------------------------------------
template <class T>
class BasicImage {
  public:
    typedef T value_type;
    typedef T PixelType;
    typedef ImageIter<T> traverser;
    typedef ImageIter<const T> const_traverser;
    typedef ImageIter<T> Iterator;
    typedef ImageIter<const T> ConstIterator;
    typedef StandardValueAccessor<T> Accessor;
    typedef StandardConstValueAccessor<T> ConstAccessor;
    typedef Size2D size_type;
    typedef Diff2D difference_type;

    BasicImage() : w_(0), h_(0) {}
    BasicImage(int w, int h) : w_(w), h_(h), d_((size_t)w * h) {}
    BasicImage(const Diff2D& s) : w_(s.x), h_(s.y), d_((size_t)s.x * s.y) {}
    BasicImage(int w, int h, const T& v) : w_(w), h_(h), d_((size_t)w * h, v) {}
    BasicImage(const Diff2D& s, SkipInitializationTag) : w_(s.x), h_(s.y), d_((size_t)s.x * s.y) {}
    BasicImage(const Diff2D& s, const T& v) : w_(s.x), h_(s.y), d_((size_t)s.x * s.y, v) {}

    int width() const { return w_; }
    int height() const { return h_; }
    Size2D size() const { return Size2D(w_, h_); }
    T* data() { return d_.data(); }
    const T* data() const { return d_.data(); }
    T& operator()(int x, int y) { return d_[(size_t)y * w_ + x]; }
    const T& operator()(int x, int y) const { return d_[(size_t)y * w_ + x]; }
    T& operator[](const Diff2D& p) { return (*this)(p.x, p.y); }
    const T& operator[](const Diff2D& p) const { return (*this)(p.x, p.y); }

    traverser upperLeft() { return traverser(d_.data(), w_, 0, 0); }
    traverser lowerRight() { return traverser(d_.data(), w_, w_, h_); }
    const_traverser upperLeft() const { return const_traverser(d_.data(), w_, 0, 0); }
    const_traverser lowerRight() const { return const_traverser(d_.data(), w_, w_, h_); }
    Accessor accessor() { return Accessor(); }
    ConstAccessor accessor() const { return ConstAccessor(); }

    void resize(int w, int h) { w_ = w; h_ = h; d_.assign((size_t)w * h, T()); }
    void init(const T& v) { std::fill(d_.begin(), d_.end(), v); }

    // scan-order iteration over all pixels (row after row)
    typedef T* ScanOrderIterator;
    typedef const T* ConstScanOrderIterator;
    T* begin() { return d_.data(); }
    T* end() { return d_.data() + d_.size(); }
    const T* begin() const { return d_.data(); }
    const T* end() const { return d_.data() + d_.size(); }

    // a column as a strided iterator
    struct column_iterator {
        T* p;
        int stride;
        T& operator*() const { return *p; }
        T* operator->() const { return p; }
        column_iterator& operator++() { p += stride; return *this; }
        bool operator!=(const column_iterator& o) const { return p != o.p; }
        bool operator==(const column_iterator& o) const { return p == o.p; }
    };
    column_iterator columnBegin(int x) { return column_iterator{d_.data() + x, w_}; }
    column_iterator columnEnd(int x) { return column_iterator{d_.data() + x + (size_t)h_ * w_, w_}; }

  private:
    int w_, h_;
    std::vector<T> d_;
};

typedef BasicImage<UInt8> BImage;
typedef BasicImage<UInt16> UInt16Image;
typedef BasicImage<RGBValue<UInt16>> UInt16RGBImage;

// ---- argument object factories --------------------------------------------------------
template <class T>
inline triple<typename BasicImage<T>::const_traverser, typename BasicImage<T>::const_traverser,
              typename BasicImage<T>::ConstAccessor>
srcImageRange(const BasicImage<T>& img)
{
    return triple<typename BasicImage<T>::const_traverser, typename BasicImage<T>::const_traverser,
                  typename BasicImage<T>::ConstAccessor>(img.upperLeft(), img.lowerRight(), img.accessor());
}

template <class T>
inline pair<typename BasicImage<T>::const_traverser, typename BasicImage<T>::ConstAccessor>
srcImage(const BasicImage<T>& img)
{
    return pair<typename BasicImage<T>::const_traverser, typename BasicImage<T>::ConstAccessor>(img.upperLeft(),
                                                                                                img.accessor());
}

template <class T>
inline pair<typename BasicImage<T>::const_traverser, typename BasicImage<T>::ConstAccessor>
maskImage(const BasicImage<T>& img)
{
    return srcImage(img);
}

template <class T>
inline triple<typename BasicImage<T>::traverser, typename BasicImage<T>::traverser, typename BasicImage<T>::Accessor>
destImageRange(BasicImage<T>& img)
{
    return triple<typename BasicImage<T>::traverser, typename BasicImage<T>::traverser,
                  typename BasicImage<T>::Accessor>(img.upperLeft(), img.lowerRight(), img.accessor());
}

template <class T>
inline pair<typename BasicImage<T>::traverser, typename BasicImage<T>::Accessor> destImage(BasicImage<T>& img)
{
    return pair<typename BasicImage<T>::traverser, typename BasicImage<T>::Accessor>(img.upperLeft(), img.accessor());
}

template <class I, class A>
inline triple<I, I, A> srcIterRange(I ul, I lr, A a)
{
    return triple<I, I, A>(ul, lr, a);
}

template <class I, class A>
inline pair<I, A> srcIter(I ul, A a)
{
    return pair<I, A>(ul, a);
}

template <class I, class A>
inline pair<I, A> maskIter(I ul, A a)
{
    return pair<I, A>(ul, a);
}

template <class I, class A>
inline triple<I, I, A> destIterRange(I ul, I lr, A a)
{
    return triple<I, I, A>(ul, lr, a);
}

template <class I, class A>
inline pair<I, A> destIter(I ul, A a)
{
    return pair<I, A>(ul, a);
}

// ---- image algorithms (serial) ----------------------------------------------------------
template <class SI, class SA, class DI, class DA, class F>
inline void transformImage(SI sul, SI slr, SA sa, DI dul, DA da, const F& f)
{
    const Diff2D s = slr - sul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            da.set(f(sa(sul, Diff2D(x, y))), dul, Diff2D(x, y));
        }
    }
}

template <class SI, class SA, class DI, class DA, class F>
inline void transformImage(triple<SI, SI, SA> s, pair<DI, DA> d, const F& f)
{
    transformImage(s.first, s.second, s.third, d.first, d.second, f);
}

template <class SI, class SA, class MI, class MA, class DI, class DA, class F>
inline void transformImageIf(SI sul, SI slr, SA sa, MI mul, MA ma, DI dul, DA da, const F& f)
{
    const Diff2D s = slr - sul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            if (ma(mul, Diff2D(x, y))) {
                da.set(f(sa(sul, Diff2D(x, y))), dul, Diff2D(x, y));
            }
        }
    }
}

template <class SI, class SA, class MI, class MA, class DI, class DA, class F>
inline void transformImageIf(triple<SI, SI, SA> s, pair<MI, MA> m, pair<DI, DA> d, const F& f)
{
    transformImageIf(s.first, s.second, s.third, m.first, m.second, d.first, d.second, f);
}

template <class S1, class A1, class S2, class A2, class DI, class DA, class F>
inline void combineTwoImages(S1 s1ul, S1 s1lr, A1 a1, S2 s2ul, A2 a2, DI dul, DA da, const F& f)
{
    const Diff2D s = s1lr - s1ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            const Diff2D p(x, y);
            da.set(f(a1(s1ul, p), a2(s2ul, p)), dul, p);
        }
    }
}

template <class S1, class A1, class S2, class A2, class DI, class DA, class F>
inline void combineTwoImages(triple<S1, S1, A1> s1, pair<S2, A2> s2, pair<DI, DA> d, const F& f)
{
    combineTwoImages(s1.first, s1.second, s1.third, s2.first, s2.second, d.first, d.second, f);
}

template <class S1, class A1, class S2, class A2, class MI, class MA, class DI, class DA, class F>
inline void combineTwoImagesIf(S1 s1ul, S1 s1lr, A1 a1, S2 s2ul, A2 a2, MI mul, MA ma, DI dul, DA da, const F& f)
{
    const Diff2D s = s1lr - s1ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            const Diff2D p(x, y);
            if (ma(mul, p)) {
                da.set(f(a1(s1ul, p), a2(s2ul, p)), dul, p);
            }
        }
    }
}

template <class S1, class A1, class S2, class A2, class S3, class A3, class DI, class DA, class F>
inline void combineThreeImages(S1 s1ul, S1 s1lr, A1 a1, S2 s2ul, A2 a2, S3 s3ul, A3 a3, DI dul, DA da, const F& f)
{
    const Diff2D s = s1lr - s1ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            const Diff2D p(x, y);
            da.set(f(a1(s1ul, p), a2(s2ul, p), a3(s3ul, p)), dul, p);
        }
    }
}

template <class S1, class A1, class S2, class A2, class S3, class A3, class DI, class DA, class F>
inline void combineThreeImages(triple<S1, S1, A1> s1, pair<S2, A2> s2, pair<S3, A3> s3, pair<DI, DA> d, const F& f)
{
    combineThreeImages(s1.first, s1.second, s1.third, s2.first, s2.second, s3.first, s3.second, d.first, d.second, f);
}

template <class SI, class SA, class DI, class DA>
inline void copyImage(SI sul, SI slr, SA sa, DI dul, DA da)
{
    const Diff2D s = slr - sul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            da.set(sa(sul, Diff2D(x, y)), dul, Diff2D(x, y));
        }
    }
}

template <class SI, class SA, class DI, class DA>
inline void copyImage(triple<SI, SI, SA> s, pair<DI, DA> d)
{
    copyImage(s.first, s.second, s.third, d.first, d.second);
}

template <class SI, class SA, class MI, class MA, class DI, class DA>
inline void copyImageIf(SI sul, SI slr, SA sa, MI mul, MA ma, DI dul, DA da)
{
    const Diff2D s = slr - sul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            if (ma(mul, Diff2D(x, y))) {
                da.set(sa(sul, Diff2D(x, y)), dul, Diff2D(x, y));
            }
        }
    }
}

template <class SI, class SA, class MI, class MA, class DI, class DA>
inline void copyImageIf(triple<SI, SI, SA> s, pair<MI, MA> m, pair<DI, DA> d)
{
    copyImageIf(s.first, s.second, s.third, m.first, m.second, d.first, d.second);
}

template <class DI, class DA, class V>
inline void initImage(DI ul, DI lr, DA da, const V& v)
{
    const Diff2D s = lr - ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            da.set(v, ul, Diff2D(x, y));
        }
    }
}

template <class DI, class DA, class V>
inline void initImage(triple<DI, DI, DA> d, const V& v)
{
    initImage(d.first, d.second, d.third, v);
}

template <class DI, class DA, class MI, class MA, class V>
inline void initImageIf(DI ul, DI lr, DA da, MI mul, MA ma, const V& v)
{
    const Diff2D s = lr - ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            if (ma(mul, Diff2D(x, y))) {
                da.set(v, ul, Diff2D(x, y));
            }
        }
    }
}

template <class DI, class DA, class MI, class MA, class V>
inline void initImageIf(triple<DI, DI, DA> d, pair<MI, MA> m, const V& v)
{
    initImageIf(d.first, d.second, d.third, m.first, m.second, v);
}

template <class SI, class SA, class F>
inline void inspectImage(SI ul, SI lr, SA sa, F& f)
{
    const Diff2D s = lr - ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            f(sa(ul, Diff2D(x, y)));
        }
    }
}

template <class SI, class SA, class F>
inline void inspectImage(triple<SI, SI, SA> s, F& f)
{
    inspectImage(s.first, s.second, s.third, f);
}

template <class SI, class SA, class MI, class MA, class F>
inline void inspectImageIf(SI ul, SI lr, SA sa, MI mul, MA ma, F& f)
{
    const Diff2D s = lr - ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            if (ma(mul, Diff2D(x, y))) {
                f(sa(ul, Diff2D(x, y)));
            }
        }
    }
}

template <class S1, class A1, class S2, class A2, class F>
inline void inspectTwoImages(S1 ul, S1 lr, A1 a1, S2 ul2, A2 a2, F& f)
{
    const Diff2D s = lr - ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            f(a1(ul, Diff2D(x, y)), a2(ul2, Diff2D(x, y)));
        }
    }
}

template <class S1, class A1, class S2, class A2, class MI, class MA, class F>
inline void inspectTwoImagesIf(S1 ul, S1 lr, A1 a1, S2 ul2, A2 a2, MI mul, MA ma, F& f)
{
    const Diff2D s = lr - ul;
    for (int y = 0; y < s.y; ++y) {
        for (int x = 0; x < s.x; ++x) {
            if (ma(mul, Diff2D(x, y))) {
                f(a1(ul, Diff2D(x, y)), a2(ul2, Diff2D(x, y)));
            }
        }
    }
}

// Used by the reference only in code paths the oracle does not take.
template <class SI, class SA, class DI, class DA, class V>
void distanceTransform(SI, SI, SA, DI, DA, V, int)
{
    vigra_fail("distanceTransform: not available in the oracle shim");
}

template <class T1, class T2>
struct LinearIntensityTransform {
    T1 scale;
    T2 offset;
    template <class V>
    V operator()(const V& v) const
    {
        return v;
    }
};

template <class A, class B>
LinearIntensityTransform<double, double> linearRangeMapping(const A&, const A&, const B&, const B&)
{
    vigra_fail("linearRangeMapping: not available in the oracle shim");
    return LinearIntensityTransform<double, double>();
}

// ---- small fixed vectors and the colour conversion functors --------------------------
template <class T, int N>
struct TinyVector {
    T d[N];
    T& operator[](int i) { return d[i]; }
    const T& operator[](int i) const { return d[i]; }
};

template <class T, int N>
inline TinyVector<T, N> operator/(TinyVector<T, N> v, double d)
{
    for (int i = 0; i < N; ++i) v[i] /= d;
    return v;
}

template <class T, int N>
inline std::ostream& operator<<(std::ostream& o, const TinyVector<T, N>& v)
{
    o << "(";
    for (int i = 0; i < N; ++i) o << (i ? ", " : "") << v[i];
    return o << ")";
}

// The non-identity colour spaces are not part of the oracle: these functors
// only give fixmath.h's colour-space classes their types.
#define ENB_SHIM_COLOUR_FUNCTOR(NAME)                                        \
    template <class T>                                                        \
    class NAME {                                                              \
      public:                                                                 \
        typedef TinyVector<T, 3> argument_type;                               \
        typedef TinyVector<T, 3> result_type;                                 \
        typedef TinyVector<T, 3> value_type;                                  \
        NAME() {}                                                             \
        explicit NAME(double) {}                                              \
        result_type operator()(const argument_type&) const                    \
        {                                                                     \
            vigra_fail(#NAME ": not available in the oracle shim");           \
            return result_type();                                             \
        }                                                                     \
    };
ENB_SHIM_COLOUR_FUNCTOR(RGB2XYZFunctor)
ENB_SHIM_COLOUR_FUNCTOR(XYZ2RGBFunctor)
ENB_SHIM_COLOUR_FUNCTOR(XYZ2LuvFunctor)
ENB_SHIM_COLOUR_FUNCTOR(Luv2XYZFunctor)
ENB_SHIM_COLOUR_FUNCTOR(XYZ2LabFunctor)
ENB_SHIM_COLOUR_FUNCTOR(Lab2XYZFunctor)
#undef ENB_SHIM_COLOUR_FUNCTOR

// The l-star and pl-star gray projectors (src/mga.h) construct these for
// every RGB projector; the oracle does not evaluate them.
#define ENB_SHIM_LAB_FUNCTOR(NAME)                                           \
    template <class T>                                                        \
    class NAME {                                                              \
      public:                                                                 \
        typedef TinyVector<T, 3> result_type;                                 \
        NAME() {}                                                             \
        explicit NAME(double) {}                                              \
        template <class V>                                                    \
        result_type operator()(const V&) const                                \
        {                                                                     \
            vigra_fail(#NAME ": not available in the oracle shim");           \
            return result_type();                                             \
        }                                                                     \
    };
ENB_SHIM_LAB_FUNCTOR(RGB2LabFunctor)
ENB_SHIM_LAB_FUNCTOR(RGBPrime2LabFunctor)
#undef ENB_SHIM_LAB_FUNCTOR

inline std::string impexListExtensions() { return "tif tiff"; }

// ---- math utilities ------------------------------------------------------------------------
template <class T>
inline T sq(T v)
{
    return v * v;
}

template <class T>
inline T clip_lower(T t)
{
    return t < T() ? T() : t;
}

inline int roundi(double v) { return v < 0.0 ? (int)(v - 0.5) : (int)(v + 0.5); }

}  // namespace vigra

// Functor expressions, point functors and the in-memory image import/export.
#include "vigra_shim_io.hxx"

// VIGRA's precondition checks are global macros.
using vigra::vigra_fail;
using vigra::vigra_postcondition;
using vigra::vigra_precondition;

#endif

// exposure_weights.cc -- user-defined exposure weight functions for the
// tests of enbgpu-enfuse's --exposure-weight-function=SHARED-OBJECT:SYMBOL
// [:ARGUMENT...]: well-behaved ones and one for each way the front end must
// reject a function.  Built with
//   g++ -std=c++17 -shared -fPIC -I include tests/cpp/exposure_weights.cc
#include <cerrno>
#include <cmath>
#include <cstdlib>

#include "enbgpu_exposure_weight.hpp"

// cos(min(|z|, pi/2))^p with z = (y - optimum) / width and the exponent p
// from the first argument (default 2).
class CosinePower : public ExposureWeight {
  public:
    void initialize(double optimum, double width, argument_const_iterator first, argument_const_iterator last) override
    {
        p_ = 2.0;
        if (first != last) {
            char* tail = nullptr;
            errno = 0;
            p_ = std::strtod(first->c_str(), &tail);
            if (*tail != 0 || errno != 0) {
                throw ExposureWeight::error("exponent is not a number");
            }
            if (p_ <= 0.0 || p_ > 8.0) {
                throw ExposureWeight::error("exponent outside (0, 8]");
            }
        }
        ExposureWeight::initialize(optimum, width, first, last);
    }
    double weight(double y) override
    {
        const double z = std::fabs(normalize(y));
        return z >= 1.5707963267948966 ? 0.0 : std::pow(std::cos(z), p_);
    }

  private:
    double p_ = 2.0;
};

// 1 - |z| / 4 clipped at 0: a tent four widths wide.
class Tent : public ExposureWeight {
  public:
    double weight(double y) override
    {
        const double t = 1.0 - std::fabs(normalize(y)) / 4.0;
        return t > 0.0 ? t : 0.0;
    }
};

struct Negative : public ExposureWeight {
    double weight(double y) override { return y - 0.5; }
};

struct AboveOne : public ExposureWeight {
    double weight(double y) override { return 1.0 + y; }
};

struct AllZero : public ExposureWeight {
    double weight(double) override { return 0.0; }
};

struct OldInterface : public ExposureWeight {
    double weight(double) override { return 0.5; }
    int interface_version() const override { return 1; }
};

CosinePower cosine_power;
Tent tent;
Negative negative;
AboveOne above_one;
AllZero all_zero;
OldInterface old_interface;

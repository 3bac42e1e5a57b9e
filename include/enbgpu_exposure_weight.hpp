/*
 * enbgpu_exposure_weight.hpp -- user-defined exposure weight functions for
 * the enbgpu-enfuse front end (--exposure-weight-function=SHARED-OBJECT:
 * SYMBOL[:ARGUMENT[:...]], src/enfuse.cc:401-410, src/exposure_weight.cc:
 * 44-129).
 *
 * A shared object defines a global object of a class derived from
 * ExposureWeight under the name SYMBOL.  The front end opens the object,
 * checks interface_version(), calls initialize(optimum, width, arguments)
 * with the --exposure-optimum, --exposure-width and the ARGUMENTs that follow
 * SYMBOL, checks the function on 65,536 points of [0, 1] (no weight below 0
 * or above 1, not all zero; src/exposure_weight.cc:237-264), and tabulates
 * weight(g / max) for every sample value g of the images, which the GPU
 * weights then read (enb_enfuse_params.exposure_table).
 *
 * Binary interface: the class below has the members and the virtual
 * functions, in this order, of the reference's ExposureWeight
 * (src/exposure_weight_base.h, interface version 2): initialize, normalize,
 * weight, the destructor, interface_version; data y_optimum, width and the
 * argument list.  So a shared object built for the reference's enfuse loads
 * here unchanged (same compiler and C++ library), and one built against this
 * header loads into the reference's enfuse.
 */
#ifndef ENBGPU_EXPOSURE_WEIGHT_HPP
#define ENBGPU_EXPOSURE_WEIGHT_HPP

#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

#define EXPOSURE_WEIGHT_INTERFACE_VERSION 2

// Full width at half maximum of the Gaussian exposure weight, 2 sqrt(2 ln 2):
// the built-in functions rescale their widths to it.
#define FWHM_GAUSSIAN 2.3548200450309493820231386529193992755

class ExposureWeight {
  public:
    typedef std::vector<std::string> argument_list_t;
    typedef argument_list_t::const_iterator argument_const_iterator;

    ExposureWeight() : optimum_(0.5), width_(0.2) {}
    ExposureWeight(double optimum, double width) : optimum_(optimum), width_(width) { validate(); }

    // Called once after loading with the options' optimum and width and the
    // arguments after SYMBOL; a derived class may rescale the width and must
    // end in this base version.
    virtual void initialize(double optimum, double width, argument_const_iterator first, argument_const_iterator last)
    {
        optimum_ = optimum;
        width_ = width;
        arguments_.assign(first, last);
        validate();
    }

    double optimum() const { return optimum_; }
    double width() const { return width_; }
    const argument_list_t& arguments() const { return arguments_; }

    // (y - optimum) / width, the argument of the bell-shaped functions.
    virtual double normalize(double y) const { return (y - optimum()) / width(); }

    // The weight of normalised luminance y in [0, 1]; must lie in [0, 1].
    virtual double weight(double y) = 0;

    virtual ~ExposureWeight() {}

    // Thrown from initialize() to reject the arguments.
    struct error : public std::runtime_error {
        explicit error(const std::string& message) : std::runtime_error(message) {}
    };

    virtual int interface_version() const { return EXPOSURE_WEIGHT_INTERFACE_VERSION; }

  private:
    void validate() const
    {
        if (optimum_ < 0.0 || optimum_ > 1.0) {
            throw std::invalid_argument("y_optimum");
        }
        if (width_ <= 0.0) {
            throw std::invalid_argument("width_parameter");
        }
    }

    double optimum_;
    double width_;
    argument_list_t arguments_;
};

#endif /* ENBGPU_EXPOSURE_WEIGHT_HPP */

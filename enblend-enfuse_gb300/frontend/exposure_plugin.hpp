// exposure_plugin.hpp -- user-defined exposure weight functions of
// enbgpu-enfuse (--exposure-weight-function=SHARED-OBJECT:SYMBOL[:ARGUMENT
// [:...]], src/exposure_weight.cc:44-129): the shared object's
// ExposureWeight object (enbgpu_exposure_weight.hpp) is opened with dlopen,
// checked as the reference checks it (interface version, initialize's
// exceptions, weights in [0, 1] and not all zero on 65,536 points,
// src/exposure_weight.cc:237-264, src/enfuse.cc:1913-1945), and tabulated
// at y = g / max for the images' sample values, the table enb_enfuse reads.
#pragma once

#include <dlfcn.h>

#include <cstdint>
#include <limits>
#include <string>
#include <vector>

#include "cli_common.hpp"
#include "enbgpu_exposure_weight.hpp"

namespace enbfront {

struct UserWeightFunction {
    std::string library, symbol;
    std::vector<std::string> arguments;
    ExposureWeight* fn = nullptr;  // owned by the shared object, which stays loaded

    bool loaded() const { return fn != nullptr; }

    // dlopen / dlsym, the interface version and initialize(optimum, width,
    // arguments); errors carry the reference's wording.
    void load(const std::string& command, double optimum, double width)
    {
        void* handle = dlopen(library.c_str(), RTLD_LAZY);
        if (!handle) {
            const char* e = dlerror();
            throw UsageError("cannot load exposure weight function from \"" + library + "\": " + (e ? e : "?"));
        }
        dlerror();
        void* sym = dlsym(handle, symbol.c_str());
        const char* e = dlerror();
        if (e || !sym) {
            throw UsageError("symbol \"" + symbol + "\" not found in shared object \"" + library + "\"" +
                             (e ? std::string(": ") + e : std::string()));
        }
        fn = static_cast<ExposureWeight*>(sym);
        const int version = fn->interface_version();
        if (version != EXPOSURE_WEIGHT_INTERFACE_VERSION) {
            fn = nullptr;
            throw UsageError("user-defined weight function \"" + symbol + "\"\n" + command +
                             ": defined in shared object \"" + library + "\"\n" + command +
                             ": matches interface version " + std::to_string(version) + ", but " + command +
                             " requires version " + std::to_string(EXPOSURE_WEIGHT_INTERFACE_VERSION));
        }
        try {
            fn->initialize(optimum, width, arguments.begin(), arguments.end());
        } catch (const std::exception& x) {
            fn = nullptr;
            throw UsageError("user-defined weight function \"" + symbol + "\"\n" + command +
                             ": defined in shared object \"" + library + "\"\n" + command +
                             ": raised exception: " + x.what());
        }
    }

    // check_weight_function with n points (src/exposure_weight.cc:237-264):
    // "" when usable, else the reference's note.
    std::string check(int n = 65536) const
    {
        int zeros = 0;
        for (int i = 0; i < n; ++i) {
            const double y = (double)i / (double)(n - 1);
            const double w = fn->weight(y);
            if (w < 0.0) {
                return "at least one weight is negative";
            }
            if (w > 1.0) {
                return "at least one weight is larger than one";
            }
            if (w >= 0.0 && w <= std::numeric_limits<double>::denorm_min()) {
                ++zeros;
            }
        }
        return zeros == n ? "too many zeros" : "";
    }

    // weight(g / max) for g = 0..max, the ExposureFunctor's argument
    // (src/enfuse.h:638) for every sample value.
    std::vector<double> table(uint32_t maxv) const
    {
        std::vector<double> t((size_t)maxv + 1);
        for (uint32_t g = 0; g <= maxv; ++g) {
            t[g] = fn->weight((double)g / (double)maxv);
        }
        return t;
    }
};

}  // namespace enbfront

// enfuse_main.cpp -- the enfuse command line over the GB300 path.
//
// Parses the weighting and pyramid options of the reference's enfuse
// (src/enfuse.cc:934-980 option table, :1100-1760 their meaning and ranges),
// reads the images (TIFF or .npy, all of the union's size), runs enb_enfuse
// with host buffers and writes the result with its alpha band as the
// reference's checkpoint does.  Options of the reference that this build does
// not provide (GPU/OpenCL selection, ICC colour spaces, layer selection,
// expert parameters, edge-scale contrast, OpenCL weight functions) are
// rejected with a message instead of being ignored.  User-defined exposure
// weight functions in shared objects are loaded, checked and tabulated for
// the images' sample values (exposure_plugin.hpp).
//
// --dry-run (this front end's own option) prints the parsed settings as JSON
// and exits without touching the GPU.
#include <cuda_runtime.h>
#include <getopt.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <regex>
#include <sstream>
#include <string>
#include <vector>

#include "cli_common.hpp"
#include "enbgpu.h"
#include "exposure_plugin.hpp"
#include "image_io.hpp"

using namespace enbfront;

namespace {

const char* kCommand = "enbgpu-enfuse";

struct Settings {
    enb_enfuse_params prm{};
    enb_fuse_options opt{};
    std::string output = "a.tif";
    std::string soft_template = "softmask-%n.tif";
    std::string hard_template = "hardmask-%n.tif";
    bool save_masks = false, load_masks = false, dry_run = false;
    std::string depth;  // "" = the input's
    int verbose = 0;
    std::vector<std::string> inputs;
    std::string exp_fn_name = "gaussian";
    UserWeightFunction user_fn;  // library set: a user-defined exposure weight function
    std::vector<double> exp_table;
};

void usage()
{
    std::cout <<
        "Usage: " << kCommand << " [options] -o OUTPUT INPUT...\n"
        "Fuse exposures with enfuse's weights and multiresolution blend on a GB300.\n"
        "Images: uncompressed TIFF or .npy (uint8, uint16, float32), all of one size.\n"
        "  -o, --output=FILE                output image (default a.tif)\n"
        "  -l, --levels=LEVELS              pyramid levels: 1..29, -N fewer than automatic, auto\n"
        "  -w, --wrap[=MODE]                periodic in x (none, horizontal; vertical and both wrap in x)\n"
        "  -d, --depth=DEPTH                output depth: the input's (8, 16, float)\n"
        "      --exposure-weight=W          default 1.0\n"
        "      --saturation-weight=W        default 0.0\n"
        "      --contrast-weight=W          default 0.0\n"
        "      --entropy-weight=W           default 0.0\n"
        "      --exposure-optimum=O         default 0.5\n"
        "      --exposure-width=W           default 0.2\n"
        "      --exposure-weight-function=F gaussian, lorentzian, half-sine, full-sine, bi-square,\n"
        "                                   or SHARED-OBJECT:SYMBOL[:ARGUMENT[:...]]\n"
        "      --exposure-cutoff=L[:U[:LP[:UP]]]   values or percentages, projectors\n"
        "      --contrast-window-size=N     odd, >= 3 (default 5)\n"
        "      --entropy-window-size=N      odd, >= 3 (default 3)\n"
        "      --entropy-cutoff=L[:U]       values or percentages\n"
        "      --gray-projector=P           average, value, anti-value, lightness, luminance,\n"
        "                                   channel-mixer:R:G:B\n"
        "      --hard-mask / --soft-mask\n"
        "      --save-masks[=SOFT[:HARD]]   weight masks (default softmask-%n.tif, hardmask-%n.tif)\n"
        "      --load-masks[=SOFT[:HARD]]   use saved masks instead of computing the weights\n"
        "      --blend-colorspace=identity  the only colour space of this build\n"
        "      --dry-run                    print the parsed settings and exit\n"
        "  -v, --verbose, -h, --help, -V, --version\n";
}

// numberOfString's clamping (src/common.h:345-456): values outside the range
// are replaced by the bound, with a warning.
double bounded(const std::string& opt, const char* arg, double lo, double hi)
{
    double v = number(opt, arg);
    if (v < lo) {
        std::cerr << kCommand << ": warning: " << opt << " less than " << lo << "; will use " << lo << "\n";
        v = lo;
    }
    if (v > hi) {
        std::cerr << kCommand << ": warning: " << opt << " greater than " << hi << "; will use " << hi << "\n";
        v = hi;
    }
    return v;
}

void mask_templates(const char* arg, std::string& soft, std::string& hard)
{
    if (!arg || !*arg) {
        return;
    }
    const std::regex delim("[,;:]");  // PATH_OPTION_DELIMITERS_REGEX, src/common.h:47
    const std::string a(arg);
    std::sregex_token_iterator t(a.begin(), a.end(), delim, -1), e;
    if (t != e) {
        soft = t->str();
        ++t;
    }
    if (t != e) {
        hard = t->str();
    }
}

// The built-in exposure weight functions (src/exposure_weight.cc:139-163);
// -1 for any other name.
int builtin_exposure_function(const std::string& name)
{
    const std::string n = lower(name);
    if (n == "gauss" || n == "gaussian") return ENB_EXP_GAUSSIAN;
    if (n == "lorentz" || n == "lorentzian") return ENB_EXP_LORENTZIAN;
    if (n == "halfsine" || n == "half-sine") return ENB_EXP_HALF_SINE;
    if (n == "fullsine" || n == "full-sine") return ENB_EXP_FULL_SINE;
    if (n == "bisquare" || n == "bi-square") return ENB_EXP_BISQUARE;
    return -1;
}

// --exposure-weight-function NAME[:SYMBOL[:ARGUMENT...]], split at the path
// delimiters ",;:" (src/enfuse.cc:1524-1560): a built-in NAME, else the shared
// object NAME with the weight object SYMBOL and its arguments.
void exposure_function_option(Settings& s, const std::string& arg)
{
    const std::regex delim("[,;:]");  // PATH_OPTION_DELIMITERS_REGEX, src/common.h:47
    std::vector<std::string> t;
    for (std::sregex_token_iterator i(arg.begin(), arg.end(), delim, -1), e; i != e; ++i) {
        t.push_back(i->str());
    }
    if (t.empty() || t[0].empty()) {
        throw UsageError("option \"--exposure-weight-function\" requires an argument");
    }
    s.exp_fn_name = t[0];
    s.user_fn = UserWeightFunction{};
    const int builtin = builtin_exposure_function(t[0]);
    if (builtin >= 0) {
        s.prm.exp_function = builtin;
        return;
    }
    if (t.size() < 2) {
        // built-in functions take no arguments, so a lone name must be one
        throw UsageError("unknown built-in exposure weight function \"" + t[0] + "\"");
    }
    s.user_fn.library = t[0];
    s.user_fn.symbol = t[1];
    s.user_fn.arguments.assign(t.begin() + 2, t.end());
}

Settings parse(int argc, char** argv)
{
    Settings s;
    enb_default_enfuse_params(&s.prm);
    enb_default_fuse_options(&s.opt);
    s.opt.host_buffers = 1;
    enum {
        kExpW = 1000, kSatW, kConW, kEntW, kExpOpt, kExpWidth, kExpFn, kExpCut, kConWin, kEntWin, kEntCut, kGray,
        kHard, kSoft, kSave, kLoad, kBlendCs, kDry, kUnsupported, kMinCurv, kEdge, kCompression
    };
    static struct option longopts[] = {
        {"exposure-weight", required_argument, 0, kExpW},
        {"saturation-weight", required_argument, 0, kSatW},
        {"contrast-weight", required_argument, 0, kConW},
        {"entropy-weight", required_argument, 0, kEntW},
        {"exposure-optimum", required_argument, 0, kExpOpt},
        {"exposure-width", required_argument, 0, kExpWidth},
        {"exposure-weight-function", required_argument, 0, kExpFn},
        {"exposure-cutoff", required_argument, 0, kExpCut},
        {"contrast-window-size", required_argument, 0, kConWin},
        {"entropy-window-size", required_argument, 0, kEntWin},
        {"entropy-cutoff", required_argument, 0, kEntCut},
        {"gray-projector", required_argument, 0, kGray},
        {"hard-mask", no_argument, 0, kHard},
        {"soft-mask", no_argument, 0, kSoft},
        {"save-masks", optional_argument, 0, kSave},
        {"save-mask", optional_argument, 0, kSave},
        {"load-masks", optional_argument, 0, kLoad},
        {"load-mask", optional_argument, 0, kLoad},
        {"blend-colorspace", required_argument, 0, kBlendCs},
        {"blend-color-space", required_argument, 0, kBlendCs},
        {"contrast-min-curvature", required_argument, 0, kMinCurv},
        {"contrast-edge-scale", required_argument, 0, kEdge},
        {"compression", required_argument, 0, kCompression},
        {"levels", required_argument, 0, 'l'},
        {"wrap", optional_argument, 0, 'w'},
        {"depth", required_argument, 0, 'd'},
        {"output", required_argument, 0, 'o'},
        {"verbose", optional_argument, 0, 'v'},
        {"help", no_argument, 0, 'h'},
        {"version", no_argument, 0, 'V'},
        {"dry-run", no_argument, 0, kDry},
        // options of the reference that this build does not provide
        {"gpu", no_argument, 0, kUnsupported},
        {"no-gpu", no_argument, 0, kUnsupported},
        {"prefer-gpu", required_argument, 0, kUnsupported},
        {"preferred-gpu", required_argument, 0, kUnsupported},
        {"output-mask", optional_argument, 0, kUnsupported},
        {"fallback-profile", required_argument, 0, kUnsupported},
        {"layer-selector", required_argument, 0, kUnsupported},
        {"parameter", required_argument, 0, kUnsupported},
        {"no-parameter", required_argument, 0, kUnsupported},
        {"show-image-formats", no_argument, 0, kUnsupported},
        {"show-signature", no_argument, 0, kUnsupported},
        {"show-globbing-algorithms", no_argument, 0, kUnsupported},
        {"show-software-components", no_argument, 0, kUnsupported},
        {"show-gpu-info", no_argument, 0, kUnsupported},
        {0, 0, 0, 0}};
    // projectors of the exposure cutoff: anti-value / value unless given
    // (src/enfuse.cc:126-127, 1322-1330)
    std::string lower_proj = "anti-value", upper_proj = "value", gray_name;
    bool lower_given = false, upper_given = false;
    opterr = 0;
    optind = 1;
    int c, idx = 0;
    while ((c = getopt_long(argc, argv, ":l:w::d:o:v::hVf:", longopts, &idx)) != -1) {
        const std::string name = c >= 1000 ? std::string("--") + longopts[idx].name : std::string("-") + (char)c;
        switch (c) {
        case kExpW: s.prm.w_exposure = bounded(name, optarg, 0.0, 1.0); break;
        case kSatW: s.prm.w_saturation = bounded(name, optarg, 0.0, 1.0); break;
        case kConW: s.prm.w_contrast = bounded(name, optarg, 0.0, 1.0); break;
        case kEntW: s.prm.w_entropy = bounded(name, optarg, 0.0, 1.0); break;
        case kExpOpt: s.prm.exp_optimum = bounded(name, optarg, 0.0, 1.0); break;
        case kExpWidth: {
            const double v = number(name, optarg);
            if (v <= 0.0) {
                throw UsageError("exposure width must be positive");
            }
            s.prm.exp_width = v;
            break;
        }
        case kExpFn: exposure_function_option(s, optarg); break;
        case kExpCut: {
            const std::vector<std::string> t = split_numeric(optarg);
            if (t.empty() || t[0].empty()) {
                throw UsageError("no value given to \"--exposure-cutoff\"; lower cutoff is required");
            }
            cutoff_value(name, t[0], s.prm.exp_cutoff_lower, s.prm.exp_cutoff_lower_pct);
            if (t.size() > 1) {
                cutoff_value(name, t[1], s.prm.exp_cutoff_upper, s.prm.exp_cutoff_upper_pct);
            }
            if (t.size() > 2) {
                lower_proj = t[2];
                lower_given = true;
            }
            if (t.size() > 3) {
                upper_proj = t[3];
                upper_given = true;
            }
            if (t.size() > 4) {
                std::cerr << kCommand << ": warning: ignoring trailing garbage in \"--exposure-cutoff\"\n";
            }
            break;
        }
        case kConWin: {
            int v = integer(name, optarg);
            if (v < 3) {
                std::cerr << kCommand << ": warning: contrast window size too small; will use size = 3\n";
                v = 3;
            }
            if (v % 2 == 0) {
                std::cerr << kCommand << ": warning: contrast window size is even; increasing size to next odd number\n";
                ++v;
            }
            s.prm.contrast_window = v;
            break;
        }
        case kEntWin: {
            int v = integer(name, optarg);
            if (v < 3) {
                std::cerr << kCommand << ": warning: entropy window size too small; will use size = 3\n";
                v = 3;
            }
            if (v % 2 == 0) {
                std::cerr << kCommand << ": warning: entropy window size is even; increasing size to next odd number\n";
                ++v;
            }
            s.prm.entropy_window = v;
            break;
        }
        case kEntCut: {
            const std::vector<std::string> t = split_numeric(optarg);
            if (t.empty() || t[0].empty()) {
                throw UsageError("no scale given to \"--entropy-cutoff\"; lower cutoff is required");
            }
            cutoff_value(name, t[0], s.prm.ent_cutoff_lower, s.prm.ent_cutoff_lower_pct);
            if (t.size() > 1) {
                cutoff_value(name, t[1], s.prm.ent_cutoff_upper, s.prm.ent_cutoff_upper_pct);
            }
            break;
        }
        case kGray:
            s.prm.gray_projector = gray_projector(optarg, s.prm.mixer);
            gray_name = optarg;
            break;
        case kHard: s.opt.hard_mask = 1; break;
        case kSoft: s.opt.hard_mask = 0; break;
        case kSave:
            s.save_masks = true;
            mask_templates(optarg, s.soft_template, s.hard_template);
            break;
        case kLoad:
            s.load_masks = true;
            mask_templates(optarg, s.soft_template, s.hard_template);
            break;
        case kBlendCs:
            if (lower(optarg) != "identity" && lower(optarg) != "id" && lower(optarg) != "unit") {
                throw UsageError("blend colour space \"" + std::string(optarg) +
                                 "\" needs ICC profiles, which this build does not support (use identity)");
            }
            break;
        case kMinCurv:
        case kEdge:
            if (number(name, std::string(optarg).substr(0, std::string(optarg).find_first_of(";:/%"))) != 0.0) {
                throw UsageError(name + " (edge-scale contrast) is not supported by this build");
            }
            break;
        case kCompression:
            if (lower(optarg) != "none") {
                throw UsageError("only uncompressed output is supported (--compression=none)");
            }
            break;
        case 'l': s.opt.levels = levels_arg(optarg); break;
        case 'w': s.opt.wrap = wrap_mode(optarg ? optarg : ""); break;
        case 'd': s.depth = lower(optarg); break;
        case 'o': s.output = optarg; break;
        case 'v': s.verbose = optarg ? integer("--verbose", optarg) : s.verbose + 1; break;
        case 'h': usage(); std::exit(0);
        case 'V': std::cout << kCommand << " (GB300 enfuse path, ABI " << ENBGPU_ABI_VERSION << ")\n"; std::exit(0);
        case kDry: s.dry_run = true; break;
        case 'f':
        case kUnsupported:
            throw UsageError("option " + name + " is not supported by this build");
        case ':': throw UsageError(std::string("option ") + argv[optind - 1] + " requires an argument");
        default: throw UsageError(std::string("unknown option ") + argv[optind - 1]);
        }
    }
    // an empty lower projector name stands for --gray-projector, an empty
    // upper one for the lower one's name (src/enfuse.h:982-986)
    const std::string lname = lower_proj.empty() ? gray_name : lower_proj;
    const std::string uname = upper_proj.empty() ? lower_proj : upper_proj;
    double junk[3] = {0.0, 0.0, 0.0};
    if (lower_given || upper_given) {
        s.prm.exp_cutoff_lower_projector = gray_projector(lname, lname == gray_name ? s.prm.mixer : junk);
        s.prm.exp_cutoff_upper_projector =
            gray_projector(uname.empty() ? gray_name : uname, (uname.empty() || uname == gray_name) ? s.prm.mixer : junk);
        if ((s.prm.exp_cutoff_lower_projector == ENB_GRAY_MIXER || s.prm.exp_cutoff_upper_projector == ENB_GRAY_MIXER) &&
            s.prm.gray_projector != ENB_GRAY_MIXER) {
            throw UsageError("a channel-mixer cutoff projector needs --gray-projector=channel-mixer with the same "
                             "weights in this build");
        }
    }
    for (int i = optind; i < argc; ++i) {
        s.inputs.push_back(argv[i]);
    }
    if (s.inputs.empty()) {
        throw UsageError("no input files specified");
    }
    if (!s.user_fn.library.empty() && s.prm.w_exposure > 0.0) {
        // loaded and checked once all options are known (src/enfuse.cc:1913-1945)
        s.user_fn.load(kCommand, s.prm.exp_optimum, s.prm.exp_width);
        const std::string note = s.user_fn.check();
        if (!note.empty()) {
            throw UsageError("unusable exposure weight function \"" + s.exp_fn_name + "\"\n" + kCommand +
                             ": note: " + note);
        }
    }
    return s;
}

std::string cutoff_json(double v, int pct) { return "[" + std::to_string(v) + ", " + (pct ? "true" : "false") + "]"; }

void print_json(const Settings& s)
{
    const enb_enfuse_params& p = s.prm;
    std::ostringstream o;
    o << "{\"w_exposure\": " << p.w_exposure << ", \"w_saturation\": " << p.w_saturation
      << ", \"w_contrast\": " << p.w_contrast << ", \"w_entropy\": " << p.w_entropy
      << ", \"exp_optimum\": " << p.exp_optimum << ", \"exp_width\": " << p.exp_width
      << ", \"exp_function\": " << p.exp_function << ", \"contrast_window\": " << p.contrast_window
      << ", \"entropy_window\": " << p.entropy_window << ", \"gray_projector\": " << p.gray_projector
      << ", \"mixer\": [" << p.mixer[0] << ", " << p.mixer[1] << ", " << p.mixer[2] << "]"
      << ", \"exp_cutoff\": [" << cutoff_json(p.exp_cutoff_lower, p.exp_cutoff_lower_pct) << ", "
      << cutoff_json(p.exp_cutoff_upper, p.exp_cutoff_upper_pct) << "]"
      << ", \"exp_cutoff_projectors\": [" << p.exp_cutoff_lower_projector << ", " << p.exp_cutoff_upper_projector << "]"
      << ", \"ent_cutoff\": [" << cutoff_json(p.ent_cutoff_lower, p.ent_cutoff_lower_pct) << ", "
      << cutoff_json(p.ent_cutoff_upper, p.ent_cutoff_upper_pct) << "]"
      << ", \"levels\": " << s.opt.levels << ", \"wrap\": " << s.opt.wrap << ", \"hard_mask\": " << s.opt.hard_mask
      << ", \"save_masks\": " << (s.save_masks ? "true" : "false") << ", \"load_masks\": "
      << (s.load_masks ? "true" : "false") << ", \"soft_template\": \"" << s.soft_template << "\", \"hard_template\": \""
      << s.hard_template << "\", \"output\": \"" << s.output << "\", \"inputs\": " << s.inputs.size();
    if (s.user_fn.loaded()) {
        // the loaded function's library, symbol, arguments and weights at y = 0, 1/4, 1/2, 3/4, 1
        o << ", \"user_weight\": {\"library\": \"" << s.user_fn.library << "\", \"symbol\": \"" << s.user_fn.symbol
          << "\", \"arguments\": [";
        for (size_t i = 0; i < s.user_fn.arguments.size(); ++i) {
            o << (i ? ", " : "") << "\"" << s.user_fn.arguments[i] << "\"";
        }
        o << "], \"samples\": [";
        o.precision(17);
        for (int i = 0; i <= 4; ++i) {
            o << (i ? ", " : "") << s.user_fn.fn->weight(i / 4.0);
        }
        o << "]}";
    }
    o << "}";
    std::cout << o.str() << std::endl;
}

int run(Settings& s)
{
    std::vector<Image> imgs;
    for (const std::string& f : s.inputs) {
        imgs.push_back(read_image(f));
        const Image& a = imgs.front();
        const Image& b = imgs.back();
        if (b.width != a.width || b.height != a.height || b.type != a.type || b.samples != a.samples) {
            throw UsageError(f + ": all images need the same size, sample type and samples a pixel "
                             "(this front end does not assemble images at offsets)");
        }
        if (b.samples - b.extra != 1 && b.samples - b.extra != 3) {
            throw UsageError(f + ": gray or RGB images (optionally with alpha) expected");
        }
    }
    const Image& first = imgs.front();
    if (!s.depth.empty()) {
        const std::string want = first.type == SampleType::U8 ? "8" : (first.type == SampleType::U16 ? "16" : "float");
        if (!(s.depth == want || (want == "8" && s.depth == "uint8") || (want == "16" && s.depth == "uint16") ||
              (want == "float" && (s.depth == "32" || s.depth == "r32")))) {
            throw UsageError("--depth=" + s.depth + ": this build writes the input's depth (" + want + ") only");
        }
    }
    const int K = (int)imgs.size(), w = first.width, h = first.height;
    const int C = first.samples - first.extra >= 3 ? 3 : 1;
    if (s.user_fn.loaded()) {
        if (first.type == SampleType::F32) {
            throw UsageError("user-defined exposure weight functions are tabulated for 8- and 16-bit images; "
                             "this build has none for float images");
        }
        s.exp_table = s.user_fn.table(first.type == SampleType::U8 ? 255u : 65535u);
        s.prm.exposure_table = s.exp_table.data();
        s.prm.exposure_table_size = (int32_t)s.exp_table.size();
    }
    enb_ctx* ctx = nullptr;
    check(nullptr, enb_create(0, &ctx), "enb_create");
    std::vector<enb_image> di;
    for (Image& im : imgs) {
        di.push_back(pixel_desc(im));
    }
    std::vector<std::vector<float>> masks;
    std::vector<enb_image> dm;
    if (s.load_masks) {
        // --load-masks: soft (or, with the hard mask, hard) masks replace the
        // weights (src/enfuse.h:1288-1331)
        for (int k = 0; k < K; ++k) {
            const std::string f = expand_template(s.opt.hard_mask ? s.hard_template : s.soft_template, K, k);
            Image m = read_image(f);
            if (m.samples != 1) {
                throw UsageError("mask image \"" + f + "\" is not grayscale or has an alpha channel");
            }
            if (m.width != w || m.height != h) {
                throw UsageError("mask in \"" + f + "\" does not have the size of the images");
            }
            std::vector<float> v((size_t)w * h);
            for (size_t i = 0; i < v.size(); ++i) {
                v[i] = m.type == SampleType::F32 ? reinterpret_cast<const float*>(m.data.data())[i]
                       : m.type == SampleType::U16 ? (float)reinterpret_cast<const uint16_t*>(m.data.data())[i]
                                                    : (float)m.data[i];
            }
            masks.push_back(std::move(v));
        }
    } else if (s.save_masks) {
        // --save-masks: the weights of each image (enfuseMask; the soft masks
        // the reference saves, src/enfuse.h:1336-1370) are computed first and
        // then passed as loaded masks, so that they are computed once
        for (int k = 0; k < K; ++k) {
            std::vector<float> v((size_t)w * h);
            void* dimg = nullptr;
            void* dw = nullptr;
            const size_t ib = imgs[k].data.size();
            if (cudaMalloc(&dimg, ib) != cudaSuccess || cudaMalloc(&dw, v.size() * 4) != cudaSuccess ||
                cudaMemcpy(dimg, imgs[k].data.data(), ib, cudaMemcpyHostToDevice) != cudaSuccess) {
                throw std::runtime_error("device buffers for the weights");
            }
            enb_image src = di[k];
            src.data = dimg;
            enb_image out = plane_desc(dw, w, h, (int64_t)w * 4, ENB_F32);
            check(ctx, enb_enfuse_mask(ctx, &s.prm, &src, nullptr, &out), "enb_enfuse_mask");
            if (cudaMemcpy(v.data(), dw, v.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
                throw std::runtime_error("copying the weights back");
            }
            cudaFree(dimg);
            cudaFree(dw);
            masks.push_back(std::move(v));
        }
        std::vector<std::vector<float>> saved = masks;
        if (s.opt.hard_mask) {
            // the hard masks (src/enfuse.h:1399-1442): 255 for the largest
            // weight, 0 for the others, 255/K where every weight is 0
            for (size_t p = 0; p < (size_t)w * h; ++p) {
                float mx = 0.0f;
                int mi = 0;
                for (int k = 0; k < K; ++k) {
                    if (masks[k][p] > mx) {
                        mx = masks[k][p];
                        mi = k;
                    }
                }
                for (int k = 0; k < K; ++k) {
                    saved[k][p] = mx == 0.0f ? 255.0f / (float)K : (k == mi ? 255.0f : 0.0f);
                }
            }
        }
        for (int k = 0; k < K; ++k) {
            Image m;
            m.width = w;
            m.height = h;
            m.samples = 1;
            m.type = SampleType::F32;
            m.data.resize((size_t)w * h * 4);
            std::memcpy(m.data.data(), saved[k].data(), m.data.size());
            write_image(expand_template(s.opt.hard_mask ? s.hard_template : s.soft_template, K, k), m);
        }
    }
    for (std::vector<float>& v : masks) {
        dm.push_back(plane_desc(v.data(), w, h, (int64_t)w * 4, ENB_F32));
    }
    Image colour = first;  // the output's colour samples (and alpha band if the inputs had one)
    std::vector<uint8_t> alpha((size_t)w * h);
    enb_image dout = pixel_desc(colour);
    enb_image da = plane_desc(alpha.data(), w, h, w, ENB_U8);
    const bool computed_masks = s.save_masks && !s.load_masks;
    check(ctx,
          enb_enfuse(ctx, &s.prm, K, di.data(), nullptr, (s.load_masks || computed_masks) ? dm.data() : nullptr,
                     &dout, &da, &s.opt),
          "enb_enfuse");
    enb_destroy(ctx);
    write_image(s.output, with_alpha(colour, C, alpha));
    if (s.verbose) {
        std::cerr << kCommand << ": info: wrote \"" << s.output << "\" (" << w << "x" << h << ", " << K
                  << " exposures)\n";
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    try {
        Settings s = parse(argc, argv);
        if (s.dry_run) {
            print_json(s);
            return 0;
        }
        return run(s);
    } catch (const UsageError& e) {
        std::cerr << kCommand << ": " << e.what() << "\n";
        return 1;
    } catch (const std::exception& e) {
        std::cerr << kCommand << ": " << e.what() << "\n";
        return 1;
    }
}

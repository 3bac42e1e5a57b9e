// enblend_main.cpp -- the enblend command line over the GB300 path.
//
// The reference blends its inputs one after another into the accumulated
// result under seam masks (src/enblend.h:56-560).  The masks come from files
// (--load-masks, src/mask.h:1002-1063: mask i, template "%n" = i + 1,
// default mask-%n.tif, 8-bit gray, 255 where the new image wins, blends
// input i + 1 into the result of inputs 0..i), or, with --fine-mask
// --no-optimize, from the nearest-feature transform of the two footprints on
// the GPU (enb_nft_mask; the reference's mask for those options,
// src/mask.h:1101-1180); --save-masks writes them.  The coarse masks and the
// seam optimisers (vectorised seams, annealing, Dijkstra, graph cut) are not
// part of this build.  All images share the union canvas (RGBA with the
// footprint in the alpha band, or RGB).  The pyramid options (--levels,
// --wrap, --depth, --output) are the reference's (src/enblend.cc:780-860);
// the other seam-generation, colour-space and GPU options are rejected with
// a message.
//
// --dry-run (this front end's own option) prints the parsed settings as JSON
// and exits without touching the GPU.
#include <getopt.h>

#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "cli_common.hpp"
#include "enbgpu.h"
#include "image_io.hpp"

using namespace enbfront;

namespace {

const char* kCommand = "enbgpu-enblend";

struct Settings {
    enb_fuse_options opt{};
    std::string output = "a.tif";
    std::string mask_template = "mask-%n.tif";  // src/enblend.cc:140-142
    bool load_masks = false, save_masks = false, dry_run = false;
    bool coarse_mask = true, optimize = true;   // the reference's defaults (src/enblend.cc:133, 136)
    std::string depth;
    int verbose = 0;
    std::vector<std::string> inputs;
};

void usage()
{
    std::cout <<
        "Usage: " << kCommand << " [options] --load-masks[=TEMPLATE] -o OUTPUT INPUT...\n"
        "Blend images on one canvas under given seam masks (multiresolution spline) on a GB300.\n"
        "  -o, --output=FILE          output image (default a.tif)\n"
        "  -l, --levels=LEVELS        pyramid levels: 1..29, -N fewer than automatic, auto\n"
        "  -w, --wrap[=MODE]          periodic in x (none, horizontal; vertical and both wrap in x)\n"
        "  -d, --depth=DEPTH          output depth: the input's (8, 16, float)\n"
        "      --load-masks[=TEMPLATE] seam masks (default mask-%n.tif): mask i blends input i+1\n"
        "      --fine-mask --no-optimize  seams from the nearest-feature transform (on the GPU)\n"
        "      --save-masks[=TEMPLATE] write the generated seam masks\n"
        "      --dry-run              print the parsed settings and exit\n"
        "  -v, --verbose, -h, --help, -V, --version\n";
}

Settings parse(int argc, char** argv)
{
    Settings s;
    enb_default_fuse_options(&s.opt);
    s.opt.host_buffers = 1;
    enum { kLoad = 1000, kDry, kUnsupported, kBlendCs, kCompression, kSave, kFine, kCoarse, kOpt, kNoOpt };
    static struct option longopts[] = {
        {"load-masks", optional_argument, 0, kLoad},
        {"load-mask", optional_argument, 0, kLoad},
        {"levels", required_argument, 0, 'l'},
        {"wrap", optional_argument, 0, 'w'},
        {"depth", required_argument, 0, 'd'},
        {"output", required_argument, 0, 'o'},
        {"verbose", optional_argument, 0, 'v'},
        {"help", no_argument, 0, 'h'},
        {"version", no_argument, 0, 'V'},
        {"dry-run", no_argument, 0, kDry},
        {"blend-colorspace", required_argument, 0, kBlendCs},
        {"blend-color-space", required_argument, 0, kBlendCs},
        {"compression", required_argument, 0, kCompression},
        {"save-masks", optional_argument, 0, kSave},
        {"save-mask", optional_argument, 0, kSave},
        {"fine-mask", no_argument, 0, kFine},
        {"coarse-mask", optional_argument, 0, kCoarse},
        {"optimize", no_argument, 0, kOpt},
        {"no-optimize", no_argument, 0, kNoOpt},
        // seam generation, mask output and GPU selection of the reference
        {"primary-seam-generator", required_argument, 0, kUnsupported},
        {"image-difference", required_argument, 0, kUnsupported},
        {"anneal", required_argument, 0, kUnsupported},
        {"dijkstra", required_argument, 0, kUnsupported},
        {"mask-vectorize", required_argument, 0, kUnsupported},
        {"optimizer-weights", required_argument, 0, kUnsupported},
        {"smooth-difference", required_argument, 0, kUnsupported},
        {"gpu", no_argument, 0, kUnsupported},
        {"no-gpu", no_argument, 0, kUnsupported},
        {"output-mask", optional_argument, 0, kUnsupported},
        {"fallback-profile", required_argument, 0, kUnsupported},
        {"layer-selector", required_argument, 0, kUnsupported},
        {"parameter", required_argument, 0, kUnsupported},
        {"no-parameter", required_argument, 0, kUnsupported},
        {"pre-assemble", no_argument, 0, kUnsupported},
        {"no-pre-assemble", no_argument, 0, kUnsupported},
        {"stop-after-mask-generation", no_argument, 0, kUnsupported},
        {0, 0, 0, 0}};
    opterr = 0;
    optind = 1;
    int c, idx = 0;
    while ((c = getopt_long(argc, argv, ":l:w::d:o:v::hVaf:x", longopts, &idx)) != -1) {
        const std::string name = c >= 1000 ? std::string("--") + longopts[idx].name : std::string("-") + (char)c;
        switch (c) {
        case kLoad:
            s.load_masks = true;
            if (optarg && *optarg) {
                s.mask_template = optarg;
            }
            break;
        case kSave:
            s.save_masks = true;
            if (optarg && *optarg) {
                s.mask_template = optarg;
            }
            break;
        case kFine: s.coarse_mask = false; break;
        case kCoarse: s.coarse_mask = true; break;
        case kOpt: s.optimize = true; break;
        case kNoOpt: s.optimize = false; break;
        case 'l': s.opt.levels = levels_arg(optarg); break;
        case 'w': s.opt.wrap = wrap_mode(optarg ? optarg : ""); break;
        case 'd': s.depth = lower(optarg); break;
        case 'o': s.output = optarg; break;
        case 'v': s.verbose = optarg ? integer("--verbose", optarg) : s.verbose + 1; break;
        case 'h': usage(); std::exit(0);
        case 'V': std::cout << kCommand << " (GB300 enblend path, ABI " << ENBGPU_ABI_VERSION << ")\n"; std::exit(0);
        case kDry: s.dry_run = true; break;
        case kBlendCs:
            if (lower(optarg) != "identity" && lower(optarg) != "id" && lower(optarg) != "unit") {
                throw UsageError("blend colour space \"" + std::string(optarg) +
                                 "\" needs ICC profiles, which this build does not support (use identity)");
            }
            break;
        case kCompression:
            if (lower(optarg) != "none") {
                throw UsageError("only uncompressed output is supported (--compression=none)");
            }
            break;
        case 'a':
        case 'f':
        case 'x':
        case kUnsupported:
            throw UsageError("option " + name + " is not supported by this build (no seam generation; "
                             "give the seam masks with --load-masks)");
        case ':': throw UsageError(std::string("option ") + argv[optind - 1] + " requires an argument");
        default: throw UsageError(std::string("unknown option ") + argv[optind - 1]);
        }
    }
    for (int i = optind; i < argc; ++i) {
        s.inputs.push_back(argv[i]);
    }
    if (s.inputs.size() < 2) {
        throw UsageError("at least two input images are needed");
    }
    if (!s.load_masks && (s.coarse_mask || s.optimize)) {
        throw UsageError("this build generates seams only with --fine-mask --no-optimize (the nearest-feature "
                         "transform); coarse masks and seam optimisation are not supported: give "
                         "--fine-mask --no-optimize, or the seam masks with --load-masks");
    }
    if (s.load_masks && s.save_masks) {
        throw UsageError("--load-masks and --save-masks exclude each other");
    }
    return s;
}

int run(Settings& s)
{
    std::vector<Image> imgs;
    for (const std::string& f : s.inputs) {
        imgs.push_back(read_image(f));
        const Image& a = imgs.front();
        const Image& b = imgs.back();
        if (b.width != a.width || b.height != a.height || b.type != a.type || b.samples != a.samples) {
            throw UsageError(f + ": all images need the canvas size, sample type and samples a pixel of the first");
        }
        if (b.samples - b.extra != 1 && b.samples - b.extra != 3) {
            throw UsageError(f + ": gray or RGB images (optionally with alpha) expected");
        }
    }
    Image& first = imgs.front();
    if (!s.depth.empty()) {
        const std::string want = first.type == SampleType::U8 ? "8" : (first.type == SampleType::U16 ? "16" : "float");
        if (s.depth != want) {
            throw UsageError("--depth=" + s.depth + ": this build writes the input's depth (" + want + ") only");
        }
    }
    const int n = (int)imgs.size(), w = first.width, h = first.height;
    const int C = first.samples - first.extra >= 3 ? 3 : 1;
    enb_ctx* ctx = nullptr;
    check(nullptr, enb_create(0, &ctx), "enb_create");
    Image result = first;  // the accumulated (black) image, blended into in place
    std::vector<uint8_t> alpha = alpha_plane(first);  // the accumulated union alpha
    for (int i = 1; i < n; ++i) {
        const std::string mf = expand_template(s.mask_template, (unsigned)(n - 1), (unsigned)(i - 1));
        Image m;
        if (s.load_masks) {
            m = read_image(mf);
            if (m.samples != 1 || m.type != SampleType::U8) {
                throw UsageError("mask image \"" + mf + "\" must be 8-bit gray without alpha");
            }
            if (m.width != w || m.height != h) {
                throw UsageError("mask in \"" + mf + "\" does not have the canvas size");
            }
        } else {
            // the nearest-feature transform of the new image's footprint
            // against the accumulated one (src/mask.h:1130-1136)
            m.width = w;
            m.height = h;
            m.samples = 1;
            m.type = SampleType::U8;
            m.data.assign((size_t)w * h, 0);
            std::vector<uint8_t> wa = alpha_plane(imgs[i]);
            enb_image wd = plane_desc(wa.data(), w, h, w, ENB_U8), bd = plane_desc(alpha.data(), w, h, w, ENB_U8);
            enb_image md = plane_desc(m.data.data(), w, h, w, ENB_U8);
            check(ctx, enb_nft_mask(ctx, &wd, &bd, &md, &s.opt), "enb_nft_mask");
            if (s.save_masks) {
                write_image(mf, m);
            }
        }
        enb_image white = pixel_desc(imgs[i]), black = pixel_desc(result);
        enb_image mask = plane_desc(m.data.data(), w, h, w, ENB_U8);
        enb_image oa = plane_desc(alpha.data(), w, h, w, ENB_U8);
        check(ctx, enb_enblend(ctx, &white, nullptr, &black, nullptr, &mask, &black, &oa, &s.opt), "enb_enblend");
        if (s.verbose) {
            std::cerr << kCommand << ": info: blended \"" << s.inputs[i] << "\" under \"" << mf << "\"\n";
        }
    }
    enb_destroy(ctx);
    write_image(s.output, with_alpha(result, C, alpha));
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    try {
        Settings s = parse(argc, argv);
        if (s.dry_run) {
            std::cout << "{\"levels\": " << s.opt.levels << ", \"wrap\": " << s.opt.wrap << ", \"mask_template\": \""
                      << s.mask_template << "\", \"output\": \"" << s.output << "\", \"inputs\": " << s.inputs.size()
                      << ", \"seams\": \"" << (s.load_masks ? "loaded" : "nearest-feature")
                      << "\", \"save_masks\": " << (s.save_masks ? "true" : "false") << "}" << std::endl;
            return 0;
        }
        return run(s);
    } catch (const std::exception& e) {
        std::cerr << kCommand << ": " << e.what() << "\n";
        return 1;
    }
}

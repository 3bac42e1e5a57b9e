// adaptor_enblend.cpp -- enblendMain's pyramid section (src/enblend.h:
// 384-510) written against the header-only C++ adaptor (include/enbgpu.hpp)
// the way code using the reference's templates is written: the mask's
// Gaussian pyramid, the Laplacian pyramids of both images with their alpha,
// blend, collapse and the output conversion.  Test program of
// tests/test_cpu_adaptor.py and tests/test_gpu_adaptor.py.
//
// usage: adaptor_enblend W H LEVELS white.raw black.raw mask.raw out.raw
//   white/black: H x W x 3 uint16, alpha 65535 where nonzero sum; mask: H x W
//   uint8 (0/255); out: H x W x 3 uint16.  Exit 2 when there is no GPU.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "enbgpu.hpp"

template <typename T>
static std::vector<T> load(const char* path, size_t n)
{
    std::vector<T> v(n);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
    if (!f) {
        throw std::runtime_error(std::string("cannot read ") + path);
    }
    return v;
}

template <typename T>
static T* to_device(const std::vector<T>& v)
{
    void* p = nullptr;
    if (cudaMalloc(&p, v.size() * sizeof(T)) != cudaSuccess ||
        cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
        throw std::runtime_error("device buffer");
    }
    return static_cast<T*>(p);
}

int main(int argc, char** argv)
{
    if (argc != 8) {
        std::cerr << "usage: adaptor_enblend W H LEVELS white.raw black.raw mask.raw out.raw\n";
        return 1;
    }
    const int w = std::atoi(argv[1]), h = std::atoi(argv[2]), levels = std::atoi(argv[3]);
    const size_t npx = (size_t)w * h;
    try {
        enbgpu::Context ctx(0);
        const std::vector<uint16_t> white = load<uint16_t>(argv[4], npx * 3), black = load<uint16_t>(argv[5], npx * 3);
        const std::vector<uint8_t> mask = load<uint8_t>(argv[6], npx);
        std::vector<uint8_t> wa(npx), ba(npx), ua(npx);
        for (size_t p = 0; p < npx; ++p) {
            wa[p] = (white[3 * p] | white[3 * p + 1] | white[3 * p + 2]) ? 255 : 0;
            ba[p] = (black[3 * p] | black[3 * p + 1] | black[3 * p + 2]) ? 255 : 0;
            ua[p] = (wa[p] | ba[p]) ? 255 : 0;
        }
        uint16_t* dw = to_device(white);
        uint16_t* db = to_device(black);
        uint8_t* dm = to_device(mask);
        uint8_t* dwa = to_device(wa);
        uint8_t* dba = to_device(ba);
        uint8_t* dua = to_device(ua);
        uint16_t* dout = to_device(black);
        using enbgpu::ImageRef;
        const ImageRef W = ImageRef::pixels(dw, w, h, 3, 3), B = ImageRef::pixels(db, w, h, 3, 3);
        const ImageRef WA = ImageRef::plane(dwa, w, h), BA = ImageRef::plane(dba, w, h), UA = ImageRef::plane(dua, w, h);
        const ImageRef M = ImageRef::plane(dm, w, h), OUT = ImageRef::pixels(dout, w, h, 3, 3);
        // enblend.h:384-388: the mask pyramid without alpha (8-bit mask ->
        // Int32 9.15 mask pyramid of 16-bit images)
        enbgpu::Pyramid maskGP(ctx, levels, w, h, 1, ENB_I32);
        ctx.check(enb_gaussian_pyramid(ctx.get(), 0, M.get(), nullptr, 15, maskGP.get()));
        // enblend.h:418-446: the two Laplacian pyramids with their alpha
        enbgpu::Pyramid whiteLP = enbgpu::laplacianPyramid<uint16_t>(ctx, "whiteLP", levels, false, W, &WA);
        enbgpu::Pyramid blackLP = enbgpu::laplacianPyramid<uint16_t>(ctx, "blackLP", levels, false, B, &BA);
        // enblend.h:471-474: blend with the mask pyramid's white 255 << 15
        enbgpu::blend(ctx, maskGP, whiteLP, blackLP, 255 << 15);
        // enblend.h:503-510: collapse and convert where the union alpha is set
        enbgpu::collapsePyramid(ctx, false, blackLP);
        enbgpu::copyFromPyramidImageIf<uint16_t>(ctx, blackLP, UA, OUT);
        ctx.synchronize();
        std::vector<uint16_t> out(npx * 3);
        cudaMemcpy(out.data(), dout, out.size() * 2, cudaMemcpyDeviceToHost);
        std::ofstream(argv[7], std::ios::binary).write(reinterpret_cast<const char*>(out.data()),
                                                       (std::streamsize)(out.size() * 2));
        for (void* p : {(void*)dw, (void*)db, (void*)dm, (void*)dwa, (void*)dba, (void*)dua, (void*)dout}) {
            cudaFree(p);
        }
    } catch (const enbgpu::Error& e) {
        std::cerr << "enbgpu error " << e.status << ": " << e.what() << "\n";
        return e.status == ENB_ERR_CUDA ? 2 : 3;
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 4;
    }
    return 0;
}

// ref_harness.cpp -- runs the reference's own host code on the CPU and prints
// golden vectors as JSON (test infrastructure; built by `make -C oracle ref`
// only where the reference sources are mounted).
//
// Compiled together with the reference's FIRGaussianConvolver.cu and
// including, unmodified and in place:
//   TU/cu/FIRGaussianConvolver.h   lobe design  (FIRGaussianConvolver.h:123-170)
//   FIRGaussianConvolver.cu        lobeSize     (FIRGaussianConvolver.cu:52-98)
//   TU/cu/GuidedFilter.h           init_coeffs / trans_guides (GuidedFilter.h:59-125)
//   Testprog/filterTest/filterImageGold.h   CPU FIR gold (filterImageGold.h:11-47)
// Floats are printed as IEEE-754 bit patterns so the fixtures are exact.
#include "TU/cu/FIRGaussianConvolver.h"
#include "TU/cu/GuidedFilter.h"
#include "filterImageGold.h"

#include <cstdint>
#include <cstdio>
#include <cstring>

static uint32_t bits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// Deterministic generator (64-bit LCG, top 24 bits) so the harness needs no
// input; the inputs are printed next to the outputs.
struct Lcg
{
    uint64_t s;
    float next()
    {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        return float(s >> 40) / float(1 << 24);
    }
};

static void print_farray(const char* key, const float* v, size_t n, bool last = false)
{
    std::printf("\"%s\": [", key);
    for (size_t i = 0; i < n; ++i)
        std::printf("%s\"%08x\"", i ? ", " : "", bits(v[i]));
    std::printf("]%s", last ? "" : ", ");
}

int main()
{
    using namespace TU;
    std::printf("{\n");

    // 1. Gaussian lobe design over a sweep of sigmas.
    const float sigmas[] = {0.2f, 0.35f, 0.5f, 0.6f, 0.75f, 0.9f, 1.0f, 1.1f, 1.25f, 1.5f,
                            1.75f, 2.0f, 2.25f, 2.5f, 2.75f, 3.0f, 3.5f, 4.0f, 4.5f,
                            5.0f, 6.0f, 7.0f, 8.0f, 10.0f, 12.0f, 16.0f};
    std::printf("\"lobes\": [\n");
    for (size_t k = 0; k < sizeof(sigmas) / sizeof(sigmas[0]); ++k)
    {
        TU::Array<float> l0, l1, l2;
        cu::FIRGaussianConvolver2<float>::initialize(sigmas[k], l0, l1, l2);
        std::printf("  {\"sigma\": \"%08x\", ", bits(sigmas[k]));
        print_farray("lobe0", l0.data(), l0.size());
        print_farray("lobe1", l1.data(), l1.size());
        print_farray("lobe2", l2.data(), l2.size(), true);
        std::printf("}%s\n", k + 1 < sizeof(sigmas) / sizeof(sigmas[0]) ? "," : "");
    }
    std::printf("],\n");

    // 2. lobeSize on crafted lobes: all zero, a single spike at each index,
    //    and random decaying profiles.
    std::printf("\"lobe_size\": [\n");
    Lcg rng{12345};
    bool first = true;
    for (int even = 0; even < 2; ++even)
    {
        for (int c = 0; c < 40; ++c)
        {
            float lb[17] = {0};
            if (c == 0) {
            } else if (c <= 17) {
                lb[c - 1] = 1.0f;
                lb[0] = 0.5f;
            } else {
                const float decay = 0.3f + 0.7f * rng.next();
                float v = 1.0f;
                for (int i = 0; i < 17; ++i) {
                    lb[i] = (rng.next() < 0.5f ? -v : v);
                    v *= decay;
                }
            }
            std::printf("%s  {\"even\": %d, ", first ? "" : ",\n", even);
            first = false;
            print_farray("lobe", lb, 17);
            std::printf("\"size\": %zu}", cu::detail::lobeSize(lb, even != 0));
        }
    }
    std::printf("\n],\n");

    // 3. filterImageGold's separable FIR (symmetric lobes, transposed twice)
    //    on a small random image with the sigma=1 and sigma=2 lobes.
    std::printf("\"fir_gold\": [\n");
    const float fsig[] = {1.0f, 2.0f};
    for (int k = 0; k < 2; ++k)
    {
        TU::Array<float> l0, l1, l2;
        cu::FIRGaussianConvolver2<float>::initialize(fsig[k], l0, l1, l2);
        const size_t rows = 37, cols = 45;
        TU::Array2<TU::Array<float>> in(rows, cols), mid, out;
        Lcg r{uint64_t(777 + k)};
        for (size_t y = 0; y < rows; ++y)
            for (size_t x = 0; x < cols; ++x)
                in[y][x] = std::floor(255.0f * r.next());
        filter1D(in, mid, l0);
        filter1D(mid, out, l0);
        std::printf("  {\"sigma\": \"%08x\", \"rows\": %zu, \"cols\": %zu, ", bits(fsig[k]), rows, cols);
        std::vector<float> flat_in, flat_out;
        for (size_t y = 0; y < rows; ++y)
            for (size_t x = 0; x < cols; ++x) {
                flat_in.push_back(in[y][x]);
                flat_out.push_back(out[y][x]);
            }
        print_farray("lobe", l0.data(), l0.size());
        print_farray("in", flat_in.data(), flat_in.size());
        print_farray("out", flat_out.data(), flat_out.size(), true);
        std::printf("}%s\n", k == 0 ? "," : "");
    }
    std::printf("],\n");

    // 4. Guided-filter coefficient functors on random window sums.
    std::printf("\"guided\": [\n");
    Lcg g{4242};
    for (int c = 0; c < 64; ++c)
    {
        const size_t w = 3 + 2 * (c % 8);
        const size_t n = w * w;
        const float e = (c % 3 == 0) ? 0.1f : (c % 3 == 1) ? 2.5f : 25.5f;
        // window sums of plausible 0..255 images
        float sp = 0, sg = 0, spg = 0, sgg = 0;
        for (size_t i = 0; i < n; ++i) {
            const float pv = std::floor(255.0f * g.next()), gv = std::floor(255.0f * g.next());
            sp += pv; sg += gv; spg += pv * gv; sgg += gv * gv;
        }
        const cu::vec<float, 4> params{sp, sg, spg, sgg};
        const cu::vec<float, 2> sparams{sp, spg};
        const auto cf = cu::device::init_coeffs<float>(n, e)(params);
        const auto cs = cu::device::init_coeffs<float>(n, e)(sparams);
        const float A = cf.x * float(n) * (0.9f + 0.2f * g.next());
        const float B = cf.y * float(n) * (0.9f + 0.2f * g.next());
        const float gv = std::floor(255.0f * g.next());
        float outv = 0;
        const cu::device::trans_guides<float> trans(n);
        trans(std::tuple<float, float&>(gv, outv), cu::vec<float, 2>{A, B});
        std::printf("  {\"n\": %zu, \"e\": \"%08x\", ", n, bits(e));
        const float s4[4] = {sp, sg, spg, sgg};
        print_farray("sums", s4, 4);
        const float c4[4] = {cf.x, cf.y, cs.x, cs.y};
        print_farray("coeffs", c4, 4);
        const float t4[4] = {A, B, gv, outv};
        print_farray("trans", t4, 4, true);
        std::printf("}%s\n", c + 1 < 64 ? "," : "");
    }
    std::printf("]\n}\n");
    return 0;
}

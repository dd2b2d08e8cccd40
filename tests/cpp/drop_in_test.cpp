// drop_in_test.cpp -- calls the C++ drop-in classes (include/TU/cu/*.h) the
// way code written against the reference's TU::cu classes calls them, with
// the reference's own template argument lists (the instantiations of
// Testprog/cudaStereoTest/cudaJob.cu:18-19 and 57-58, TU/cu/SuperPixels.h:
// 596-597, Testprog/boxFilterTest/main.cu:19-21 and 70-71,
// Testprog/boxFilterTest2/main.cu:19-23, Testprog/guidedFilterTest/
// cudaJob.cu:14, Testprog/filterTest/main.cu:90, Testprog/gaussTest/
// main.cu:90), on deterministic images, and writes each input and output to
// <dir> as raw files (rows, cols, dtype header + pitched-free pixels) for the
// Python test to compare with the Python path.  Also checks the error
// behaviour: lobes and windows that are too large throw, images smaller than
// the support are a silent no-op.  Exit status 0 = every check held.
#include <thrust/functional.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "TU/cu/BoxFilter.h"
#include "TU/cu/FIRFilter.h"
#include "TU/cu/FIRGaussianConvolver.h"
#include "TU/cu/GuidedFilter.h"
#include "TU/cu/StereoUtility.h"

using TU::cu::Array2;
namespace cu = TU::cu;

// Pixel (y, x) of image k: a fixed integer hash, 0..255.
static uint32_t pix(int k, int y, int x)
{
    uint32_t h = (uint32_t)(y * 131 + x * 71 + k * 1009 + 17) * 2654435761u;
    return (h >> 11) % 256u;
}

template <class T>
static Array2<T> image(int k, int rows, int cols)
{
    std::vector<T> host((size_t)rows * cols);
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x)
            host[(size_t)y * cols + x] = (T)(float)pix(k, y, x);
    Array2<T> a(rows, cols);
    a.upload(host.data(), cols * sizeof(T));
    return a;
}

template <class T>
static void fill(Array2<T>& a, T v)
{
    std::vector<T> host((size_t)a.nrow() * a.ncol(), v);
    a.upload(host.data(), a.ncol() * sizeof(T));
}

template <class T>
static void save(const std::string& dir, const char* name, const Array2<T>& a, int dtype)
{
    std::vector<T> host((size_t)a.nrow() * a.ncol());
    a.download(host.data(), a.ncol() * sizeof(T));
    FILE* f = std::fopen((dir + "/" + name + ".bin").c_str(), "wb");
    if (!f)
        throw std::runtime_error(std::string("cannot write ") + name);
    const int32_t hdr[3] = {a.nrow(), a.ncol(), dtype};
    std::fwrite(hdr, sizeof(hdr), 1, f);
    std::fwrite(host.data(), sizeof(T), host.size(), f);
    std::fclose(f);
}

static int failures = 0;
static void expect(bool ok, const char* what)
{
    if (!ok) {
        std::fprintf(stderr, "FAILED: %s\n", what);
        ++failures;
    }
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s OUTDIR\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
    try {
        // Gaussian smooth and diffH, float -> float (configuration 1 shape)
        Array2<float> g_in = image<float>(0, 480, 640), g_sm(480, 640), g_dh(480, 640);
        fill(g_sm, -1.0f);
        fill(g_dh, -1.0f);
        cu::FIRGaussianConvolver2<float> gauss(2.0f);  // gaussTest/main.cu:90
        expect(gauss.sigma() == 2.0f, "sigma()");
        gauss.smooth(g_in.cbegin(), g_in.cend(), g_sm.begin());
        gauss.diffH(g_in.cbegin(), g_in.cend(), g_dh.begin(), false);

        // the tensor-core switch: Gaussian smooth sigma 8 of an f16 image -> float
        Array2<__half> t_in = image<__half>(0, 480, 640);
        Array2<float> t_out(480, 640);
        fill(t_out, -1.0f);
        TU::cu::FIRGaussianConvolver2<float> tgauss(8.0f);
        tgauss.setTensorCores(true).smooth(t_in.cbegin(), t_in.cend(), t_out.begin());

        // FIRFilter2 with caller lobes (5 and 4 taps), u8 -> float
        Array2<unsigned char> f_in = image<unsigned char>(1, 200, 333);
        Array2<float> f_out(200, 333);
        fill(f_out, -1.0f);
        cu::FIRFilter2<float> fir;  // filterTest/main.cu:90
        const std::vector<float> lobeH = {0.05f, 0.1f, 0.2f, 0.25f, 0.4f}, lobeV = {-0.1f, -0.2f, -0.3f, -0.4f};
        fir.initialize(lobeH, lobeV);
        expect(fir.offsetH() == 4 && fir.offsetV() == 4 && fir.outSizeH(333) == 325, "FIRFilter2 geometry");
        fir.convolve(f_in.cbegin(), f_in.cend(), f_out.begin());

        // BoxFilter2 15x15 sums, u8 -> int32 (configuration 2 plane)
        Array2<unsigned char> b_in = image<unsigned char>(2, 300, 401);
        Array2<int32_t> b_out(300, 401);
        fill(b_out, (int32_t)-7);
        // the boxFilterTest shape (const filter, BlockTraits<32, 16>)
        const cu::BoxFilter2<cu::device::box_convolver<int>, cu::BlockTraits<32, 16>, 31> box(15, 15);
        expect(box.outSizeV(300) == 286 && box.offsetH() == 7, "BoxFilter2 geometry");
        expect(box.BlockDimX == 32 && box.BlockDimY == 16, "BoxFilter2 block traits");
        box.convolve(b_in.cbegin(), b_in.cend(), b_out.begin());

        // BoxFilter2 with extrema_finder<extrema_value_position<less>>: 7x9
        // window minima of the same plane and their (x, y) positions
        Array2<unsigned char> e_val(300, 401);
        Array2<int2> e_pos(300, 401);
        fill(e_val, (unsigned char)200);
        fill(e_pos, make_int2(-5, -5));
        using min_finder = cu::device::extrema_finder<
            cu::device::extrema_value_position<thrust::less<unsigned char>>>;  // boxFilterTest2 shape
        const cu::BoxFilter2<min_finder> ext(7, 9);
        expect(ext.outSizeH(401) == 393 && ext.offsetV() == 3, "extrema BoxFilter2 geometry");
        ext.convolve(b_in.cbegin(), b_in.cend(), e_val.begin(), e_pos.begin());
        // extrema_value alone (boxFilterTest/main.cu:70-71) gives the same minima
        Array2<unsigned char> e_val2(300, 401);
        fill(e_val2, (unsigned char)200);
        const cu::BoxFilter2<cu::device::extrema_finder<cu::device::extrema_value<thrust::less<unsigned char>>>,
                             cu::BlockTraits<32, 16>>
            ext_v(7, 9);
        ext_v.convolve(b_in.cbegin(), b_in.cend(), e_val2.begin());

        // stereo cost aggregation: 7x7 windows, 16 disparities, diff<u8>(50),
        // left = the box input, right = image 6 (disparity-major costs)
        Array2<unsigned char> s_right = image<unsigned char>(6, 300, 401);
        TU::cu::Array3<int32_t> s_costs(16, 300, 401);
        // cudaStereoTest/cudaJob.cu:18-19 with S = int32_t, timed by cu::clock
        cu::BoxFilter2<cu::device::box_convolver<int32_t>, cu::BlockTraits<>, 23, cu::clock> sbox(7, 7);
        sbox.convolve(b_in.cbegin(), b_in.cend(), s_right.cbegin(), s_costs.begin(),
                      cu::diff<unsigned char>(50), 16);
        sbox.print(std::cerr);
        // cudaJob.cu:57-58: the host clock as CLOCK
        cu::BoxFilter2<cu::device::box_convolver<int32_t>, cu::BlockTraits<>, 23, std::chrono::system_clock>
            hbox(7, 7);
        expect(hbox.outSizeV(300) == 294, "BoxFilter2 with a host clock");
        // DisparitySelector over the valid cost region, written from (3, 3) of
        // the disparity image as the reference's stereo test places it
        Array2<int32_t> s_disp(300, 401);
        TU::cu::DisparitySelector<int32_t> selector(40, 2);
        selector.select(s_costs, TU::cu::RowIterator<int32_t>((s_disp.begin() + 3).ptr() + 3, s_disp.pitch(), 398),
                        sbox.outSizeV(300), sbox.outSizeH(401));

        // box_convolver<vec<float, 4>>: feature vectors as float4 pixels
        Array2<float4> v_in(120, 333), v_out(120, 333);
        {
            std::vector<float4> host((size_t)120 * 333);
            for (int y = 0; y < 120; ++y)
                for (int x = 0; x < 333; ++x)
                    host[(size_t)y * 333 + x] = make_float4((float)pix(7, y, x), (float)pix(8, y, x),
                                                            (float)pix(9, y, x), (float)pix(10, y, x));
            v_in.upload(host.data(), 333 * sizeof(float4));
        }
        fill(v_out, make_float4(-1.f, -1.f, -1.f, -1.f));
        // SuperPixels.h:596-597 with feature_type = vec<float, 4>
        using feature_type = cu::vec<float, 4>;
        using filter_type = TU::cu::BoxFilter2<TU::cu::device::box_convolver<feature_type>>;
        filter_type vbox(5, 9);
        vbox.convolve(v_in.cbegin(), v_in.cend(), v_out.begin());

        // GuidedFilter2 17x17, e = 25.5, with a guide and self-guided
        Array2<float> p = image<float>(3, 210, 300), gd = image<float>(4, 210, 300), o1(210, 300), o2(210, 300);
        fill(o1, -3.0f);
        fill(o2, -3.0f);
        // guidedFilterTest/cudaJob.cu:14 (U = float), timed by cu::clock
        cu::GuidedFilter2<float, cu::BlockTraits<>, 23, cu::clock> guided(17, 17, 25.5f);
        expect(guided.offsetV() == 16 && guided.outSizeH(300) == 268, "GuidedFilter2 geometry");
        guided.convolve(p.cbegin(), p.cend(), gd.cbegin(), gd.cend(), o1.begin());
        guided.convolve(p.cbegin(), p.cend(), o2.begin());
        guided.print(std::cerr);

        // an image smaller than the support: silent no-op, output untouched
        Array2<float> tiny = image<float>(5, 10, 10), tiny_out(10, 10);
        fill(tiny_out, 9.0f);
        gauss.smooth(tiny.cbegin(), tiny.cend(), tiny_out.begin());
        std::vector<float> t(100);
        tiny_out.download(t.data(), 10 * sizeof(float));
        bool untouched = true;
        for (float v : t)
            untouched = untouched && v == 9.0f;
        expect(untouched, "small image is a no-op");

        // too-long lobe and too-wide window throw
        bool threw = false;
        try {
            const std::vector<float> big(18, 0.1f);
            fir.initialize(big, big);
        } catch (const std::runtime_error&) {
            threw = true;
        }
        expect(threw, "18-tap lobe throws");
        threw = false;
        try {
            cu::BoxFilter2<cu::device::box_convolver<int>, cu::BlockTraits<32, 16>, 31> wide(15, 15);
            wide.setWinSizeH(33);
        } catch (const std::runtime_error&) {
            threw = true;
        }
        expect(threw, "window above WMAX throws");

        cudaDeviceSynchronize();
        save(dir, "g_in", g_in, TUCU_F32);
        save(dir, "g_smooth", g_sm, TUCU_F32);
        save(dir, "g_diffh_noshift", g_dh, TUCU_F32);
        save(dir, "f_in", f_in, TUCU_U8);
        save(dir, "f_out", f_out, TUCU_F32);
        save(dir, "b_in", b_in, TUCU_U8);
        save(dir, "b_out", b_out, TUCU_I32);
        save(dir, "e_val", e_val, TUCU_U8);
        save(dir, "e_pos", e_pos, TUCU_I32);  // rows x cols int2: two int32 per pixel
        save(dir, "e_val2", e_val2, TUCU_U8);
        save(dir, "s_right", s_right, TUCU_U8);
        save(dir, "t_in", t_in, TUCU_F16);
        save(dir, "t_out", t_out, TUCU_F32);
        save(dir, "s_disp", s_disp, TUCU_I32);
        save(dir, "v_in", v_in, TUCU_F32);    // rows x cols float4: four floats per pixel
        save(dir, "v_out", v_out, TUCU_F32);
        {
            std::vector<int32_t> host((size_t)16 * 300 * 401);
            s_costs.download(host.data());
            FILE* f = std::fopen((dir + "/s_costs.bin").c_str(), "wb");
            if (!f)
                throw std::runtime_error("cannot write s_costs");
            const int32_t hdr[3] = {16 * 300, 401, TUCU_I32};
            std::fwrite(hdr, sizeof(hdr), 1, f);
            std::fwrite(host.data(), sizeof(int32_t), host.size(), f);
            std::fclose(f);
        }
        save(dir, "p", p, TUCU_F32);
        save(dir, "gd", gd, TUCU_F32);
        save(dir, "o_guided", o1, TUCU_F32);
        save(dir, "o_self", o2, TUCU_F32);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "FAILED with exception: %s\n", e.what());
        return 1;
    }
    if (failures)
        return 1;
    std::printf("drop-in ok\n");
    return 0;
}

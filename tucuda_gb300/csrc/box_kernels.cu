// box_kernels.cu -- BoxFilter2's launcher, task planning and kernel
// selection for the one-pass window-sum strip (box_strip.cuh); the guided
// passes are in guided.cuh.
#include <algorithm>

#include "box_kernels.h"
#include "box_plain.cuh"

namespace tucu
{
namespace box
{

template <int CPT, bool WIN = false>
static size_t plain_smem_cpt(int in_dtype)
{
    switch (in_dtype) {
    case U8: return PlainRing<uint8_t, true, CPT, WIN>::kSmem;
    case I32: return PlainRing<int32_t, true, CPT, WIN>::kSmem;
    case F16: return PlainRing<__half, true, CPT, WIN>::kSmem;
    case BF16: return PlainRing<__nv_bfloat16, true, CPT, WIN>::kSmem;
    case F32: return PlainRing<float, true, CPT, WIN>::kSmem;
    default: return 0;
    }
}

size_t plain_smem_bytes(int in_dtype, int cpt, bool win)
{
    if (win)
        return plain_smem_cpt<4, true>(in_dtype);
    return cpt == 8 ? plain_smem_cpt<8>(in_dtype) : plain_smem_cpt<4>(in_dtype);
}

bool plain_win(int in_dtype, int out_dtype, bool vec, int cpt, int wV)
{
    return vec && cpt == kCPT && wV <= kWinMaxV && typed_kernel(in_dtype, out_dtype, false, cpt, true);
}

const void* batch_kernel(int in_dtype, int out_dtype, bool vec, int cpt, bool win)
{
    const void* fn = vec ? typed_kernel(in_dtype, out_dtype, true, cpt, win) : nullptr;
    return fn ? fn : generic_kernel(in_dtype, vec, true, cpt);
}

// ---- launchers ------------------------------------------------------------------

// Rows of es-byte pixels aligned for the copies of cpt-pixel groups (copies
// of at most 16 bytes: 8-pixel groups of 4-byte pixels are two copies).
static bool rows_aligned(const void* p, size_t pitch, size_t es, int cpt)
{
    const size_t a = std::min<size_t>((size_t)cpt * es, 16);
    return (reinterpret_cast<uintptr_t>(p) % a) == 0 && (pitch % a) == 0;
}

bool plain_vec(const void* src, size_t pitch, int in_dtype, int cpt)
{
    // The 8-column kernels (wide windows only) load synchronously.
    return cpt == kCPT && rows_aligned(src, pitch, dtype_size(in_dtype), cpt);
}

int plain_cpt(int wH)
{
    return out_cols_per_warp(wH, 4) > 0 ? 4 : 8;
}

// Warp tasks for an image: the strip height (a multiple of the restart
// period) that minimises rounds x (strip + window set-up), where a round is
// one task for every warp the grid keeps resident.
TaskGrid plan_tasks(int orows, int ocols, int wV, int wH, int strip_rows, int ctas_per_sm,
                    int restart, int copies, int cpt, bool exact)
{
    TaskGrid t;
    t.restart = restart;
    const int tw = out_cols_per_warp(wH, cpt);
    t.nwc = (ocols + tw - 1) / tw;
    const long warps = (long)ctas_per_sm * sm_count() * kWarps;
    auto tasks_of = [&](int strip) { return (long)t.nwc * ((orows + strip - 1) / strip) * copies; };
    if (strip_rows > 0) {
        t.strip_rows = (strip_rows + 15) / 16 * 16;
    } else {
        // Bands that are multiples of the restart period: whole rounds of
        // warp tasks x (band + wV), over the bands whose tasks fill at least
        // 90% of a round of resident warps when any does.  (Measured on the
        // box strip: a single round that leaves a quarter of the warp slots
        // empty runs its steps no faster than full rounds do, so for 15x15
        // f16 means at 6480x11520 three rounds of 64-row bands, 126 us, beat
        // one round of 192-row bands at 72% occupancy, 137 us.)
        t.strip_rows = restart;
        double best = 1e300;
        bool best_full = false;
        for (int k = 1; k <= 32; ++k) {
            const int strip = k * restart;
            const long tasks = tasks_of(strip);
            const long rounds = (tasks + warps - 1) / warps;
            const double cost = (double)rounds * (std::min(strip, orows) + wV);
            const bool full = tasks * 10 >= warps * 9;
            if ((full && !best_full) || (full == best_full && cost < best)) {
                best = cost;
                best_full = full;
                t.strip_rows = strip;
            }
            if (strip >= orows)
                break;
        }
        // An image too small to give every SM a CTA of warp tasks gets bands
        // shorter than the restart period (halves, quarters, down to 16
        // rows, or the period when it is shorter): a band inside a restart
        // block replays the rows of the block above it, which costs little
        // next to the idle SMs it fills.
        // Exact (integer) sums replay nothing, so their bands halve down to 8
        // rows while the tasks fill less than 90% of the resident warps.
        const long fill = exact ? warps * 9 / 10 : (long)sm_count() * kWarps * 3 / 4;
        const int min_strip = exact ? 8 : std::min(16, restart);
        while (t.strip_rows > min_strip && t.strip_rows <= restart && tasks_of(t.strip_rows) < fill)
            t.strip_rows /= 2;
    }
    t.ntask = (int)tasks_of(t.strip_rows) / copies;
    return t;
}

static dim3 grid_for(const Geo& G, int ctas_per_sm)
{
    const long want = (G.tg.ntask + kWarps - 1) / kWarps;
    return dim3((unsigned)std::max(1L, std::min(want, (long)ctas_per_sm * sm_count())));
}

cudaError_t launch_box(const BoxLaunch& L, cudaStream_t st)
{
    Geo G;
    G.wV = L.wV;
    G.wH = L.wH;
    G.orows = L.rows + 1 - L.wV;
    G.ocols = L.cols + 1 - L.wH;
    if (L.in_dtype < U8 || L.in_dtype > I32)
        return cudaErrorInvalidValue;
    const int cpt = plain_cpt(L.wH);
    const int ctas = cpt == 8 ? PlainCfg<8>::kCtas : PlainCfg<4>::kCtas;
    const bool vec = plain_vec(L.src, L.src_pitch, L.in_dtype, cpt);
    // Integer sums are exact in any order, so their bands are planned in
    // 16-row units and small images split down to 8 rows (more warp tasks);
    // float sums keep the 64-row restart grid the batched launch uses, so
    // both agree bit for bit.
    const bool integral = L.in_dtype == U8 || L.in_dtype == I32;
    G.tg = plan_tasks(G.orows, G.ocols, L.wV, L.wH, L.strip_rows, ctas, integral ? 16 : kRestart, 1, cpt,
                      integral);
    const bool win = plain_win(L.in_dtype, L.out_dtype, vec, cpt, L.wV);
    const void* fn = vec ? typed_kernel(L.in_dtype, L.out_dtype, false, cpt, win) : nullptr;
    if (!fn)
        fn = generic_kernel(L.in_dtype, vec, false, cpt);
    BoxArgs A;
    A.src = L.src;
    A.src_pitch = L.src_pitch;
    A.rows = L.rows;
    A.cols = L.cols;
    A.dst = L.dst;
    A.dst_pitch = L.dst_pitch;
    A.out_dtype = L.out_dtype;
    A.oy = L.oy;
    A.ox = L.ox;
    A.normalize = L.normalize;
    A.inv_n = 1.0f / (float)(L.wV * L.wH);
    A.cls = store_class(L.dst, L.dst_pitch, L.ox, dtype_size(L.out_dtype));
    void* args[] = {&G, &A};
    return cudaLaunchKernel(fn, grid_for(G, ctas), dim3(kThreads), args, plain_smem_bytes(L.in_dtype, cpt, win), st);
}

cudaError_t launch_guided(const GuidedLaunch& L, cudaStream_t st)
{
    // Windows wider than a 4-column warp tile holds (wH > 125) take 8 columns
    // per lane (guided_wide.cu).
    return out_cols_per_warp(L.wH, 4) > 0 ? launch_guided_narrow(L, st) : launch_guided_wide(L, st);
}

}  // namespace box
}  // namespace tucu

TUCU_DEFINE_ERROR_ACCESSOR(tucu_box_tu_error)

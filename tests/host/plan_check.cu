// Host-side check of the rectangle plans of the resident kernels (no device code runs): for a
// range of lattices, every plan that reports ok fits the per-block shared-memory budget, keeps
// one ring site per thread, covers the lattice with at most one rectangle per SM, and gives
// every thread at most its instantiated row count.  Prints the violations (none expected) and
// the plans of the benchmark lattices as JSON.  Built and run by tests/test_plans.py.
#include <cstdio>

#include "stag_resident.cuh"
#include "stag_resident_eo.cuh"
#include "stag_resident_s.cuh"

using namespace glinalg;

static int bad = 0;

static void check(const char *name, int lx, int ly, const res::Plan &p, int nsm, size_t budget, int threads,
                  int sites_x)
{
    if (!p.ok) return;
    const bool fits = p.smem <= budget;
    const bool ring = 2 * res::kTX + 2 * p.ty <= threads;
    const bool grid = p.gx * p.gy <= nsm && p.gx * p.gy <= res::kMaxBlocks;
    const bool cover = p.gx * res::kTX == sites_x && p.gy * p.ty >= ly && (p.gy - 1) * p.ty < ly;
    const bool rows = p.ny * p.wy >= p.ty;
    if (!(fits && ring && grid && cover && rows)) {
        bad++;
        std::printf("{\"violation\": \"%s\", \"lx\": %d, \"ly\": %d, \"fits\": %d, \"ring\": %d, \"grid\": %d, "
                    "\"cover\": %d, \"rows\": %d}\n", name, lx, ly, fits, ring, grid, cover, rows);
    }
}

static void show(const char *name, int lx, int ly, const res::Plan &p)
{
    std::printf("{\"plan\": \"%s\", \"lx\": %d, \"ly\": %d, \"ok\": %d, \"gx\": %d, \"gy\": %d, \"ty\": %d, "
                "\"ny\": %d, \"smem\": %zu}\n", name, lx, ly, p.ok, p.gx, p.gy, p.ty, p.ny, p.smem);
}

int main()
{
    const int nsm = 152;
    const size_t budget = 232448 - 512;  // GB300's opt-in shared memory per block, less the static part
    for (int lx = 128; lx <= 4096; lx += 128) {
        for (int ly = 2; ly <= 4096; ly += (ly < 64 ? 2 : 62)) {
            for (int wy : {4, 8}) check("fp32", lx, ly, res::plan(lx, ly, nsm, budget, wy), nsm, budget, 32 * res::kWX * wy, lx);
            check("eo", lx, ly, reseo::plan(lx, ly, nsm, budget), nsm, budget, 32 * res::kWX * reseo::kWY, lx / 2);
            // both 16-bit variants: 4-byte fields, 8-byte (FP32) links
            check("fp16", lx, ly, ress::plan(lx, ly, nsm, budget, 4, 8), nsm, budget, 32 * res::kWX * ress::kWY, lx);
            check("bf16", lx, ly, ress::plan(lx, ly, nsm, budget, 4, 8), nsm, budget, 32 * res::kWX * ress::kWY, lx);
        }
    }
    show("fp32", 1024, 1024, res::plan(1024, 1024, nsm, budget, 4));
    show("eo", 1024, 1024, reseo::plan(1024, 1024, nsm, budget));
    show("fp16", 1024, 1024, ress::plan(1024, 1024, nsm, budget, 4, 8));
    show("bf16", 1024, 1024, ress::plan(1024, 1024, nsm, budget, 4, 8));
    show("fp32", 512, 512, res::plan(512, 512, nsm, budget, 4));
    show("fp32", 2048, 2048, res::plan(2048, 2048, nsm, budget, 4));
    std::printf("{\"violations\": %d}\n", bad);
    return bad != 0;
}

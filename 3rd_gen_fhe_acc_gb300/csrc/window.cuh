// window.cuh -- step window of the persistent blind-rotation kernels.
//
// Every CTA of a blind-rotation launch walks the refresh steps in the same
// order, each over its own group of ciphertexts, and reads the step's key tile
// (Br RGSW ciphertexts) from L2. The scheme relies on the CTAs staying close:
// left alone they drift hundreds of steps apart (on the 4096-gate N = 1024
// batch, half of the CTAs ran twice as fast as the rest), the live key tiles
// outgrow L2 and every CTA streams its keys from HBM. The window bounds the
// drift: the steps are cut into buckets of `steps` steps, a CTA counts itself
// into count[b] once it has issued every item of bucket b, and before it issues
// an item of bucket b it waits until every CTA of the launch has counted into
// bucket b - 2, so no CTA runs more than two buckets ahead of the slowest.
//
// The window orders nothing that results depend on: it only delays CTAs. Waits
// are bounded; a CTA that polls spin_limit times without seeing the count stops
// waiting for the rest of the launch (counted in count[buckets]), which is what
// happens if not every CTA of the grid is resident at once.
#pragma once
#include <cstdint>

namespace fheacc {
namespace dev {

struct StepWindow {
    unsigned *count;       // [buckets + 1], zeroed before the launch; null: no window
    int steps;             // steps per bucket
    int buckets;
    unsigned spin_limit;   // polls (about 0.25 us each) before a CTA stops waiting
};

// Run by one thread of a CTA that is about to issue an item of bucket b (b =
// buckets: the CTA has issued everything). cur: first bucket the CTA has not
// counted into yet; on: the CTA still waits; target: CTAs that count into each
// bucket by the end of the current chunk of ciphertexts.
__device__ __forceinline__ void window_enter(const StepWindow &w, int &cur, int &on, int b, unsigned target)
{
    if (!w.count) return;
    if (b > w.buckets) b = w.buckets;
    for (; cur < b; cur++) atomicAdd(w.count + cur, 1u);
    if (on && b >= 2 && b < w.buckets) {
        const volatile unsigned *p = w.count + (b - 2);
        unsigned polls = 0;
        while (*p < target) {
            if (++polls > w.spin_limit) {
                on = 0;
                atomicAdd(w.count + w.buckets, 1u);
                break;
            }
            __nanosleep(256);
        }
    }
}

}  // namespace dev
}  // namespace fheacc

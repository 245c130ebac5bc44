// Host-only check of PerDevice (mpres-blas_gb300/csrc/per_device.h): the set-up
// of each device ordinal runs once however many threads ask, a failed set-up
// is retried, devices do not share values, and out-of-range ordinals are
// refused.  Prints "ok" and exits 0 on success.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "per_device.h"

static bool zero_is_ok(const int &v) { return v == 0; }

int main() {
    using mpres::PerDevice;
    // 1. eight threads x 4 devices x 1000 calls: one set-up per device
    std::atomic<int> runs[4];
    for (auto &r : runs) r = 0;
    PerDevice<int> once(zero_is_ok);
    std::vector<std::thread> ts;
    for (int t = 0; t < 8; t++)
        ts.emplace_back([&, t] {
            for (int i = 0; i < 1000; i++) {
                const int dev = (t + i) % 4;
                if (once.get(dev, -1, [&] { runs[dev]++; return 0; }) != 0) std::abort();
            }
        });
    for (auto &t : ts) t.join();
    for (int d = 0; d < 4; d++)
        if (runs[d] != 1) { std::printf("device %d set up %d times\n", d, (int)runs[d]); return 1; }
    // 2. a failing set-up is not kept: the next call runs it again
    PerDevice<int> retry(zero_is_ok);
    int calls = 0;
    if (retry.get(1, -1, [&] { calls++; return 7; }) != 7) return 2;
    if (retry.get(1, -1, [&] { calls++; return 0; }) != 0) return 3;
    if (retry.get(1, -1, [&] { calls++; return 5; }) != 0) return 4; // kept now
    if (calls != 2) return 5;
    // 3. values are per device: device 2 is set up on its own
    if (retry.get(2, -1, [&] { calls++; return 0; }) != 0 || calls != 3) return 6;
    // 4. ordinals outside 0..63 return `invalid` without running the set-up
    if (retry.get(-1, -9, [&] { calls++; return 0; }) != -9) return 7;
    if (retry.get(mpres::kMaxDevices, -9, [&] { calls++; return 0; }) != -9 || calls != 3) return 8;
    std::puts("ok");
    return 0;
}

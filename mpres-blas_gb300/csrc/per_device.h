/*
 * Once-per-device host set-up: kernel attributes and launch shapes.
 *
 * A kernel attribute such as cudaFuncAttributeMaxDynamicSharedMemorySize is
 * recorded for the device that is current when cudaFuncSetAttribute runs, and
 * an occupancy-derived grid size belongs to one device's SM count.  A single
 * process-wide "done" flag would leave every other device at the default
 * 48 KB dynamic shared-memory limit (a later launch asking for more fails
 * there) or with another device's grid.  PerDevice<R> runs a set-up function
 * at most once per device ordinal, from any number of host threads, keeps the
 * value it returns when `keep(value)` holds, and runs it again on the next
 * call otherwise (a failed set-up is retried, not cached).
 *
 * Header-only and free of CUDA types so the logic can be tested on a host
 * without a GPU; the device ordinal is an argument.
 */
#ifndef MPRES_PER_DEVICE_H
#define MPRES_PER_DEVICE_H

#include <mutex>

namespace mpres {

constexpr int kMaxDevices = 64;

template <class R> class PerDevice {
  public:
    using Keep = bool (*)(const R &);
    explicit PerDevice(Keep keep) : keep_(keep) {}

    /* the kept value for `dev`, running setup() first if there is none;
     * `invalid` for an ordinal outside 0..kMaxDevices-1 */
    template <class F> R get(int dev, R invalid, F &&setup) {
        if (dev < 0 || dev >= kMaxDevices) return invalid;
        std::lock_guard<std::mutex> lk(mu_);
        if (done_[dev]) return value_[dev];
        const R v = setup();
        if (keep_(v)) {
            value_[dev] = v;
            done_[dev] = true;
        }
        return v;
    }

  private:
    Keep keep_;
    std::mutex mu_;
    bool done_[kMaxDevices] = {};
    R value_[kMaxDevices] = {};
};

} // namespace mpres

#endif

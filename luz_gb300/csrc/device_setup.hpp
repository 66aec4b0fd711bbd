// Setup that a process does once on its device for the library's kernels: function
// attributes (the dynamic shared-memory limit a launch needs) and constant tables.
//
// Host code only (no CUDA headers), so the guard logic is tested on its own.
//
// The setup is per device and the process keeps all its contexts on one device
// (luz_ctx_create refuses a second one). A DeviceSetup records, per setup
// generation, the largest level done so far: a shared-memory limit in bytes, or 1
// for a setup done once. luz_ctx_create starts a new generation when no other
// context of the process is alive, so whatever a device reset in between undid is
// done again. Host threads that drive different contexts at once take the
// DeviceSetup's lock; within a generation a limit is only ever raised, so a launch
// that found its level done stays valid.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>

namespace luz {

struct DeviceSetup {
    std::mutex m;
    uint64_t generation = 0;   // 0: not done in any generation
    size_t level = 0;          // the largest level done in `generation`
};

// Runs f() unless this generation has done the setup at `level` (>= 1) or above, and
// records `level` when f returns 0 (success). Returns f's result, or 0 when nothing
// was to do. f runs under the lock and must not take the same DeviceSetup.
template <class F>
auto device_setup(DeviceSetup& s, uint64_t generation, size_t level, F&& f) -> decltype(f()) {
    using R = decltype(f());
    std::lock_guard<std::mutex> lock(s.m);
    if (s.generation != generation) {
        s.generation = generation;
        s.level = 0;
    }
    if (level <= s.level) return R(0);
    R r = f();
    if (r == R(0)) s.level = level;
    return r;
}

}  // namespace luz

// Host-only check of luz_gb300/csrc/device_setup.hpp (built and run by
// tests/test_device_setup.py): the setup runs once per level and generation, a failed
// setup is retried, a new generation redoes it, and under concurrent threads every
// caller returns only once its level is in place, with the level never lowered.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "../luz_gb300/csrc/device_setup.hpp"

static int failures = 0;
#define CHECK(c)                                                       \
    do {                                                               \
        if (!(c)) {                                                    \
            std::fprintf(stderr, "%s:%d: %s\n", __FILE__, __LINE__, #c); \
            ++failures;                                                \
        }                                                              \
    } while (0)

int main() {
    using luz::DeviceSetup;
    using luz::device_setup;
    {   // once per generation
        DeviceSetup s;
        int calls = 0;
        for (int i = 0; i < 10; ++i) CHECK(device_setup(s, 1, 1, [&] { ++calls; return 0; }) == 0);
        CHECK(calls == 1);
        CHECK(device_setup(s, 2, 1, [&] { ++calls; return 0; }) == 0);   // a new generation
        CHECK(calls == 2);
    }
    {   // levels only rise; a lower or equal level does nothing
        DeviceSetup s;
        std::vector<size_t> seen;
        for (size_t lv : {10, 5, 20, 20, 15, 30}) device_setup(s, 1, lv, [&] { seen.push_back(lv); return 0; });
        CHECK((seen == std::vector<size_t>{10, 20, 30}));
        seen.clear();
        device_setup(s, 2, 5, [&] { seen.push_back(5); return 0; });   // a new generation starts from 0
        CHECK((seen == std::vector<size_t>{5}));
    }
    {   // a failed setup is not recorded and its result is returned
        DeviceSetup s;
        int calls = 0;
        CHECK(device_setup(s, 1, 1, [&] { ++calls; return 7; }) == 7);
        CHECK(device_setup(s, 1, 1, [&] { ++calls; return 0; }) == 0);
        CHECK(device_setup(s, 1, 1, [&] { ++calls; return 0; }) == 0);
        CHECK(calls == 2);
    }
    {   // threads: each caller finds its level in place when it returns
        DeviceSetup s;
        std::atomic<size_t> attr{0};   // the "device attribute" the setup raises
        std::atomic<int> calls{0}, late{0}, lowered{0};
        std::vector<std::thread> ts;
        for (int t = 0; t < 8; ++t)
            ts.emplace_back([&, t] {
                unsigned x = 12345u + 977u * (unsigned)t;
                for (int i = 0; i < 20000; ++i) {
                    x = x * 1664525u + 1013904223u;
                    const size_t lv = 1 + (x >> 16) % 4096;
                    device_setup(s, 1, lv, [&] {
                        if (lv < attr.load()) ++lowered;
                        attr.store(lv);
                        ++calls;
                        return 0;
                    });
                    if (attr.load() < lv) ++late;
                }
            });
        for (auto& th : ts) th.join();
        CHECK(late.load() == 0);
        CHECK(lowered.load() == 0);
        CHECK(calls.load() <= 4096);
        CHECK(attr.load() <= 4096);
    }
    if (failures) return 1;
    std::puts("ok");
    return 0;
}

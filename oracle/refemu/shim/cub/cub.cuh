// cub stand-in for the host emulation of the reference: the reference's CUB
// helpers (cujson/utils.cu) are not on its parse path; calling one aborts.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstdio>
#include <cstdlib>
namespace cub {
struct DeviceReduce {
    template <typename... A> static int Sum(A&&...) { fprintf(stderr, "cub not emulated\n"); abort(); }
};
struct DeviceScan {
    template <typename... A> static int InclusiveSum(A&&...) { fprintf(stderr, "cub not emulated\n"); abort(); }
};
struct DeviceSelect {
    template <typename... A> static int Flagged(A&&...) { fprintf(stderr, "cub not emulated\n"); abort(); }
};
}  // namespace cub

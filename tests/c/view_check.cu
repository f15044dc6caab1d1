// The checked build's view test on the host (no GPU): a view refuses every
// access outside its logical extent -- rows, columns, negative indices, the
// transposed view's swapped extent, a view moved right by lv_from_col --
// counts it, records the first, and leaves the matrix's memory untouched.
// Compiled with -DCBK_CUDA_CHECKED against cbk_device.cuh. Prints
// "view check ok" and exits 0 when every check holds.
#include <cstdio>
#include <cstring>

#include "cbk_device.cuh"

namespace cbkcuda {
void register_check_reader(CheckReader) {} // no library here: nothing to register with
} // namespace cbkcuda

using cbkdev::host_check_word;

static int fails = 0;
static void expect(bool ok, const char *what)
{
    if (!ok) {
        std::printf("FAILED: %s\n", what);
        ++fails;
    }
}

int main()
{
    // two interleaved 3 x 3 matrices, leading dimension 4 (one padding row)
    double buf[4 * 3 * 2];
    for (int k = 0; k < 24; ++k)
        buf[k] = (double)k;
    double orig[24];
    std::memcpy(orig, buf, sizeof buf);
    const auto A = cbkdev::lv_make<double>(buf + 1, false, 4, 2, 3, 3); // lane 1
    expect(A(2, 1) == buf[1 + (1 * 4 + 2) * 2], "in-range read");
    A(2, 2) = 100.0;
    expect(host_check_word().count == 0, "no count for in-range accesses");
    orig[1 + (2 * 4 + 2) * 2] = 100.0;
    A(3, 0) = -1.0; // the padding row: outside the 3 x 3 matrix
    expect(host_check_word().count == 1, "row past the matrix counted");
    expect(host_check_word().first == (3ull << 32), "first recorded as (3, 0)");
    (void)A(0, 3);
    (void)A(-1, 0);
    expect(host_check_word().count == 3, "column past the matrix and negative row counted");
    const auto At = A.t(); // 3 x 3 transposed: (i, j) -> A(j, i)
    expect(At(0, 2) == A(2, 0) && host_check_word().count == 3, "transposed view in range");
    const auto Ar = cbkdev::lv_make<double>(buf, true, 4, 2, 2, 4); // row-major 2 x 4
    (void)Ar(1, 3);
    expect(host_check_word().count == 3, "row-major view in range");
    (void)Ar(2, 0);
    expect(host_check_word().count == 4, "row-major row past the matrix counted");
    const auto Ac = cbkdev::lv_from_col(A, 1); // columns 1, 2 of A
    expect(Ac(0, 1) == A(0, 2) && host_check_word().count == 4, "moved view in range");
    Ac(0, 2) = -2.0;
    expect(host_check_word().count == 5, "moved view's shrunk extent counted");
    expect(std::memcmp(buf, orig, sizeof buf) == 0, "no refused access touched the matrix");
    if (fails) return 1;
    std::printf("view check ok\n");
    return 0;
}

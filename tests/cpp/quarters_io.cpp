// Reads the harness quarter files with include/gb300_ntt_io.hpp and writes
// them back: quarters_io <in int16 folder> <in int32 folder> <out folder>.
#include <cstdio>
#include <string>

#include "gb300_ntt_io.hpp"

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    const std::string out = argv[3];
    const auto a = gb300ntt::read_quarters<int16_t>(argv[1], 4096, 4);
    gb300ntt::write_quarters(out, a.data(), 4096, 4, "i16");
    const auto b = gb300ntt::read_quarters<int32_t>(argv[2], 2048, 4);
    gb300ntt::write_quarters(out, b.data(), 2048, 4, "i32");
    std::printf("%d %d %d %d\n", (int)a[0], (int)a[4095], (int)b[0], (int)b[2047]);
    return 0;
}

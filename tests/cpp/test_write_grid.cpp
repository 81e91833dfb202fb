// Prints lvr2gb::writeGrid (the HashGrid::saveGrid stream format) for two
// fixed cells; tests/test_cpp_host.py compares it with printf-style %g.
#include <iostream>
#include <vector>

#include "lvr2gb.hpp"

int main() {
    const std::vector<float> centers = {0.5f, -1.25f, 1e-7f, 1234567.0f, 0.1f, -0.0f};
    std::vector<float> tsdf(16);
    for (int i = 0; i < 16; i++) tsdf[i] = (i - 7) * 0.3f;
    lvr2gb::writeGrid(std::cout, centers, tsdf);
    return 0;
}

// Prints the reference's marching-cubes and grid tables, compiled directly
// from the lvr2 headers (include/lvr2/reconstruction/MCTable.hpp,
// FastBoxTables.hpp, FastReconstructionTables.hpp), as one JSON object.
// Test infrastructure: pins the tables used by the oracle and the GPU code.
#include <cstdio>
#include "lvr2/reconstruction/MCTable.hpp"
#include "lvr2/reconstruction/FastBoxTables.hpp"
#include "lvr2/reconstruction/FastReconstructionTables.hpp"

template <int R, int C>
static void dump(const char* name, const int (&t)[R][C], bool last = false) {
    std::printf("\"%s\": [", name);
    for (int r = 0; r < R; r++) {
        std::printf("[");
        for (int c = 0; c < C; c++) std::printf("%d%s", t[r][c], c + 1 < C ? "," : "");
        std::printf("]%s", r + 1 < R ? "," : "");
    }
    std::printf("]%s\n", last ? "" : ",");
}

int main() {
    std::printf("{\n");
    dump("MCTable", lvr2::MCTable);
    dump("neighbor_table", lvr2::neighbor_table);
    dump("neighbor_vertex_table", lvr2::neighbor_vertex_table);
    dump("vertex_edge_table", lvr2::vertex_edge_table);
    dump("shared_vertex_table", lvr2::shared_vertex_table);
    dump("box_creation_table", lvr2::box_creation_table, true);
    std::printf("}\n");
    return 0;
}

// ref_lbvh -- runs lvr2's own CUDA LBVH (LBVHIndex, src/liblvr2/reconstruction/
// cuda/LBVHIndex.cu) unmodified, for the tests' golden vectors and as the GPU
// comparator of the benchmark.  Test infrastructure: it is built by
// oracle/Makefile (target ref-lbvh) from a copy of the lvr2 sources under
// oracle/_ref/ and never linked into the product.
//
//   ref_lbvh jit <K>
//       NVRTC-compiles the two kernels LBVHIndex loads at run time
//       (query_knn_kernel, knn_normals_kernel) and exits; needs no GPU.
//   ref_lbvh run <points.bin> <out_prefix> <K> [<queries.bin>] [--no-normals]
//       points/queries: int64 count, then count x 3 float32.
//       LBVHIndex(1, sort_queries = true, compact = true).build(points), as
//       SearchTreeLBVH builds it (SearchTreeLBVH.tcc:9), then
//       LBVHIndex::kSearch(queries or points, K)  -> <out>_knn_{idx,dist,cnt}.bin
//       a fresh LBVHIndex(1, true, true) built on the points, then
//       LBVHIndex::knn_normals(K)              -> <out>_normals.bin
//       and one JSON line of wall-clock times on stdout.  An <out_prefix>
//       of "-" writes no arrays (timing runs).
//
// Leaf size 1 only.  With a leaf size above 1 (CudaKSearchSurface uses 32,
// CudaKSearchSurface.tcc:20) LBVHIndex::build optimises and compacts the
// tree, and that path wrote to an illegal address on a GB300 (reported at
// the cudaFree of LBVHIndex.cu:289, after compact_tree_kernel).  Read from
// the source: the prefix sums of the m valid flags have m + 1 entries, but
// their host and device buffers are sizeof(unsigned) * m + 1 bytes
// (LBVHIndex.cu:217-218, 249, 253-255), and valid_node reads entry m
// (lbvh_kernels.cu:160-163), so three of its bytes lie past the allocation.
// A wrong entry m makes node m - 1 look valid, compact_tree_kernel then reads
// free_positions one past its end and writes a node to that address.
// Leaf size 1 skips the optimisation and compaction; knn_normals then runs
// on that tree (its kNN, and so its normals, do not depend on the leaf size
// except for the order of equal distances).
//
// Before any query runs, the tree LBVHIndex::build left on the device is
// checked on the host: every node reachable from the root once, both children
// of an internal node valid with matching parent links, the root's parent
// UINT_MAX, leaves covering [0, n) exactly, and the sorted indices a
// permutation.  lvr2's traversal (query.cuh:87-166) follows child and parent
// links without bounds checks, so a malformed tree is reported and no query is
// launched on it.
//
// knn_normals frees m_d_sorted_indices through an alias (LBVHIndex.cu:723)
// and the destructor frees it again, so each knn_normals call gets its own
// LBVHIndex, destroyed right after the call with no device allocation in
// between.
#include <chrono>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

// lvr2's LBVH sources, compiled with this driver as one translation unit:
// lbvh_kernels.cu calls device functions that morton_code.cu defines, which
// needs whole-program device code (or relocatable device code and a device
// link step).
#include "LBVHIndex.cu"
#include "lbvh/lbvh_kernels.cu"
#include "lbvh/morton_code.cu"
#include "lbvh/normals_kernel.cu"

using lvr2::lbvh::BVHNode;
using lvr2::lbvh::LBVHIndex;

namespace {

__global__ void probe_kernel(int* out) { *out = 42; }

// A launch of a trivial kernel of this file: tells a broken CUDA set-up from
// a failure inside the reference's calls.
bool probe_launch() {
    int* d = nullptr;
    int h = 0;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return false;
    probe_kernel<<<1, 1>>>(d);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::fprintf(stderr, "probe launch: %s\n", cudaGetErrorString(e));
        return false;
    }
    cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return h == 42;
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

std::vector<float> read_points(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    int64_t n = 0;
    if (std::fread(&n, sizeof(n), 1, f) != 1 || n < 0) { std::fprintf(stderr, "bad header in %s\n", path); std::exit(2); }
    std::vector<float> v(size_t(n) * 3);
    if (n && std::fread(v.data(), sizeof(float), v.size(), f) != v.size()) {
        std::fprintf(stderr, "short read in %s\n", path);
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <typename T>
void write_array(const std::string& path, const T* data, size_t count) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::fprintf(stderr, "cannot write %s\n", path.c_str()); std::exit(2); }
    std::fwrite(data, sizeof(T), count, f);
    std::fclose(f);
}

// Host check of the tree LBVHIndex::build left on the device (see the file
// header).  Returns an empty string when the tree is well formed.
std::string check_tree(const LBVHIndex& t, size_t n) {
    const unsigned nn = t.m_num_nodes;
    const unsigned root = t.m_root_node[0];
    if (nn == 0 || root >= nn) return "root index out of range";
    std::vector<BVHNode> nodes(nn);
    if (cudaMemcpy(nodes.data(), t.m_d_nodes, sizeof(BVHNode) * nn, cudaMemcpyDeviceToHost) != cudaSuccess)
        return "cannot read the nodes";
    std::vector<unsigned> perm(n);
    if (cudaMemcpy(perm.data(), t.m_d_sorted_indices, sizeof(unsigned) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return "cannot read the sorted indices";
    std::vector<char> seen_idx(n, 0);
    for (unsigned v : perm) {
        if (v >= n || seen_idx[v]) return "sorted indices are not a permutation";
        seen_idx[v] = 1;
    }
    if (nodes[root].parent != UINT_MAX) return "root has a parent";
    const BVHNode& r = nodes[root];
    if (r.child_left == UINT_MAX || r.child_right == UINT_MAX) return "root is a leaf";
    std::vector<char> seen(nn, 0), covered(n, 0);
    std::vector<unsigned> stack{root};
    size_t leaf_points = 0;
    while (!stack.empty()) {
        const unsigned i = stack.back();
        stack.pop_back();
        if (seen[i]) return "node reached twice";
        seen[i] = 1;
        const BVHNode& d = nodes[i];
        const bool l0 = d.child_left == UINT_MAX, l1 = d.child_right == UINT_MAX;
        if (l0 != l1) return "node with one child";
        if (l0) {
            if (d.range_left > d.range_right || d.range_right >= n) return "leaf range out of bounds";
            for (unsigned p = d.range_left; p <= d.range_right; p++) {
                if (covered[p]) return "leaves overlap";
                covered[p] = 1;
            }
            leaf_points += size_t(d.range_right - d.range_left) + 1;
            continue;
        }
        for (unsigned c : {d.child_left, d.child_right}) {
            if (c >= nn) return "child index out of range";
            if (nodes[c].parent != i) return "parent link mismatch";
            stack.push_back(c);
        }
    }
    if (leaf_points != n) return "leaves do not cover every point";
    return "";
}

int usage() {
    std::fprintf(stderr,
                 "usage: ref_lbvh jit <K>\n"
                 "       ref_lbvh run <points.bin> <out_prefix> <K> [<queries.bin>] [--no-normals]\n");
    return 2;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return usage();
    const std::string mode = argv[1];
    if (mode == "jit") {
        const int K = std::atoi(argv[2]);
        // Never destroyed: the default constructor leaves the device pointers
        // that ~LBVHIndex frees uninitialised (LBVHIndex.cu:26-38, 60-72).
        LBVHIndex& probe = *new LBVHIndex();
        double t0 = now_ms();
        std::string ptx;
        const std::string dir = LBVH_KERNEL_DIR;
        for (const char* name : {"query_knn_kernels.cu", "knn_normals_kernel.cu"}) {
            FILE* f = std::fopen((dir + "/" + name).c_str(), "rb");
            if (!f) { std::fprintf(stderr, "missing %s\n", name); return 1; }
            std::string src;
            char buf[4096];
            size_t got;
            while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) src.append(buf, got);
            std::fclose(f);
            probe.getPtxFromCuString(ptx, name, src.c_str(), K);
            if (ptx.empty()) return 1;
        }
        std::printf("{\"jit\": \"ok\", \"K\": %d, \"ms\": %.1f}\n", K, now_ms() - t0);
        return 0;
    }
    if (mode != "run" || argc < 5) return usage();
    std::vector<float> pts = read_points(argv[2]);
    const std::string out = argv[3];
    const int K = std::atoi(argv[4]);
    const int leaf = 1;  // see the file header: no optimised / compacted trees
    bool normals = true;
    std::vector<float> qs;
    bool own_queries = false;
    for (int a = 5; a < argc; a++) {
        if (std::strcmp(argv[a], "--no-normals") == 0) normals = false;
        else { qs = read_points(argv[a]); own_queries = true; }
    }
    const size_t n = pts.size() / 3;
    if (K < 1 || leaf < 1 || n < size_t(4 * (leaf > K ? leaf : K))) {
        std::fprintf(stderr, "need K >= 1, leaf >= 1 and at least 4 * max(K, leaf) points\n");
        return 2;
    }
    cudaFree(nullptr);
    if (!probe_launch()) {
        std::fprintf(stderr, "CUDA set-up check failed\n");
        return 5;
    }
    double t0 = now_ms();
    std::string report = "{";
    {
        LBVHIndex tree(leaf, true, true);
        tree.build(pts.data(), n);
        cudaDeviceSynchronize();
        const double t_build = now_ms() - t0;
        const std::string bad = check_tree(tree, n);
        if (!bad.empty()) {
            std::printf("{\"tree\": \"malformed: %s\", \"leaf\": %d}\n", bad.c_str(), leaf);
            return 3;
        }
        const float* q = own_queries ? qs.data() : pts.data();
        const size_t nq = own_queries ? qs.size() / 3 : n;
        std::vector<unsigned> idx(nq * size_t(K)), cnt(nq);
        std::vector<float> dist(nq * size_t(K));
        std::vector<float> qcopy(q, q + 3 * nq);  // kSearch takes a non-const pointer
        double t1 = now_ms();
        tree.kSearch(qcopy.data(), nq, K, cnt.data(), idx.data(), dist.data());
        cudaError_t e = cudaDeviceSynchronize();
        const double t_knn = now_ms() - t1;
        if (e != cudaSuccess) {
            std::fprintf(stderr, "kSearch: %s\n", cudaGetErrorString(e));
            return 4;
        }
        // kSearch frees its query buffer twice (process_queries_dev_ptr, then
        // process_queries, LBVHIndex.cu:460 and :578).  The second cudaFree
        // returns cudaErrorInvalidValue, which stays the runtime's last error;
        // the next LBVHIndex::build checks cudaPeekAtLastError
        // (LBVHIndex.cu:117) and would exit on it.  Read and clear it here.
        const cudaError_t after_ksearch = cudaGetLastError();
        if (out != "-") {
            write_array(out + "_knn_idx.bin", idx.data(), idx.size());
            write_array(out + "_knn_dist.bin", dist.data(), dist.size());
            write_array(out + "_knn_cnt.bin", cnt.data(), cnt.size());
        }
        char buf[320];
        std::snprintf(buf, sizeof(buf),
                      "\"n\": %zu, \"nq\": %zu, \"K\": %d, \"leaf\": %d, \"build_ms\": %.2f, \"ksearch_ms\": %.2f, "
                      "\"ksearch_last_error\": \"%s\"",
                      n, nq, K, leaf, t_build, t_knn, cudaGetErrorString(after_ksearch));
        report += buf;
    }
    if (normals) {
        std::vector<float> nrm(3 * n);
        double t2 = now_ms();
        {
            LBVHIndex tree(leaf, true, true);
            tree.build(pts.data(), n);
            cudaDeviceSynchronize();
            const double t_b = now_ms() - t2;
            const std::string bad = check_tree(tree, n);
            if (!bad.empty()) {
                std::printf("{\"tree\": \"malformed: %s\", \"leaf\": %d}\n", bad.c_str(), leaf);
                return 3;
            }
            double t3 = now_ms();
            tree.knn_normals(K, nrm.data(), n);
            cudaError_t e = cudaDeviceSynchronize();
            const double t_nrm = now_ms() - t3;
            if (e != cudaSuccess) {
                std::fprintf(stderr, "knn_normals: %s\n", cudaGetErrorString(e));
                return 4;
            }
            char buf[160];
            std::snprintf(buf, sizeof(buf), ", \"normals_build_ms\": %.2f, \"knn_normals_ms\": %.2f", t_b, t_nrm);
            report += buf;
        }  // destroyed here: its second free of the aliased index array meets no new allocation
        if (out != "-") write_array(out + "_normals.bin", nrm.data(), nrm.size());
    }
    cudaError_t e = cudaDeviceSynchronize();
    report += "}";
    std::printf("%s\n", report.c_str());
    return e == cudaSuccess ? 0 : 4;
}

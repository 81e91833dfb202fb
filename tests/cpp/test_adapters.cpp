// C++ host interface (lvr2_gb300/cpp/lvr2gb.hpp) on a GPU: the lvr2-style
// call sequence of lvr2_reconstruct and CudaSurface through liblvrgb.so.
// Exit status 0 = all checks passed.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "lvr2gb.hpp"

static int failures = 0;
#define EXPECT(cond)                                                   \
    do {                                                               \
        if (!(cond)) {                                                 \
            std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
            failures++;                                                \
        }                                                              \
    } while (0)

int main() {
    // noisy sphere around (0.5, 0.5, 0.5)
    std::mt19937 rng(7);
    std::normal_distribution<float> g(0.0f, 1.0f);
    const size_t n = 30000;
    std::vector<float> xyz(3 * n);
    for (size_t i = 0; i < n; i++) {
        float v[3] = {g(rng), g(rng), g(rng)};
        float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int a = 0; a < 3; a++) xyz[3 * i + a] = 0.5f + 0.3f * v[a] / l + 1e-3f * g(rng);
    }
    lvr2gb::Surface s(xyz.data(), n, 10, 10, 5, 3);
    auto bb = s.getBoundingBox();
    EXPECT(bb[0].x < 0.25f && bb[1].x > 0.75f);
    s.setFlipPoint(lvr2gb::Vec3{0.5f, 0.5f, 0.5f});
    s.calculateSurfaceNormals();
    auto nrm = s.normals();
    EXPECT(nrm.size() == 3 * n);
    size_t inward = 0;
    for (size_t i = 0; i < n; i++) {
        float len = std::sqrt(nrm[3 * i] * nrm[3 * i] + nrm[3 * i + 1] * nrm[3 * i + 1] + nrm[3 * i + 2] * nrm[3 * i + 2]);
        EXPECT(std::fabs(len - 1.0f) < 1e-4f);
        float d = 0;
        for (int a = 0; a < 3; a++) d += nrm[3 * i + a] * (0.5f - xyz[3 * i + a]);
        inward += d > 0;
    }
    EXPECT(inward > n * 99 / 100);

    // SearchTree::kSearch against brute force for a few queries
    for (size_t qi = 0; qi < n; qi += 997) {
        lvr2gb::Vec3 q{xyz[3 * qi], xyz[3 * qi + 1], xyz[3 * qi + 2]};
        std::vector<size_t> idx;
        std::vector<float> dist;
        int c = s.kSearch(q, 8, idx, dist);
        EXPECT(c == 8);
        EXPECT(idx[0] == qi && dist[0] == 0.0f);
        float worst = dist[7];
        size_t closer = 0;
        for (size_t j = 0; j < n; j++) {
            float dx = q.x - xyz[3 * j], dy = q.y - xyz[3 * j + 1], dz = q.z - xyz[3 * j + 2];
            if (std::sqrt(dx * dx + dy * dy + dz * dz) < worst * 0.999f) closer++;
        }
        EXPECT(closer <= 7);
    }

    // PointsetSurface::distance inside / outside the sphere (normals point inward)
    auto din = s.distance(lvr2gb::Vec3{0.5f, 0.5f, 0.5f + 0.28f});
    auto dout = s.distance(lvr2gb::Vec3{0.5f, 0.5f, 0.5f + 0.32f});
    EXPECT(din.first > 0.0f && dout.first < 0.0f);

    // grid + marching cubes: every face index is a valid vertex
    lvr2gb::GridOptions go;
    go.voxelsize = 0.02f;
    lvr2gb::Mesh m = s.reconstruct(go);
    EXPECT(m.info.faces > 1000 && m.info.vertices > 500);
    for (uint32_t f : m.faces) EXPECT(f < uint32_t(m.info.vertices));
    // vertex normals: unit length, along the sphere's radius
    EXPECT(m.vertexNormals.size() == m.vertices.size());
    size_t radial = 0;
    for (size_t v = 0; v < size_t(m.info.vertices); v++) {
        const float* p = &m.vertices[3 * v];
        const float* q = &m.vertexNormals[3 * v];
        const float rx = p[0] - 0.5f, ry = p[1] - 0.5f, rz = p[2] - 0.5f;
        const float rl = std::sqrt(rx * rx + ry * ry + rz * rz);
        EXPECT(std::fabs(std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]) - 1.0f) < 1e-5f);
        radial += std::fabs(q[0] * rx + q[1] * ry + q[2] * rz) > 0.9f * rl;
    }
    EXPECT(radial > size_t(0.95 * double(m.info.vertices)));

    // HashGrid::toPointBuffer of the kept cells (what -g writes): every corner
    // of a kept cell is valid, so its distance is finite
    std::vector<float> centers, tsdf;
    s.cellTsdf(centers, tsdf);
    EXPECT(m.info.cells_valid > 0 && centers.size() == size_t(3 * m.info.cells_valid) &&
           tsdf.size() == size_t(8 * m.info.cells_valid));
    size_t finite = 0;
    for (float d : tsdf) finite += std::isfinite(d) ? 1 : 0;
    EXPECT(finite == tsdf.size());

    // CudaKSearchSurface (--pcm LBVH_CUDA): unit normals pointing toward (1e6, 1e6, 1e6)
    {
        lvr2gb::CudaKSearchSurface ks(xyz.data(), n, 20);
        ks.calculateSurfaceNormals();
        auto kn = ks.normals();
        EXPECT(kn.size() == 3 * n);
        size_t unit = 0, toward = 0;
        for (size_t i = 0; i < n; i++) {
            const float* q = &kn[3 * i];
            const float* p = &xyz[3 * i];
            unit += std::fabs(std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]) - 1.0f) < 1e-5f;
            toward += q[0] * (1e6f - p[0]) + q[1] * (1e6f - p[1]) + q[2] * (1e6f - p[2]) >= -1.0f;
        }
        EXPECT(unit == n && toward == n);
        bool threw = false;
        try {
            ks.distance(lvr2gb::Vec3{0, 0, 0});
        } catch (const std::runtime_error&) {
            threw = true;
        }
        EXPECT(threw);
    }

    // the CudaSurface call sequence of lvr2_reconstruct --useGPU (Main.cpp:353-379)
    std::shared_ptr<float[]> pts(new float[3 * n]);
    std::copy(xyz.begin(), xyz.end(), pts.get());
    lvr2gb::CudaSurface gs(pts, n);
    gs.setKn(10);
    gs.setKi(10);
    gs.setFlippoint(0.5f, 0.5f, 0.5f);
    gs.calculateNormals();
    std::shared_ptr<float[]> out(new float[3 * n]);
    gs.getNormals(out);
    size_t same = 0;
    for (size_t i = 0; i < 3 * n; i++) same += out[i] == nrm[i];
    EXPECT(same == 3 * n);  // same configuration (kn 10, ki 10, PCA) -> identical normals
    std::vector<lvr2gb::QueryPoint> qp(3);
    qp[0].m_position = {0.5f, 0.5f, 0.78f};
    qp[1].m_position = {0.5f, 0.5f, 0.82f};
    qp[2].m_position = {0.5f, 0.5f, 0.5f};
    gs.distances(qp, 0.02f);
    EXPECT(!qp[0].m_invalid && !qp[1].m_invalid && qp[2].m_invalid);
    // setMethod("RANSAC"): calcPlaneRANSAC (nem 1); unit normals, or the null
    // normal where a degenerate candidate plane wins
    gs.setMethod("RANSAC");
    gs.calculateNormals();
    gs.getNormals(out);
    size_t unit = 0;
    for (size_t i = 0; i < n; i++) {
        const float* v = &out[3 * i];
        const float len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        unit += std::fabs(len - 1.0f) < 1e-5f || len == 0.0f;
    }
    EXPECT(unit == n);

    if (failures) {
        std::fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    std::printf("C++ adapter checks passed: %lld faces\n", (long long)m.info.faces);
    return 0;
}

// lvr2gb.hpp -- C++ host interface over liblvrgb.so (include/lvrgb.h),
// mirroring the lvr2 classes a reconstruction uses:
//
//   lvr2gb::Surface      AdaptiveKSearchSurface / PointsetSurface
//                        (include/lvr2/reconstruction/AdaptiveKSearchSurface.hpp:99-107,
//                         PointsetSurface.hpp:61-166) and its search tree
//                        (SearchTree.hpp:71-125)
//   lvr2gb::CudaSurface  the GpuSurface API
//                        (include/lvr2/reconstruction/cuda/CudaSurface.hpp:70-158)
//   lvr2gb::QueryPoint   QueryPoint<BaseVecT> (QueryPoint.hpp:47-93)
//
// Same parameter names, defaults and call order as lvr2; errors throw
// std::runtime_error as CudaSurface does (CudaSurface.hpp:53-62).  Header only;
// link with -llvrgb.
#pragma once
#include <lvrgb.h>

#include <array>
#include <cstdint>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace lvr2gb {

inline void check(lvrgb_status s, const char* what) {
    if (s != LVRGB_OK) throw std::runtime_error(std::string(what) + ": " + lvrgb_last_error());
}

// HashGrid::saveGrid (HashGrid.tcc:380-397): the cell count, then each cell's
// centre and the distances at its 8 corners, every number written with
// operator<< and no separator, as lvr2_reconstruct -g writes fastgrid.grid
// (Main.cpp:604-607).  centers: 3 per cell, tsdf: 8 per cell.
inline void writeGrid(std::ostream& out, const std::vector<float>& centers, const std::vector<float>& tsdf) {
    const unsigned long cells = static_cast<unsigned long>(centers.size() / 3);
    if (tsdf.size() != 8 * size_t(cells)) throw std::runtime_error("writeGrid: need 8 distances per cell");
    out << cells;
    for (size_t i = 0; i < cells; i++) {
        out << centers[3 * i] << centers[3 * i + 1] << centers[3 * i + 2];
        for (size_t j = 0; j < 8; j++) out << tsdf[8 * i + j];
    }
}

struct Vec3 {
    float x = 0, y = 0, z = 0;
};

// QueryPoint<BaseVecT>: a grid vertex with its distance and invalid flag.
struct QueryPoint {
    Vec3 m_position;
    float m_distance = 0;
    bool m_invalid = false;
};

struct Mesh {
    std::vector<float> vertices;  // V x 3
    std::vector<uint32_t> faces;  // F x 3 vertex indices
    // calcVertexNormals(mesh, calcFaceNormals(mesh), surface), as handed to the
    // finalizer (src/tools/lvr2_reconstruct/Main.cpp:855-873); V x 3
    std::vector<float> vertexNormals;
    // calcColorFromPointCloud (ColorAlgorithms.tcc:43-92), V x 3; empty for a cloud without colours
    std::vector<uint8_t> vertexColors;
    lvrgb_mesh_info info{};
};

// lvr2_reconstruct's grid options (--voxelsize, --intersections, --noExtrusion,
// --decomposition; src/tools/lvr2_reconstruct/Options.cpp:69-74).
struct GridOptions {
    float voxelsize = 10.0f;
    int intersections = -1;
    bool extrude = true;
    std::string decomposition = "PMC";
    // PMC meshes get BilinearFastBox::optimizePlanarFaces with kc = 5, as in
    // FastReconstruction::getMesh (FastReconstruction.tcc:158-168)
    bool optimizePlanarFaces = true;
};

class Surface {
  public:
    // AdaptiveKSearchSurface(buffer, searchTreeName, kn = 10, ki = 10, kd = 10,
    // calcMethod = 0): the flip point defaults to the bounding-box centroid.
    Surface(const float* xyz, size_t n, int kn = 10, int ki = 10, int kd = 10, int calcMethod = 0, int device = 0) {
        lvrgb_surface_config cfg;
        lvrgb_surface_config_default(&cfg);
        cfg.kn = kn;
        cfg.ki = ki;
        cfg.kd = kd;
        cfg.nem = calcMethod;
        cfg.flip_set = 0;
        cfg.device = device;
        check(lvrgb_surface_create(&cfg, xyz, int64_t(n), 0, nullptr, &h_), "lvrgb_surface_create");
        n_ = n;
    }
    Surface(const Surface&) = delete;
    Surface& operator=(const Surface&) = delete;
    ~Surface() {
        if (h_) lvrgb_surface_destroy(h_);
    }

    size_t numPoints() const { return n_; }
    void setKn(int k) { check(lvrgb_surface_set_k(h_, k, -1, -1), "setKn"); }
    void setKi(int k) { check(lvrgb_surface_set_k(h_, -1, k, -1), "setKi"); }
    void setKd(int k) { check(lvrgb_surface_set_k(h_, -1, -1, k), "setKd"); }
    void setFlipPoint(const Vec3& p) { check(lvrgb_surface_set_flip_point(h_, p.x, p.y, p.z), "setFlipPoint"); }
    void setCalcMethod(int nem) { check(lvrgb_surface_set_method(h_, nem), "setCalcMethod"); }
    // The scan poses of AdaptiveKSearchSurface's posefile argument (x y z each).
    void setScanPoses(const std::vector<float>& poses) {
        check(lvrgb_surface_set_scan_poses(h_, poses.data(), int64_t(poses.size() / 3)), "setScanPoses");
    }

    // getBoundingBox(): min, max, centroid
    std::array<Vec3, 3> getBoundingBox() const {
        float b[9];
        check(lvrgb_surface_bounding_box(h_, b), "getBoundingBox");
        return {Vec3{b[0], b[1], b[2]}, Vec3{b[3], b[4], b[5]}, Vec3{b[6], b[7], b[8]}};
    }

    // calculateSurfaceNormals(): estimation and, when ki > 0, interpolation.
    void calculateSurfaceNormals() { check(lvrgb_calculate_normals(h_, nullptr), "calculateSurfaceNormals"); }
    void interpolateSurfaceNormals() { check(lvrgb_interpolate_normals(h_, nullptr), "interpolateSurfaceNormals"); }

    // The "normals" channel of the point buffer (n x 3, input order).
    std::vector<float> normals() const {
        std::vector<float> out(3 * n_);
        check(lvrgb_get_normals(h_, out.data(), 0, nullptr), "normals");
        return out;
    }
    void setNormals(const float* normals) { check(lvrgb_set_normals(h_, normals, 0, nullptr), "setNormals"); }

    // PointsetSurface::distance: (projected, Euclidean).
    std::pair<float, float> distance(const Vec3& v) const {
        float q[3] = {v.x, v.y, v.z}, p = 0, e = 0;
        check(lvrgb_distance(h_, q, 1, &p, &e, 0, nullptr), "distance");
        return {p, e};
    }
    // Batched distance for many positions.
    void distances(const std::vector<Vec3>& q, std::vector<float>& projected, std::vector<float>& euclidean) const {
        projected.resize(q.size());
        euclidean.resize(q.size());
        check(lvrgb_distance(h_, &q[0].x, int64_t(q.size()), projected.data(), euclidean.data(), 0, nullptr),
              "distances");
    }
    // PointsetGrid::calcDistanceValues for given query points.
    void calcDistanceValues(std::vector<QueryPoint>& qp, float voxelsize) const {
        std::vector<float> pos(3 * qp.size()), d(qp.size());
        std::vector<uint8_t> inv(qp.size());
        for (size_t i = 0; i < qp.size(); i++) {
            pos[3 * i] = qp[i].m_position.x;
            pos[3 * i + 1] = qp[i].m_position.y;
            pos[3 * i + 2] = qp[i].m_position.z;
        }
        check(lvrgb_grid_distances(h_, pos.data(), int64_t(qp.size()), voxelsize, d.data(), inv.data(), 0, nullptr),
              "calcDistanceValues");
        for (size_t i = 0; i < qp.size(); i++) {
            qp[i].m_distance = d[i];
            qp[i].m_invalid = inv[i] != 0;
        }
    }
    // PointsetSurface::getInterpolatedNormal: the mean of (0, 1, 0) and the ki
    // nearest normals, not normalised (as lvr2 returns it)
    Vec3 getInterpolatedNormal(const Vec3& v) const {
        float q[3] = {v.x, v.y, v.z}, o[3];
        check(lvrgb_interpolated_normal(h_, q, 1, o, 0, nullptr), "getInterpolatedNormal");
        return Vec3{o[0], o[1], o[2]};
    }

    // SearchTree::kSearch(qp, k, indices, distances): returns the count found.
    int kSearch(const Vec3& qp, int k, std::vector<size_t>& indices, std::vector<float>& distances) const {
        std::vector<uint32_t> idx(static_cast<size_t>(k));
        std::vector<float> dist(static_cast<size_t>(k));
        int32_t cnt = 0;
        float q[3] = {qp.x, qp.y, qp.z};
        check(lvrgb_knn(h_, q, 1, k, idx.data(), dist.data(), &cnt, 0, nullptr), "kSearch");
        indices.assign(idx.begin(), idx.begin() + cnt);
        distances.assign(dist.begin(), dist.begin() + cnt);
        return cnt;
    }
    // SearchTree::kSearchParallel(query, n, k, indices, distances): n x k rows.
    void kSearchParallel(const Vec3* query, int n, int k, std::vector<size_t>& indices,
                         std::vector<float>& distances) const {
        std::vector<uint32_t> idx(size_t(n) * size_t(k));
        distances.resize(size_t(n) * size_t(k));
        check(lvrgb_knn(h_, &query[0].x, n, k, idx.data(), distances.data(), nullptr, 0, nullptr), "kSearchParallel");
        indices.assign(idx.begin(), idx.end());
    }

    // createGridAndReconstruction + getMesh (src/tools/lvr2_reconstruct/Main.cpp:404-453, 587-610)
    Mesh reconstruct(const GridOptions& o) {
        lvrgb_grid_config g;
        g.is_voxelsize = o.intersections <= 0 ? 1 : 0;
        g.resolution = g.is_voxelsize ? o.voxelsize : float(o.intersections);
        g.extrude = o.extrude ? 1 : 0;
        if (o.decomposition == "MC") {
            g.decomposition = 0;
        } else if (o.decomposition == "PMC") {
            g.decomposition = 1;
        } else {
            throw std::runtime_error("decomposition " + o.decomposition + " is not supported (MC, PMC)");
        }
        Mesh m;
        check(lvrgb_reconstruct(h_, &g, &m.info, nullptr), "reconstruct");
        mesh_vertices_ = m.info.vertices;
        grid_cells_ = m.info.cells_valid;
        if (g.decomposition == 1 && o.optimizePlanarFaces)
            check(lvrgb_optimize_planar_faces(h_, 5, nullptr, nullptr), "optimizePlanarFaces");
        m.vertices.resize(size_t(3 * m.info.vertices));
        m.faces.resize(size_t(3 * m.info.faces));
        check(lvrgb_get_mesh(h_, m.vertices.data(), m.faces.data(), nullptr, 0, nullptr), "getMesh");
        m.vertexNormals.resize(m.vertices.size());
        check(lvrgb_mesh_vertex_normals(h_, m.vertexNormals.data(), 0, nullptr), "calcVertexNormals");
        return m;
    }

    // calcColorFromPointCloud of the last mesh: each vertex takes its nearest
    // point's colour (pointColors: n x 3 bytes, input order).
    std::vector<uint8_t> vertexColors(const std::vector<uint8_t>& pointColors) const {
        if (pointColors.size() != 3 * n_) throw std::runtime_error("vertexColors: need 3 bytes per point");
        std::vector<uint8_t> out(size_t(3 * mesh_vertices_));
        check(lvrgb_mesh_vertex_colors(h_, pointColors.data(), 3, out.data(), 0, nullptr), "vertexColors");
        return out;
    }

    // HashGrid::toPointBuffer of the last grid (culled cells in lattice-key
    // order): centres (3 per cell) and corner distances (8 per cell).
    void cellTsdf(std::vector<float>& centers, std::vector<float>& tsdf) const {
        centers.resize(size_t(3 * grid_cells_));
        tsdf.resize(size_t(8 * grid_cells_));
        check(lvrgb_get_cell_tsdf(h_, centers.data(), tsdf.data(), 0, nullptr), "cellTsdf");
    }

    lvrgb_surface handle() const { return h_; }

  private:
    lvrgb_surface h_ = nullptr;
    size_t n_ = 0;
    int64_t mesh_vertices_ = 0;  // vertices of the last reconstruct()
    int64_t grid_cells_ = 0;     // cells kept by the last reconstruct()
};

// CudaKSearchSurface (include/lvr2/reconstruction/CudaKSearchSurface.hpp,
// .tcc:12-65; --pcm LBVH_CUDA): normals by the LBVH comparator's fit (nem 4)
// with k = kn (default 50), flipped toward its fixed point (1e6, 1e6, 1e6),
// without interpolation; distance() is not provided, as in lvr2.
class CudaKSearchSurface {
  public:
    CudaKSearchSurface(const float* xyz, size_t n, size_t k = 50, int device = 0)
        : s_(xyz, n, int(k), 0, 5, 4, device) {
        s_.setFlipPoint(Vec3{1e6f, 1e6f, 1e6f});
    }
    void setKn(int k) { s_.setKn(k); }
    void calculateSurfaceNormals() { s_.calculateSurfaceNormals(); }
    // The "normals" channel (n x 3, input order).
    std::vector<float> normals() const { return s_.normals(); }
    std::pair<float, float> distance(const Vec3&) const {
        throw std::runtime_error("Do not use this function!");
    }
    lvrgb_surface handle() const { return s_.handle(); }

  private:
    Surface s_;
};

// The GpuSurface API of lvr2 (CudaSurface.hpp:70-158) over the same handle.
class CudaSurface {
  public:
    CudaSurface(std::shared_ptr<float[]>& points, size_t num_points, int device = 0)
        : s_(points.get(), num_points, 10, 10, 10, 3, device), n_(num_points) {}
    void calculateNormals() { s_.calculateSurfaceNormals(); }
    void interpolateNormals() { s_.interpolateSurfaceNormals(); }
    void getNormals(std::shared_ptr<float[]> output_normals) {
        auto v = s_.normals();
        std::copy(v.begin(), v.end(), output_normals.get());
    }
    void setKn(int kn) { s_.setKn(kn); }
    void setKi(int ki) { s_.setKi(ki); }
    void setKd(int kd) { s_.setKd(kd); }
    void setFlippoint(float x, float y, float z) { s_.setFlipPoint(Vec3{x, y, z}); }
    // "PCA" -> nem 3; "RANSAC" -> nem 1 (calcPlaneRANSAC)
    void setMethod(const std::string& method) { s_.setCalcMethod(method == "RANSAC" ? 1 : 3); }
    void setReconstructionMode(bool) {}
    void distances(std::vector<QueryPoint>& query_points, float voxel_size) {
        s_.calcDistanceValues(query_points, voxel_size);
    }
    void freeGPU() {}
    Surface& surface() { return s_; }

  private:
    Surface s_;
    size_t n_;
};

}  // namespace lvr2gb

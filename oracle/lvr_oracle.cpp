/*
 * lvr_oracle.cpp -- CPU restatement of the lvr2 reconstruction hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle that the GPU implementation's tests
 * compare against, and the timed CPU baseline.  Nothing in the product
 * (lvr2_gb300/, liblvrgb.so) links or calls this file.
 *
 * Parity status: the reference's CPU path cannot be compiled in this
 * environment (it needs Eigen, Boost and FLANN) and the reference ships no
 * tests, golden vectors or fixtures for this path, so the arithmetic below is
 * "parity unpinned": it is a line-by-line restatement of the cited reference
 * code, not checked against reference outputs.  The marching-cubes and grid
 * tables are pinned: tests/test_tables.py compares them with the reference
 * headers compiled by oracle/Makefile.
 *
 * Compile with -ffp-contract=off: every float expression is evaluated in the
 * order written, without fused multiply-add, like the reference built for
 * generic x86-64.
 *
 * Followed reference files (paths inside the lvr2 tree):
 *   include/lvr2/algorithm/KDTree.tcc:48-313        kd-tree build and kNN
 *   include/lvr2/algorithm/KDTree.tcc:317-375       SearchKDTree
 *   include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:158-290  normals
 *   include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:293-335  interpolation
 *   include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:337-350  boundingBoxOK
 *   include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:414-457  distance
 *   include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:467-673  plane fits
 *   include/lvr2/reconstruction/AdaptiveKSearchSurface.tcc:689-781  RANSAC plane fit
 *   include/lvr2/reconstruction/PointsetSurface.tcc:39-74           bbox, getInterpolatedNormal
 *   include/lvr2/geometry/BaseVector.tcc, Normal.tcc, BoundingBox.tcc:158-252
 *   include/lvr2/reconstruction/HashGrid.tcc:48-80, 235-378, HashGrid.hpp:263-287
 *   include/lvr2/reconstruction/PointsetGrid.tcc:41-185
 *   include/lvr2/reconstruction/FastBox.tcc:84-269, BilinearFastBox.tcc:55-138
 *   include/lvr2/reconstruction/FastReconstruction.tcc:47-66
 */
#include "lvr_oracle.h"

#include <algorithm>
#include <random>
#include <functional>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <queue>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ------------------------------------------------------------------------ */
/* BaseVector<float> / Normal<float> (BaseVector.tcc, Normal.tcc)           */
/* ------------------------------------------------------------------------ */
struct V3 {
    float x = 0, y = 0, z = 0;
    V3() = default;
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
    float dot(const V3& o) const { return x * o.x + y * o.y + z * o.z; }
    float length() const { return std::sqrt(x * x + y * y + z * z); }
    V3 cross(const V3& o) const {
        return V3(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
    }
    // BaseVector::normalize(): the null vector is left unchanged.
    void normalize() {
        if (!(x == 0 && y == 0 && z == 0)) {
            float len = length();
            x /= len; y /= len; z /= len;
        }
    }
    V3 normalized() const { V3 r = *this; r.normalize(); return r; }
    bool operator==(const V3& o) const { return x == o.x && y == o.y && z == o.z; }
};

// BoundingBox<BaseVector<float>> (BoundingBox.tcc:45-53, 198-252)
struct BBox {
    V3 mn{FLT_MAX, FLT_MAX, FLT_MAX};
    V3 mx{-FLT_MAX, -FLT_MAX, -FLT_MAX};
    V3 centroid;
    void expand(const V3& v) {
        mn.x = std::min(v.x, mn.x); mn.y = std::min(v.y, mn.y); mn.z = std::min(v.z, mn.z);
        mx.x = std::max(v.x, mx.x); mx.y = std::max(v.y, mx.y); mx.z = std::max(v.z, mx.z);
        centroid = V3(mn.x + 0.5f * xs(), mn.y + 0.5f * ys(), mn.z + 0.5f * zs());
    }
    float xs() const { return mx.x - mn.x; }
    float ys() const { return mx.y - mn.y; }
    float zs() const { return mx.z - mn.z; }
    bool contains(const V3& v) const {
        return (mn.x <= v.x && mx.x >= v.x) && (mn.y <= v.y && mx.y >= v.y) &&
               (mn.z <= v.z && mx.z >= v.z);
    }
    float longest() const { return std::max({xs(), ys(), zs()}); }
};

/* ------------------------------------------------------------------------ */
/* kd-tree (KDTree.tcc)                                                      */
/* ------------------------------------------------------------------------ */
struct IPoint {  // IndexedPoint<BaseVector<float>> (KDTree.hpp:224-233)
    float p[3];
    uint32_t index;
};

struct KDNode {
    bool leaf;
    unsigned axis;
    double split;
    size_t start, end;  // leaf range
    std::unique_ptr<KDNode> lesser, greater;
};

static inline float d2_canonical(const float* q, const float* p) {
    float dx = q[0] - p[0];
    float dy = q[1] - p[1];
    float dz = q[2] - p[2];
    float a = dx * dx;
    float b = dy * dy;
    float c = dz * dz;
    return (a + b) + c;
}

static inline uint64_t make_key(float d2, uint32_t idx) {
    uint32_t bits;
    std::memcpy(&bits, &d2, 4);
    return (uint64_t(bits) << 32) | idx;
}

class KDTree {
  public:
    KDTree(const float* xyz, size_t n, size_t leaf) : n_(n), pts_(n) {
        for (size_t i = 0; i < n; i++) {
            pts_[i].p[0] = xyz[3 * i];
            pts_[i].p[1] = xyz[3 * i + 1];
            pts_[i].p[2] = xyz[3 * i + 2];
            pts_[i].index = uint32_t(i);
        }
        // KDTree::init (KDTree.tcc:48-75): bounding box in double
        double mn[3], mx[3];
        for (int j = 0; j < 3; j++) { mn[j] = std::numeric_limits<double>::max(); mx[j] = -mn[j]; }
        for (size_t i = 0; i < n; i++)
            for (int j = 0; j < 3; j++) {
                mn[j] = std::min(mn[j], double(pts_[i].p[j]));
                mx[j] = std::max(mx[j], double(pts_[i].p[j]));
            }
        if (n == 0) return;
#pragma omp parallel
#pragma omp single
        root_ = build(0, n, mn, mx, leaf);
    }

    size_t size() const { return n_; }

    // Reference-faithful kNN (KDTree.tcc:101-128, 186-198, 227-246).
    // Returns indices sorted by ascending distance, distances = sqrt(d2).
    size_t knn_ref(const float* qf, size_t k, std::vector<uint32_t>& idx,
                   std::vector<float>* dist) const {
        double q[3] = {qf[0], qf[1], qf[2]};
        double worst = std::numeric_limits<double>::infinity();
        std::priority_queue<DP> queue;
        if (root_) knn_ref_rec(root_.get(), q, k, queue, worst);
        size_t m = queue.size();
        idx.resize(m);
        if (dist) dist->resize(m);
        size_t i = m;
        while (!queue.empty()) {
            i--;
            idx[i] = queue.top().index;
            if (dist) (*dist)[i] = float(std::sqrt(queue.top().d2));
            queue.pop();
        }
        return m;
    }

    // Canonical kNN: exact k smallest keys (d2_f32, index), ascending.
    size_t knn_canon(const float* q, size_t k, std::vector<uint32_t>& idx,
                     std::vector<float>* dist) const {
        std::priority_queue<uint64_t> heap;
        float worst = std::numeric_limits<float>::infinity();
        if (root_ && k > 0) knn_canon_rec(root_.get(), q, k, heap, worst);
        size_t m = heap.size();
        idx.resize(m);
        if (dist) dist->resize(m);
        size_t i = m;
        while (!heap.empty()) {
            i--;
            uint64_t key = heap.top();
            heap.pop();
            idx[i] = uint32_t(key & 0xffffffffu);
            if (dist) {
                uint32_t b = uint32_t(key >> 32);
                float d2;
                std::memcpy(&d2, &b, 4);
                (*dist)[i] = std::sqrt(d2);
            }
        }
        return m;
    }

  private:
    struct DP {
        double d2;
        uint32_t index;
        bool operator<(const DP& o) const { return d2 < o.d2; }
    };

    std::unique_ptr<KDNode> build(size_t s, size_t e, const double* mn, const double* mx,
                                  size_t leaf) {
        size_t n = e - s;
        auto node = std::make_unique<KDNode>();
        if (n <= leaf) {
            node->leaf = true;
            node->start = s;
            node->end = e;
            return node;
        }
        unsigned axis = 0;
        double len = mx[0] - mn[0];
        for (unsigned i = 1; i < 3; i++)
            if (mx[i] - mn[i] > len) { axis = i; len = mx[i] - mn[i]; }
        size_t mid = s + n / 2;
        std::nth_element(pts_.begin() + s, pts_.begin() + mid, pts_.begin() + e,
                         [axis](const IPoint& a, const IPoint& b) { return a.p[axis] < b.p[axis]; });
        double split = pts_[mid].p[axis];
        double lmx[3] = {mx[0], mx[1], mx[2]};
        double gmn[3] = {mn[0], mn[1], mn[2]};
        lmx[axis] = split;
        gmn[axis] = split;
        node->leaf = false;
        node->axis = axis;
        node->split = split;
        if (n > 8 * leaf) {
#pragma omp task shared(node)
            node->lesser = build(s, mid, mn, lmx, leaf);
#pragma omp task shared(node)
            node->greater = build(mid, e, gmn, mx, leaf);
#pragma omp taskwait
        } else {
            node->lesser = build(s, mid, mn, lmx, leaf);
            node->greater = build(mid, e, gmn, mx, leaf);
        }
        return node;
    }

    void knn_ref_rec(const KDNode* nd, const double* q, size_t k, std::priority_queue<DP>& queue,
                     double& worst) const {
        if (nd->leaf) {
            for (size_t i = nd->start; i < nd->end; i++) {
                const IPoint& p = pts_[i];
                double d2 = 0;
                for (int j = 0; j < 3; j++) {
                    double t = q[j] - double(p.p[j]);
                    d2 += t * t;
                }
                if (d2 < worst) {
                    queue.push(DP{d2, p.index});
                    if (queue.size() > k) {
                        queue.pop();
                        worst = queue.top().d2;
                    }
                }
            }
            return;
        }
        double t = q[nd->axis] - nd->split;
        double cmp = t * t;
        const KDNode* first = q[nd->axis] < nd->split ? nd->lesser.get() : nd->greater.get();
        const KDNode* second = q[nd->axis] < nd->split ? nd->greater.get() : nd->lesser.get();
        knn_ref_rec(first, q, k, queue, worst);
        if (cmp < worst) knn_ref_rec(second, q, k, queue, worst);
    }

    void knn_canon_rec(const KDNode* nd, const float* q, size_t k, std::priority_queue<uint64_t>& heap,
                       float& worst) const {
        if (nd->leaf) {
            for (size_t i = nd->start; i < nd->end; i++) {
                const IPoint& p = pts_[i];
                float d2 = d2_canonical(q, p.p);
                if (d2 <= worst) {
                    uint64_t key = make_key(d2, p.index);
                    if (heap.size() < k) {
                        heap.push(key);
                    } else if (key < heap.top()) {
                        heap.pop();
                        heap.push(key);
                    }
                    if (heap.size() == k) {
                        uint32_t b = uint32_t(heap.top() >> 32);
                        std::memcpy(&worst, &b, 4);
                    }
                }
            }
            return;
        }
        double t = double(q[nd->axis]) - nd->split;
        double cmp = t * t;
        bool lo = double(q[nd->axis]) < nd->split;
        const KDNode* first = lo ? nd->lesser.get() : nd->greater.get();
        const KDNode* second = lo ? nd->greater.get() : nd->lesser.get();
        knn_canon_rec(first, q, k, heap, worst);
        // Conservative pruning: a float32 squared distance can be below the
        // exact one by a few ulp, so the plane test is widened by 1e-5.
        if (cmp * (1.0 - 1e-5) <= double(worst)) knn_canon_rec(second, q, k, heap, worst);
    }

    size_t n_;
    std::vector<IPoint> pts_;
    std::unique_ptr<KDNode> root_;
};

}  // namespace

/* ------------------------------------------------------------------------ */
/* Surface                                                                   */
/* ------------------------------------------------------------------------ */
struct orc_surface {
    std::vector<V3> pts;
    BBox bb;
    std::unique_ptr<KDTree> tree;

    size_t ksearch(const V3& q, int k, bool canonical, std::vector<uint32_t>& idx) const {
        float qf[3] = {q.x, q.y, q.z};
        if (k <= 0) { idx.clear(); return 0; }
        return canonical ? tree->knn_canon(qf, size_t(k), idx, nullptr)
                         : tree->knn_ref(qf, size_t(k), idx, nullptr);
    }
};

namespace {

static int set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
    return omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

// AdaptiveKSearchSurface::boundingBoxOK (AdaptiveKSearchSurface.tcc:337-350)
static bool bbox_ok(const BBox& bb) {
    float dx = bb.xs(), dy = bb.ys(), dz = bb.zs();
    float e = 0.05f;
    return dx >= e * dy && dx >= e * dz && dy >= e * dx && dy >= e * dz && dz >= e * dx &&
           dz >= e * dy;
}

// calcPlane, nem 0 (AdaptiveKSearchSurface.tcc:467-520).  The reference
// solves the least-squares system y = C0 + C1 x + C2 z with Eigen's
// JacobiSVD in float; here the same least-squares solution is computed in
// double from centred normal equations and rounded to float.  Parity for this
// mode is therefore by angle, not by bits.
static V3 plane_lsq(const std::vector<V3>& P, const std::vector<uint32_t>& id, const V3& q) {
    const float epsilon = 100.0f;
    size_t m = id.size();
    double mx = 0, my = 0, mz = 0;
    for (auto i : id) { mx += P[i].x; my += P[i].y; mz += P[i].z; }
    mx /= double(m); my /= double(m); mz /= double(m);
    double sxx = 0, sxz = 0, szz = 0, sxy = 0, szy = 0;
    for (auto i : id) {
        double x = P[i].x - mx, y = P[i].y - my, z = P[i].z - mz;
        sxx += x * x; sxz += x * z; szz += z * z; sxy += x * y; szy += z * y;
    }
    double det = sxx * szz - sxz * sxz;
    double c1 = 0, c2 = 0;
    if (det != 0) {
        c1 = (sxy * szz - szy * sxz) / det;
        c2 = (szy * sxx - sxy * sxz) / det;
    }
    double c0 = my - c1 * mx - c2 * mz;
    float C0 = float(c0), C1 = float(c1), C2 = float(c2);
    float z1 = C0 + C1 * (q.x + epsilon) + C2 * q.z;
    float z2 = C0 + C1 * q.x + C2 * (q.z + epsilon);
    V3 diff1 = V3(q.x + epsilon, z1, q.z) - q;
    V3 diff2 = V3(q.x, z2, q.z + epsilon) - q;
    return diff1.cross(diff2).normalized();
}

// calcPlaneRANSAC, nem 1 (AdaptiveKSearchSurface.tcc:689-781), as the
// reference runs it: a default-constructed std::default_random_engine per
// call, bound by copy with uniform_int_distribution(0, |id| - 1) (:715-717);
// the three plane points are P[r] for draws r in [0, |id|) -- indices of the
// whole cloud (:736-740) -- and the scoring points P[id[r]] (:746-753).
// Returns false where the reference would read past its draw set (fewer than
// three distinct draws within 21).  The caller keeps the RANSAC plane: lvr2
// never sets `ok` (:223-231).
static bool plane_ransac(const std::vector<V3>& P, const std::vector<uint32_t>& id, V3& out) {
    if (id.size() < 3) return false;
    V3 best_norm(0, 0, 1);
    float bestdist = FLT_MAX;
    int iterations = 0, nonimproving = 0;
    std::unordered_set<size_t> draws;
    std::default_random_engine engine;
    std::uniform_int_distribution<size_t> uniform(0, id.size() - 1);
    auto next = std::bind(uniform, engine);
    while (nonimproving < 5 && iterations < 10) {
        int c = 0;
        draws.clear();
        do {
            draws.insert(next());
            c++;
        } while (draws.size() < 3 && c <= 20);
        if (draws.size() < 3) return false;
        auto it = draws.begin();
        const V3 a = P[*it];
        const V3 b = P[*(++it)];
        const V3 c3 = P[*(++it)];
        const V3 n0 = (a - b).cross(a - c3).normalized();
        float dist = 0;
        const int n = std::min(50, int(id.size()));
        for (int i = 0; i < n; i++) {
            const V3 r = P[id[next()]];
            dist += std::fabs(r.dot(n0) - a.dot(n0));
        }
        if (n != 0) dist /= float(n);
        if (dist < bestdist) {
            bestdist = dist;
            best_norm = n0;
            nonimproving = 0;
        } else {
            nonimproving++;
        }
        iterations++;
    }
    out = best_norm;
    return true;
}

// calcPlaneIterative, nem 2 (AdaptiveKSearchSurface.tcc:522-607)
static V3 plane_iterative(const std::vector<V3>& P, const std::vector<uint32_t>& id, const V3& q) {
    float xx = 0, xy = 0, xz = 0, yy = 0, yz = 0, zz = 0;
    for (auto i : id) {
        V3 r = P[i] - q;
        xx += r.x * r.x; xy += r.x * r.y; xz += r.x * r.z;
        yy += r.y * r.y; yz += r.y * r.z; zz += r.z * r.z;
    }
    float det_x = yy * zz - yz * yz;
    float det_y = xx * zz - xz * xz;
    float det_z = xx * yy - xy * xy;
    float dx, dy, dz;
    if (det_x >= det_y && det_x >= det_z) {
        dx = 1.0f;
        dy = (xz * yz - xy * zz) / det_x;
        dz = (xy * yz - xz * yy) / det_x;
    } else if (det_y >= det_x && det_y >= det_z) {
        dx = (yz * xz - xy * zz) / det_y;
        dy = 1.0f;
        dz = (xy * xz - yz * xx) / det_y;
    } else {
        dx = (yz * xy - xz * yy) / det_z;
        dy = (xz * xy - yz * xx) / det_z;
        dz = 1.0f;
    }
    const float invnorm = 1 / std::sqrt(dx * dx + dy * dy + dz * dz);
    return V3(dx * invnorm, dy * invnorm, dz * invnorm);
}

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix in double;
// returns the unit eigenvector of the smallest eigenvalue.
static void jacobi3_smallest(const double A_in[3][3], double v_out[3]) {
    double A[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) A[i][j] = A_in[i][j];
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        if (off == 0) break;
        for (int p = 0; p < 2; p++)
            for (int qq = p + 1; qq < 3; qq++) {
                if (A[p][qq] == 0) continue;
                double theta = (A[qq][qq] - A[p][p]) / (2 * A[p][qq]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < 3; k++) {
                    double akp = A[k][p], akq = A[k][qq];
                    A[k][p] = c * akp - s * akq;
                    A[k][qq] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    double apk = A[p][k], aqk = A[qq][k];
                    A[p][k] = c * apk - s * aqk;
                    A[qq][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    double vkp = V[k][p], vkq = V[k][qq];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][qq] = s * vkp + c * vkq;
                }
            }
    }
    int m = 0;
    if (A[1][1] < A[m][m]) m = 1;
    if (A[2][2] < A[m][m]) m = 2;
    double n = std::sqrt(V[0][m] * V[0][m] + V[1][m] * V[1][m] + V[2][m] * V[2][m]);
    for (int k = 0; k < 3; k++) v_out[k] = V[k][m] / n;
}

// calcPlaneIPCAExact, nem 3 (AdaptiveKSearchSurface.tcc:609-673): the
// incremental mean/covariance starts from the query point (n = 1) and adds
// every neighbour, in float with float weights.  The reference then calls
// Eigen's EigenSolver on the float matrix; this restatement takes the
// smallest eigenvector with a double-precision Jacobi solver.
static V3 plane_ipca(const std::vector<V3>& P, const std::vector<uint32_t>& id, const V3& q) {
    float mean[3] = {q.x, q.y, q.z};
    float cov[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double n_meas = 1.0;
    for (auto i : id) {
        const float p[3] = {P[i].x, P[i].y, P[i].z};
        const double n_new = n_meas + 1.0;
        float w1 = float(n_meas / n_new);
        float w2 = float(1.0 / n_new);
        float mn[3], a[3], b[3];
        for (int j = 0; j < 3; j++) mn[j] = mean[j] * w1 + p[j] * w2;
        for (int j = 0; j < 3; j++) { a[j] = mean[j] - mn[j]; b[j] = p[j] - mn[j]; }
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                float P1 = a[r] * a[c];
                float P2 = b[r] * b[c];
                cov[r][c] = (cov[r][c] + P1) * w1 + P2 * w2;
            }
        n_meas = n_new;
        for (int j = 0; j < 3; j++) mean[j] = mn[j];
    }
    double A[3][3], v[3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) A[r][c] = cov[r][c];
    jacobi3_smallest(A, v);
    return V3(float(v[0]), float(v[1]), float(v[2]));
}

}  // namespace

extern "C" {

orc_surface* orc_create(const float* xyz, int64_t n, int leaf_size, int threads) {
    set_threads(threads);
    auto* s = new orc_surface();
    s->pts.resize(size_t(n));
    for (int64_t i = 0; i < n; i++) {
        s->pts[size_t(i)] = V3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        s->bb.expand(s->pts[size_t(i)]);  // PointsetSurface.tcc:39-58
    }
    s->tree = std::make_unique<KDTree>(xyz, size_t(n), size_t(leaf_size > 0 ? leaf_size : 20));
    return s;
}

void orc_destroy(orc_surface* s) { delete s; }

void orc_bbox(const orc_surface* s, float* o) {
    o[0] = s->bb.mn.x; o[1] = s->bb.mn.y; o[2] = s->bb.mn.z;
    o[3] = s->bb.mx.x; o[4] = s->bb.mx.y; o[5] = s->bb.mx.z;
    o[6] = s->bb.centroid.x; o[7] = s->bb.centroid.y; o[8] = s->bb.centroid.z;
}

int orc_knn(const orc_surface* s, const float* q, int64_t nq, int k, int canonical, uint32_t* idx,
            float* dist, int32_t* count, int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < nq; i++) {
        std::vector<uint32_t> id;
        std::vector<float> d;
        size_t m = canonical ? s->tree->knn_canon(q + 3 * i, size_t(k), id, &d)
                             : s->tree->knn_ref(q + 3 * i, size_t(k), id, &d);
        for (int j = 0; j < k; j++) {
            idx[i * k + j] = size_t(j) < m ? id[size_t(j)] : 0xffffffffu;
            dist[i * k + j] = size_t(j) < m ? d[size_t(j)] : std::numeric_limits<float>::infinity();
        }
        if (count) count[i] = int32_t(m);
    }
    return 0;
}

int orc_normals(const orc_surface* s, int kn, int nem, int adaptive, const float* flip3,
                int canonical, float* normals, int32_t* k_used, int threads, const float* flip_targets) {
    if (nem < 0 || nem > 3) return -1;
    set_threads(threads);
    const std::vector<V3>& P = s->pts;
    const V3 flip = flip3 ? V3(flip3[0], flip3[1], flip3[2]) : s->bb.centroid;
    const int64_t n = int64_t(P.size());
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; i++) {
        std::vector<uint32_t> id;
        size_t k = size_t(kn);
        int rounds = 0;
        // AdaptiveKSearchSurface.tcc:187-216: k is doubled before each search,
        // at most 5 searches, stop once the neighbourhood box is well formed.
        while (rounds < 5) {
            rounds++;
            k = k * 2;
            s->ksearch(P[size_t(i)], int(k), canonical != 0, id);
            if (!adaptive) break;
            BBox bb;
            for (auto j : id) bb.expand(P[j]);
            if (bbox_ok(bb)) break;
        }
        const V3& qp = P[size_t(i)];
        V3 nrm;
        if (nem == 1) {
            if (!plane_ransac(P, id, nrm)) nrm = V3(NAN, NAN, NAN);
        } else if (nem == 2) nrm = plane_iterative(P, id, qp);
        else if (nem == 3) nrm = plane_ipca(P, id, qp);
        else nrm = plane_lsq(P, id, qp);
        // Flip toward the flip point (AdaptiveKSearchSurface.tcc:268-274), or
        // toward the point the nearest scan pose names (:252-265) when the
        // caller gives per-point targets (NaN x: none).
        // Normal::operator-() builds a new Normal, which re-normalises.
        V3 target = flip;
        if (flip_targets && flip_targets[3 * i] == flip_targets[3 * i])
            target = V3(flip_targets[3 * i], flip_targets[3 * i + 1], flip_targets[3 * i + 2]);
        if (nrm.dot(target - qp) < 0) nrm = V3(-nrm.x, -nrm.y, -nrm.z).normalized();
        normals[3 * i] = nrm.x;
        normals[3 * i + 1] = nrm.y;
        normals[3 * i + 2] = nrm.z;
        if (k_used) k_used[i] = int32_t(k);
    }
    return 0;
}

int orc_ransac_draws(int64_t m, uint32_t* out) {
    // The draws plane_ransac consumes for a neighbour list of m entries,
    // all 10 iterations: 3 plane ranks (set order), then min(50, m) scoring
    // ranks; 53 entries per iteration.  Returns -1 where plane_ransac fails.
    if (m < 3) return -1;
    std::unordered_set<size_t> draws;
    std::default_random_engine engine;
    std::uniform_int_distribution<size_t> uniform(0, size_t(m) - 1);
    auto next = std::bind(uniform, engine);
    const int n = int(std::min<int64_t>(50, m));
    for (int t = 0; t < 10; t++) {
        uint32_t* row = out + 53 * t;
        std::fill(row, row + 53, 0u);
        int c = 0;
        draws.clear();
        do {
            draws.insert(next());
            c++;
        } while (draws.size() < 3 && c <= 20);
        if (draws.size() < 3) return -1;
        int j = 0;
        for (size_t v : draws) row[j++] = uint32_t(v);
        for (int i = 0; i < n; i++) row[3 + i] = uint32_t(next());
    }
    return 0;
}

int orc_interpolate(const orc_surface* s, int ki, const float* in, float* out, int canonical,
                    int threads) {
    set_threads(threads);
    const std::vector<V3>& P = s->pts;
    const int64_t n = int64_t(P.size());
    if (ki <= 0) {
        std::memcpy(out, in, sizeof(float) * 3 * size_t(n));
        return 0;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; i++) {
        std::vector<uint32_t> id;
        s->ksearch(P[size_t(i)], ki, canonical != 0, id);
        V3 mean(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
        for (auto j : id) mean += V3(in[3 * j], in[3 * j + 1], in[3 * j + 2]);
        V3 r = mean.normalized();
        out[3 * i] = r.x;
        out[3 * i + 1] = r.y;
        out[3 * i + 2] = r.z;
    }
    return 0;
}

}  // extern "C"

namespace {
// AdaptiveKSearchSurface::distance (AdaptiveKSearchSurface.tcc:414-457)
static void distance_one(const orc_surface* s, const float* normals, int kd, const V3& p,
                         bool canonical, float& proj, float& eucl) {
    std::vector<uint32_t> id;
    s->ksearch(p, kd, canonical, id);
    if (id.empty()) {
        proj = eucl = std::numeric_limits<float>::max();
        return;
    }
    V3 nearest, avg;
    for (auto j : id) {
        nearest += s->pts[j];
        avg += V3(normals[3 * j], normals[3 * j + 1], normals[3 * j + 2]);
    }
    avg /= float(id.size());
    nearest /= float(id.size());
    V3 nrm = avg.normalized();
    V3 d = p - nearest;
    proj = d.dot(nrm);
    eucl = d.length();
}
}  // namespace

extern "C" {

int orc_distance(const orc_surface* s, const float* normals, int kd, const float* q, int64_t nq,
                 int canonical, float* projected, float* euclidean, int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < nq; i++) {
        V3 p(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
        distance_one(s, normals, kd, p, canonical != 0, projected[i], euclidean[i]);
    }
    return 0;
}

// PointsetSurface::getInterpolatedNormal (PointsetSurface.tcc:61-74): the
// accumulator is a default Normal (0, 1, 0); every neighbour normal is
// normalised when read; the sum is divided by ki.  The return copy-constructs
// the Normal it already is, so the mean comes back un-normalised.
int orc_interpolated_normal(const orc_surface* s, const float* normals, int ki, const float* q,
                            int64_t nq, int canonical, float* out, int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < nq; i++) {
        std::vector<uint32_t> id;
        s->ksearch(V3(q[3 * i], q[3 * i + 1], q[3 * i + 2]), ki, canonical != 0, id);
        V3 r(0, 1, 0);
        for (size_t j = 0; j < id.size() && int(j) < ki; j++) {
            uint32_t t = id[j];
            r += V3(normals[3 * t], normals[3 * t + 1], normals[3 * t + 2]).normalized();
        }
        // `return Normal<float>(result)` copy-constructs from a Normal: the
        // mean is returned as it is, not normalised (PointsetSurface.tcc:72-73)
        r /= float(ki);
        out[3 * i] = r.x;
        out[3 * i + 1] = r.y;
        out[3 * i + 2] = r.z;
    }
    return 0;
}

}  // extern "C"

/* ------------------------------------------------------------------------ */
/* Grid + marching cubes                                                     */
/* ------------------------------------------------------------------------ */
namespace {

struct L3 {
    int32_t x, y, z;
    bool operator==(const L3& o) const { return x == o.x && y == o.y && z == o.z; }
    bool operator<(const L3& o) const {
        if (x != o.x) return x < o.x;
        if (y != o.y) return y < o.y;
        return z < o.z;
    }
};
struct L3Hash {
    size_t operator()(const L3& v) const {
        uint64_t h = 1469598103934665603ull;
        for (int32_t c : {v.x, v.y, v.z}) {
            h ^= uint32_t(c);
            h *= 1099511628211ull;
        }
        return size_t(h);
    }
};

// FastReconstructionTables.hpp:70 box_creation_table; corner i of a cell
// sits at lattice offset (t+1)/2 of its table row.
static const int kCornerOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// FastBoxTables.hpp:71 vertex_edge_table
static const int kEdgeCorners[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                        {6, 7}, {7, 4}, {0, 4}, {1, 5}, {3, 7}, {2, 6}};

static const uint64_t kMCTable[256] = {
#include "../lvr2_gb300/csrc/mc_table.inc"
};

// HashGrid::indexToCenter (HashGrid.hpp:276-281)
static inline float cell_center(int32_t idx, float vs) { return (float(idx) + 0.5f) * vs; }
// Grid vertex coordinate: HashGrid::addBox (HashGrid.tcc:235-259) places a
// new corner at center + table * (vs / 2).  The reference creates each shared
// corner from whichever cell is visited first in unordered_set order, so its
// coordinate can differ by one ulp between runs; this restatement always uses
// the cell whose lowest corner it is (table entry -1).
static inline float lattice_coord(int32_t L, float vs) {
    float h = vs / 2.0f;
    float off = -1.0f * h;
    return cell_center(L, vs) + off;
}

// FastBox::calcIntersection (FastBox.tcc:134-158)
static inline float calc_intersection(float x1, float x2, float d1, float d2) {
    if (d1 == 0) return x1;
    if (d2 == 0) return x2;
    if ((d1 < 0 && d2 > 0) || (d2 < 0 && d1 > 0)) {
        float interpolation = x2 - d2 * (x1 - x2) / (d1 - d2);
        return interpolation;
    }
    return 0;
}

struct EdgeKey {
    L3 l;
    int axis;
    bool operator==(const EdgeKey& o) const { return l == o.l && axis == o.axis; }
};
struct EdgeKeyHash {
    size_t operator()(const EdgeKey& e) const { return L3Hash()(e.l) * 3 + size_t(e.axis); }
};

}  // namespace

struct orc_recon {
    float vs = 0;
    std::vector<L3> cells_all, cells_valid;
    std::vector<L3> qp_lat;
    std::vector<V3> qp_pos;
    std::vector<float> qp_dist;
    std::vector<uint8_t> qp_invalid;
    std::vector<EdgeKey> mv_key;
    std::vector<V3> mv_pos;
    std::vector<int32_t> faces;
    std::vector<int64_t> cell_face_off;  // faces of valid cell c: [off[c], off[c + 1])
};

// Marching cubes over the given cells of r (cells_all, qp_pos, qp_dist set).
static void mc_cells(orc_recon* r, const std::vector<std::array<int32_t, 8>>& cell_qp,
                     const std::vector<size_t>& valid_cells, int decomposition) {
    // Marching cubes (FastReconstruction.tcc:47-66, FastBox.tcc:205-269,
    // BilinearFastBox.tcc:55-138).  Each mesh vertex is identified by the
    // grid edge it lies on; the reference shares a vertex among the four cells
    // of an edge through neighbor_table / neighbor_vertex_table, which gives
    // the same identification.
    std::unordered_map<EdgeKey, int32_t, EdgeKeyHash> vmap;
    r->cell_face_off.push_back(0);
    for (size_t vc : valid_cells) {
        const L3& ci = r->cells_all[vc];
        float dist[8];
        V3 corner[8];
        for (int k = 0; k < 8; k++) {
            int32_t q = cell_qp[vc][size_t(k)];
            dist[k] = r->qp_dist[size_t(q)];
            corner[k] = r->qp_pos[size_t(q)];
        }
        int index = 0;
        for (int k = 0; k < 8; k++)
            if (dist[k] > 0) index |= (1 << k);
        V3 epos[12];
        EdgeKey ekey[12];
        for (int e = 0; e < 12; e++) {
            int a = kEdgeCorners[e][0], b = kEdgeCorners[e][1];
            int axis = 0;
            for (int t = 0; t < 3; t++)
                if (kCornerOff[a][t] != kCornerOff[b][t]) axis = t;
            int lo = kCornerOff[a][axis] < kCornerOff[b][axis] ? a : b;
            int hi = lo == a ? b : a;
            float x = calc_intersection(corner[lo][axis], corner[hi][axis], dist[lo], dist[hi]);
            V3 p = corner[lo];
            if (axis == 0) p.x = x;
            else if (axis == 1) p.y = x;
            else p.z = x;
            epos[e] = p;
            ekey[e] = EdgeKey{L3{ci.x + kCornerOff[lo][0], ci.y + kCornerOff[lo][1],
                                 ci.z + kCornerOff[lo][2]},
                              axis};
        }
        uint64_t word = kMCTable[index];
        int ntri = int(word >> 60);
        for (int t = 0; t < ntri; t++) {
            int e3[3];
            for (int b = 0; b < 3; b++) e3[b] = int((word >> (4 * (3 * t + b))) & 0xf);
            if (decomposition == 1) {
                if (epos[e3[0]] == epos[e3[1]] || epos[e3[0]] == epos[e3[2]] ||
                    epos[e3[2]] == epos[e3[1]])
                    continue;
            }
            for (int b = 0; b < 3; b++) {
                auto it = vmap.find(ekey[e3[b]]);
                int32_t vid;
                if (it == vmap.end()) {
                    vid = int32_t(r->mv_key.size());
                    vmap.emplace(ekey[e3[b]], vid);
                    r->mv_key.push_back(ekey[e3[b]]);
                    r->mv_pos.push_back(epos[e3[b]]);
                } else {
                    vid = it->second;
                }
                r->faces.push_back(vid);
            }
        }
        r->cell_face_off.push_back(int64_t(r->faces.size() / 3));
    }
}

extern "C" {

orc_recon* orc_reconstruct(const orc_surface* s, const float* normals, float resolution,
                           int is_voxelsize, int extrude, int kd, int decomposition, int canonical,
                           const int32_t* qp_lattice, const float* qp_dist_in,
                           const uint8_t* qp_invalid_in, int64_t n_qp, int threads) {
    set_threads(threads);
    auto* r = new orc_recon();
    const BBox& bb = s->bb;  // PointsetGrid is given surface->getBoundingBox()
    // HashGrid ctor (HashGrid.tcc:48-52)
    const float vs = is_voxelsize ? resolution : bb.longest() / resolution;
    r->vs = vs;

    // Cell discovery and extrusion (PointsetGrid.tcc:61-106)
    std::unordered_set<L3, L3Hash> required;
    {
        const int64_t n = int64_t(s->pts.size());
#pragma omp parallel
        {
            std::unordered_set<L3, L3Hash> local;
#pragma omp for schedule(dynamic, 64) nowait
            for (int64_t i = 0; i < n; i++) {
                const V3& p = s->pts[size_t(i)];
                L3 idx{int32_t(std::floor(p.x / vs)), int32_t(std::floor(p.y / vs)),
                       int32_t(std::floor(p.z / vs))};
                V3 c(cell_center(idx.x, vs), cell_center(idx.y, vs), cell_center(idx.z, vs));
                if (bb.contains(c)) local.insert(idx);
            }
            if (extrude) {
                std::unordered_set<L3, L3Hash> inner = local;
                for (const L3& idx : inner)
                    for (int dx = -1; dx <= 1; dx++)
                        for (int dy = -1; dy <= 1; dy++)
                            for (int dz = -1; dz <= 1; dz++) {
                                L3 pos{idx.x + dx, idx.y + dy, idx.z + dz};
                                V3 c(cell_center(pos.x, vs), cell_center(pos.y, vs),
                                     cell_center(pos.z, vs));
                                if (bb.contains(c)) local.insert(pos);
                            }
            }
#pragma omp critical
            required.insert(local.begin(), local.end());
        }
    }
    r->cells_all.assign(required.begin(), required.end());
    std::sort(r->cells_all.begin(), r->cells_all.end());

    // Grid vertices: the 8 corners of every cell, shared between cells
    // (HashGrid::addLatticePoints / addBox / findQueryPoint).
    std::unordered_map<L3, int32_t, L3Hash> qp_index;
    std::vector<std::array<int32_t, 8>> cell_qp(r->cells_all.size());
    for (size_t c = 0; c < r->cells_all.size(); c++) {
        const L3& ci = r->cells_all[c];
        for (int k = 0; k < 8; k++) {
            L3 L{ci.x + kCornerOff[k][0], ci.y + kCornerOff[k][1], ci.z + kCornerOff[k][2]};
            auto it = qp_index.find(L);
            int32_t id;
            if (it == qp_index.end()) {
                id = int32_t(r->qp_lat.size());
                qp_index.emplace(L, id);
                r->qp_lat.push_back(L);
                r->qp_pos.push_back(V3(lattice_coord(L.x, vs), lattice_coord(L.y, vs),
                                       lattice_coord(L.z, vs)));
            } else {
                id = it->second;
            }
            cell_qp[c][size_t(k)] = id;
        }
    }
    const int64_t nqp = int64_t(r->qp_lat.size());
    r->qp_dist.assign(size_t(nqp), 0.0f);
    r->qp_invalid.assign(size_t(nqp), 0);

    if (qp_lattice) {
        for (int64_t i = 0; i < n_qp; i++) {
            L3 L{qp_lattice[3 * i], qp_lattice[3 * i + 1], qp_lattice[3 * i + 2]};
            auto it = qp_index.find(L);
            if (it == qp_index.end()) continue;
            r->qp_dist[size_t(it->second)] = qp_dist_in[i];
            r->qp_invalid[size_t(it->second)] = qp_invalid_in[i];
        }
    } else {
        // PointsetGrid::calcDistanceValues (PointsetGrid.tcc:111-150)
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < nqp; i++) {
            float proj, eucl;
            distance_one(s, normals, kd, r->qp_pos[size_t(i)], canonical != 0, proj, eucl);
            r->qp_invalid[size_t(i)] = (double(eucl) > 1.75 * double(vs)) ? 1 : 0;
            r->qp_dist[size_t(i)] = proj;
        }
    }

    // Remove cells with an invalid corner (PointsetGrid.tcc:153-184)
    std::vector<size_t> valid_cells;
    for (size_t c = 0; c < r->cells_all.size(); c++) {
        bool bad = false;
        for (int k = 0; k < 8; k++)
            if (r->qp_invalid[size_t(cell_qp[c][size_t(k)])]) bad = true;
        if (!bad) {
            valid_cells.push_back(c);
            r->cells_valid.push_back(r->cells_all[c]);
        }
    }

    mc_cells(r, cell_qp, valid_cells, decomposition);
    return r;
}

// HashGrid(chunks, innerBoxes, bb, voxelsize) (HashGrid.tcc:136-193) over
// stored chunk cells, then marching cubes: chunk by chunk, cell by cell, a
// cell whose centre its chunk's inner box contains (BoundingBox::contains)
// and whose index floor(centre / vs) is new is added; each of its corners
// reuses an existing grid vertex (findQueryPoint) or is created with this
// cell's distance (addBox).  Grid vertex positions use the lattice formula.
orc_recon* orc_reconstruct_cells(const float* centers, const float* tsdf, int64_t n, const int64_t* off,
                                 int nchunks, const float* boxes, float vs, int decomposition) {
    auto* r = new orc_recon();
    r->vs = vs;
    std::unordered_map<L3, int32_t, L3Hash> cell_index, qp_index;
    std::vector<std::array<int32_t, 8>> qp_of;
    std::vector<L3> order;
    for (int c = 0; c < nchunks; c++) {
        for (int64_t i = off[c]; i < off[c + 1]; i++) {
            const float x = centers[3 * i], y = centers[3 * i + 1], z = centers[3 * i + 2];
            if (boxes) {
                const float* b = boxes + 6 * c;
                if (!((b[0] <= x && b[3] >= x) && (b[1] <= y && b[4] >= y) && (b[2] <= z && b[5] >= z))) continue;
            }
            const float fx = std::floor(x / vs), fy = std::floor(y / vs), fz = std::floor(z / vs);
            if (!(std::fabs(fx) < 1e9f && std::fabs(fy) < 1e9f && std::fabs(fz) < 1e9f)) continue;
            const L3 idx{int32_t(fx), int32_t(fy), int32_t(fz)};
            if (cell_index.count(idx)) continue;
            std::array<int32_t, 8> q{};
            for (int k = 0; k < 8; k++) {
                const L3 L{idx.x + kCornerOff[k][0], idx.y + kCornerOff[k][1], idx.z + kCornerOff[k][2]};
                auto it = qp_index.find(L);
                if (it == qp_index.end()) {
                    const int32_t id = int32_t(r->qp_lat.size());
                    qp_index.emplace(L, id);
                    r->qp_lat.push_back(L);
                    r->qp_pos.push_back(V3(lattice_coord(L.x, vs), lattice_coord(L.y, vs), lattice_coord(L.z, vs)));
                    r->qp_dist.push_back(tsdf[8 * i + k]);
                    r->qp_invalid.push_back(0);
                    q[size_t(k)] = id;
                } else {
                    q[size_t(k)] = it->second;
                }
            }
            cell_index.emplace(idx, int32_t(qp_of.size()));
            qp_of.push_back(q);
            order.push_back(idx);
        }
    }
    // cells in lattice order (any order gives the same canonical mesh)
    r->cells_all = order;
    std::sort(r->cells_all.begin(), r->cells_all.end());
    std::vector<std::array<int32_t, 8>> cell_qp(r->cells_all.size());
    std::vector<size_t> valid_cells(r->cells_all.size());
    for (size_t c = 0; c < r->cells_all.size(); c++) {
        cell_qp[c] = qp_of[size_t(cell_index[r->cells_all[c]])];
        valid_cells[c] = c;
    }
    r->cells_valid = r->cells_all;
    mc_cells(r, cell_qp, valid_cells, decomposition);
    return r;
}

// BilinearFastBox::optimizePlanarFaces (BilinearFastBox.tcc:140-212), which
// FastReconstruction::getMesh runs on every cell with kc = 5 for PMC
// (FastReconstruction.tcc:158-168): in a cell whose faces have one or two
// border edges (edges of exactly one face of the mesh), both end vertices of
// each such edge move to the centroid of the kc nearest points.  The
// reference moves vertices in place while iterating its cell hash map, so a
// vertex on several such edges can move more than once, in an order that
// depends on the hash map.  Canonical form: every marked vertex moves once,
// from its marching-cubes position.  Returns the number of moved vertices.
int64_t orc_recon_optimize_planar(orc_recon* r, const orc_surface* s, int kc, int canonical, int threads) {
    set_threads(threads);
    const size_t nf = r->faces.size() / 3;
    auto edge_key = [&](size_t f, int e) {
        const uint64_t a = uint32_t(r->faces[3 * f + size_t(e)]);
        const uint64_t b = uint32_t(r->faces[3 * f + size_t((e + 1) % 3)]);
        return a < b ? (a << 32) | b : (b << 32) | a;
    };
    std::unordered_map<uint64_t, int> faces_of_edge;
    for (size_t f = 0; f < nf; f++)
        for (int e = 0; e < 3; e++) faces_of_edge[edge_key(f, e)]++;
    std::vector<uint8_t> mark(r->mv_pos.size(), 0);
    for (size_t c = 0; c + 1 < r->cell_face_off.size(); c++) {
        const size_t f0 = size_t(r->cell_face_off[c]), f1 = size_t(r->cell_face_off[c + 1]);
        int border = 0;
        for (size_t f = f0; f < f1; f++)
            for (int e = 0; e < 3; e++) border += faces_of_edge[edge_key(f, e)] == 1;
        if (border != 1 && border != 2) continue;
        for (size_t f = f0; f < f1; f++)
            for (int e = 0; e < 3; e++)
                if (faces_of_edge[edge_key(f, e)] == 1) {
                    mark[size_t(r->faces[3 * f + size_t(e)])] = 1;
                    mark[size_t(r->faces[3 * f + size_t((e + 1) % 3)])] = 1;
                }
    }
    const std::vector<V3> orig = r->mv_pos;
    int64_t moved = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : moved)
    for (int64_t v = 0; v < int64_t(orig.size()); v++) {
        if (!mark[size_t(v)]) continue;
        moved++;
        std::vector<uint32_t> id;
        s->ksearch(orig[size_t(v)], kc, canonical != 0, id);
        if (id.empty()) continue;
        V3 c;
        for (auto j : id) c += s->pts[j];
        c /= float(id.size());
        r->mv_pos[size_t(v)] = c;
    }
    return moved;
}

void orc_recon_destroy(orc_recon* r) { delete r; }

void orc_recon_counts(const orc_recon* r, int64_t* c, float* f) {
    c[0] = int64_t(r->cells_all.size());
    c[1] = int64_t(r->qp_lat.size());
    c[2] = int64_t(r->cells_valid.size());
    c[3] = int64_t(r->mv_key.size());
    c[4] = int64_t(r->faces.size() / 3);
    if (f) f[0] = r->vs;
}

void orc_recon_grid(const orc_recon* r, int32_t* lattice, float* pos, float* dist,
                    uint8_t* invalid) {
    std::vector<size_t> order(r->qp_lat.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = i;
    std::sort(order.begin(), order.end(),
              [&](size_t a, size_t b) { return r->qp_lat[a] < r->qp_lat[b]; });
    for (size_t o = 0; o < order.size(); o++) {
        size_t i = order[o];
        lattice[3 * o] = r->qp_lat[i].x;
        lattice[3 * o + 1] = r->qp_lat[i].y;
        lattice[3 * o + 2] = r->qp_lat[i].z;
        pos[3 * o] = r->qp_pos[i].x;
        pos[3 * o + 1] = r->qp_pos[i].y;
        pos[3 * o + 2] = r->qp_pos[i].z;
        dist[o] = r->qp_dist[i];
        invalid[o] = r->qp_invalid[i];
    }
}

void orc_recon_cells(const orc_recon* r, int32_t* all, int32_t* valid) {
    for (size_t i = 0; i < r->cells_all.size(); i++) {
        all[3 * i] = r->cells_all[i].x; all[3 * i + 1] = r->cells_all[i].y; all[3 * i + 2] = r->cells_all[i].z;
    }
    for (size_t i = 0; i < r->cells_valid.size(); i++) {
        valid[3 * i] = r->cells_valid[i].x; valid[3 * i + 1] = r->cells_valid[i].y; valid[3 * i + 2] = r->cells_valid[i].z;
    }
}

void orc_recon_mesh(const orc_recon* r, int32_t* vkeys, float* vpos, int32_t* faces) {
    for (size_t i = 0; i < r->mv_key.size(); i++) {
        vkeys[4 * i] = r->mv_key[i].l.x;
        vkeys[4 * i + 1] = r->mv_key[i].l.y;
        vkeys[4 * i + 2] = r->mv_key[i].l.z;
        vkeys[4 * i + 3] = r->mv_key[i].axis;
        vpos[3 * i] = r->mv_pos[i].x;
        vpos[3 * i + 1] = r->mv_pos[i].y;
        vpos[3 * i + 2] = r->mv_pos[i].z;
    }
    std::memcpy(faces, r->faces.data(), sizeof(int32_t) * r->faces.size());
}

int orc_mc_table(int32_t* out) {
    for (int i = 0; i < 256; i++) {
        uint64_t w = kMCTable[i];
        int ne = int(w >> 60) * 3;
        for (int j = 0; j < 13; j++) out[i * 13 + j] = j < ne ? int32_t((w >> (4 * j)) & 0xf) : -1;
    }
    return 0;
}

}  // extern "C"

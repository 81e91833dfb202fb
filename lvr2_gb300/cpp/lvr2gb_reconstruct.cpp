// lvr2gb_reconstruct -- the reconstruction part of lvr2_reconstruct
// (src/tools/lvr2_reconstruct/Main.cpp:238-610) on the GB300 path: read a
// point cloud, estimate and interpolate normals, build the grid, evaluate the
// signed distance and extract the (P)MC mesh, with lvr2_reconstruct's flag
// names and defaults (Options.cpp:60-125).
//
//   lvr2gb_reconstruct scan.pts -v 10 --kn 10 --ki 10 --kd 5 --flipPoint 0 0 0
//
// Input: ASCII .pts/.xyz/.3d (x y z [extra columns]) or PLY with float x,y,z
// (and nx,ny,nz, used unless --recalcNormals).  Output: binary PLY mesh
// (triangle_mesh.ply, or --outputFile), and with --exportPointNormals the
// points with their normals (pointnormals.ply).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "lvr2gb.hpp"

namespace {

struct Options {
    std::string input;
    std::string output = "triangle_mesh.ply";
    float voxelsize = 10.0f;
    int intersections = -1;
    std::string pcm = "LVR2";
    int nem = 0;
    std::string decomposition = "PMC";
    bool extrude = true;
    int kd = 5, ki = 10, kn = 10;
    bool flip_set = false;
    float flip[3] = {0, 0, 0};
    bool recalc = false;
    bool export_normals = false;
    bool save_grid = false;
    std::string pose_file;
    int device = 0;
};

void usage() {
    std::puts(
        "usage: lvr2gb_reconstruct <inputFile> [--voxelsize|-v F] [--intersections|-i N] [--pcm|-p NAME]\n"
        "       [--nem 0|1|2|3|4] [--decomposition|-d MC|PMC] [--noExtrusion] [--kd N] [--ki N] [--kn N]\n"
        "       [--flipPoint X Y Z] [--recalcNormals|-r] [--exportPointNormals|-e] [--outputFile PATH]\n"
        "       [--saveGrid|-g] [--scanPoseFile PATH] [--useGPU] [--threads N] [--device N]");
}

Options parse(int argc, char** argv) {
    Options o;
    auto need = [&](int& i, int count) {
        if (i + count >= argc) {
            usage();
            std::exit(2);
        }
    };
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--help" || a == "-h") {
            usage();
            std::exit(0);
        } else if (a == "--voxelsize" || a == "-v") {
            need(i, 1); o.voxelsize = std::stof(argv[++i]);
        } else if (a == "--intersections" || a == "-i") {
            need(i, 1); o.intersections = std::stoi(argv[++i]);
        } else if (a == "--pcm" || a == "-p") {
            need(i, 1); o.pcm = argv[++i];
        } else if (a == "--nem") {
            need(i, 1); o.nem = std::stoi(argv[++i]);
        } else if (a == "--decomposition" || a == "-d") {
            need(i, 1); o.decomposition = argv[++i];
        } else if (a == "--noExtrusion") {
            o.extrude = false;
        } else if (a == "--kd") {
            need(i, 1); o.kd = std::stoi(argv[++i]);
        } else if (a == "--ki") {
            need(i, 1); o.ki = std::stoi(argv[++i]);
        } else if (a == "--kn") {
            need(i, 1); o.kn = std::stoi(argv[++i]);
        } else if (a == "--flipPoint") {
            need(i, 3);
            for (int k = 0; k < 3; k++) o.flip[k] = std::stof(argv[++i]);
            o.flip_set = true;
        } else if (a == "--recalcNormals" || a == "-r") {
            o.recalc = true;
        } else if (a == "--exportPointNormals" || a == "-e") {
            o.export_normals = true;
        } else if (a == "--saveGrid" || a == "-g") {
            o.save_grid = true;
        } else if (a == "--outputFile") {
            need(i, 1); o.output = argv[++i];
        } else if (a == "--scanPoseFile") {
            need(i, 1); o.pose_file = argv[++i];
        } else if (a == "--useGPU") {
        } else if (a == "--threads" || a == "--device") {
            need(i, 1);
            int v = std::stoi(argv[++i]);
            if (a == "--device") o.device = v;
        } else if (!a.empty() && a[0] != '-') {
            o.input = a;
        } else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            usage();
            std::exit(2);
        }
    }
    if (o.input.empty()) {
        usage();
        std::exit(2);
    }
    return o;
}

bool ends_with(const std::string& s, const std::string& t) {
    return s.size() >= t.size() && s.compare(s.size() - t.size(), t.size(), t) == 0;
}

// ASCII point file as AsciiIO::read reads it (src/liblvr2/io/modelio/AsciiIO.cpp:
// 227-270, 60-200): the first line is skipped; the second line's column count
// tells the attributes after x y z (3: r g b; 4: intensity r g b; 1:
// intensity); colours are read as unsigned integers and kept as bytes.
void read_ascii(const std::string& path, std::vector<float>& xyz, std::vector<uint8_t>& rgb) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open " + path);
    std::string line;
    std::getline(in, line);  // metadata or count
    std::vector<std::string> lines;
    int rpos = -1, columns = 0;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::vector<double> v;
        double t;
        while (ss >> t) v.push_back(t);
        if (columns == 0) {
            columns = int(v.size());
            const int attributes = columns - 3;
            if (attributes == 3) rpos = 3;
            if (attributes == 4) rpos = 4;
        }
        if (v.size() < 3) continue;
        for (int a = 0; a < 3; a++) xyz.push_back(float(v[size_t(a)]));
        if (rpos >= 0) {
            for (int c = 0; c < 3; c++) {
                const size_t k = size_t(rpos + c);
                rgb.push_back(k < v.size() ? uint8_t(unsigned(v[k])) : uint8_t(0));
            }
        }
    }
}

// AdaptiveKSearchSurface::parseScanPoses (AdaptiveKSearchSurface.tcc:94-139):
// "x y z" triples read while the stream is good; the read that meets the end
// of the file leaves x, y, z unchanged and still appends them, so the last pose
// appears twice, as in lvr2's loop.
std::vector<float> read_poses(const std::string& path) {
    std::ifstream in(path);
    if (!in.good()) throw std::runtime_error("cannot open scan pose file " + path);
    std::vector<float> poses;
    float x = 0, y = 0, z = 0;
    while (in.good()) {
        in >> x >> y >> z;
        poses.push_back(x);
        poses.push_back(y);
        poses.push_back(z);
    }
    return poses;
}

// PLY with vertex float properties x, y, z (and optional nx, ny, nz).
void read_ply(const std::string& path, std::vector<float>& xyz, std::vector<float>& nrm) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    std::string line, format;
    size_t nv = 0;
    std::vector<std::string> props;
    bool in_vertex = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ss(line);
        std::string w;
        ss >> w;
        if (w == "format") ss >> format;
        else if (w == "element") {
            std::string e;
            ss >> e;
            in_vertex = e == "vertex";
            if (in_vertex) ss >> nv;
        } else if (w == "property" && in_vertex) {
            std::string type, name;
            ss >> type >> name;
            if (type != "float" && type != "float32") throw std::runtime_error("PLY vertex property " + name + " is not float");
            props.push_back(name);
        } else if (w == "end_header") {
            break;
        }
    }
    int ix = -1, iy = -1, iz = -1, inx = -1, iny = -1, inz = -1;
    for (int i = 0; i < int(props.size()); i++) {
        if (props[i] == "x") ix = i;
        if (props[i] == "y") iy = i;
        if (props[i] == "z") iz = i;
        if (props[i] == "nx") inx = i;
        if (props[i] == "ny") iny = i;
        if (props[i] == "nz") inz = i;
    }
    if (ix < 0 || iy < 0 || iz < 0) throw std::runtime_error("PLY has no x y z");
    const bool has_n = inx >= 0 && iny >= 0 && inz >= 0;
    std::vector<float> row(props.size());
    xyz.reserve(3 * nv);
    for (size_t v = 0; v < nv; v++) {
        if (format == "ascii") {
            for (auto& r : row) in >> r;
        } else if (format == "binary_little_endian") {
            in.read(reinterpret_cast<char*>(row.data()), std::streamsize(row.size() * sizeof(float)));
        } else {
            throw std::runtime_error("PLY format " + format + " is not supported");
        }
        xyz.push_back(row[ix]); xyz.push_back(row[iy]); xyz.push_back(row[iz]);
        if (has_n) { nrm.push_back(row[inx]); nrm.push_back(row[iny]); nrm.push_back(row[inz]); }
    }
}

// Vertex element x, y, z, [red, green, blue], nx, ny, nz (the vertex colours
// and normals lvr2_reconstruct hands the finalizer, in PLYIO.cpp's property
// order, :166-240), then the faces as uchar-int lists.
void write_mesh_ply(const std::string& path, const lvr2gb::Mesh& m) {
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write " + path);
    const size_t nv = m.vertices.size() / 3, nf = m.faces.size() / 3;
    const bool normals = m.vertexNormals.size() == m.vertices.size() && nv > 0;
    const bool colors = m.vertexColors.size() == m.vertices.size() && nv > 0;
    out << "ply\nformat binary_little_endian 1.0\ncomment lvr2gb_reconstruct\n"
        << "element vertex " << nv << "\nproperty float x\nproperty float y\nproperty float z\n";
    if (colors) out << "property uchar red\nproperty uchar green\nproperty uchar blue\n";
    if (normals) out << "property float nx\nproperty float ny\nproperty float nz\n";
    out << "element face " << nf << "\nproperty list uchar int vertex_indices\nend_header\n";
    const size_t stride = 12 + (colors ? 3 : 0) + (normals ? 12 : 0);
    std::vector<char> rows(stride * nv);
    for (size_t v = 0; v < nv; v++) {
        char* r = rows.data() + stride * v;
        std::memcpy(r, &m.vertices[3 * v], 12);
        if (colors) std::memcpy(r + 12, &m.vertexColors[3 * v], 3);
        if (normals) std::memcpy(r + 12 + (colors ? 3 : 0), &m.vertexNormals[3 * v], 12);
    }
    out.write(rows.data(), std::streamsize(rows.size()));
    for (size_t f = 0; f < nf; f++) {
        const unsigned char three = 3;
        const int32_t idx[3] = {int32_t(m.faces[3 * f]), int32_t(m.faces[3 * f + 1]), int32_t(m.faces[3 * f + 2])};
        out.write(reinterpret_cast<const char*>(&three), 1);
        out.write(reinterpret_cast<const char*>(idx), sizeof(idx));
    }
}

void write_point_normals_ply(const std::string& path, const std::vector<float>& xyz, const std::vector<float>& n) {
    std::ofstream out(path, std::ios::binary);
    const size_t np = xyz.size() / 3;
    out << "ply\nformat binary_little_endian 1.0\nelement vertex " << np
        << "\nproperty float x\nproperty float y\nproperty float z\nproperty float nx\nproperty float ny\n"
           "property float nz\nend_header\n";
    for (size_t i = 0; i < np; i++) {
        out.write(reinterpret_cast<const char*>(&xyz[3 * i]), 3 * sizeof(float));
        out.write(reinterpret_cast<const char*>(&n[3 * i]), 3 * sizeof(float));
    }
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
    Options o = parse(argc, argv);
    try {
        std::vector<float> xyz, given_normals;
        std::vector<uint8_t> rgb;
        if (ends_with(o.input, ".ply")) read_ply(o.input, xyz, given_normals);
        else read_ascii(o.input, xyz, rgb);
        const size_t n = xyz.size() / 3;
        std::printf("[lvr2gb_reconstruct] %zu points from %s\n", n, o.input.c_str());
        if (o.pcm != "LVR2" && o.pcm != "FLANN" && o.pcm != "NANOFLANN" && o.pcm != "LBVH_CUDA" && o.pcm != "GB300")
            std::printf("[lvr2gb_reconstruct] --pcm %s: using the GB300 LBVH\n", o.pcm.c_str());
        double t0 = now_ms();
        // --pcm LBVH_CUDA makes lvr2_reconstruct use CudaKSearchSurface (Main.cpp:310-319):
        // the comparator's fit (nem 4) with k = kn, no interpolation, flipped toward
        // its fixed point.  (lvr2's CudaKSearchSurface has no distance(); the grid
        // here uses the AdaptiveKSearchSurface distance with kd.)
        const bool lbvh = o.pcm == "LBVH_CUDA";
        lvr2gb::Surface surface(xyz.data(), n, o.kn, lbvh ? 0 : o.ki, o.kd, lbvh ? 4 : o.nem, o.device);
        auto bb = surface.getBoundingBox();
        std::printf("[lvr2gb_reconstruct] BB of points: [%g, %g, %g] - [%g, %g, %g]\n", bb[0].x, bb[0].y, bb[0].z,
                    bb[1].x, bb[1].y, bb[1].z);
        // lvr2_reconstruct sets the flip point to (0,0,0) unless --flipPoint (Main.cpp:335-349)
        if (lbvh)
            surface.setFlipPoint(lvr2gb::Vec3{1e6f, 1e6f, 1e6f});
        else
            surface.setFlipPoint(lvr2gb::Vec3{o.flip[0], o.flip[1], o.flip[2]});
        if (!o.pose_file.empty()) {
            const std::vector<float> poses = read_poses(o.pose_file);
            std::printf("[lvr2gb_reconstruct] %zu scan poses from %s\n", poses.size() / 3, o.pose_file.c_str());
            surface.setScanPoses(poses);
        }
        const bool have_normals = given_normals.size() == xyz.size() && !given_normals.empty();
        if (!have_normals || o.recalc) {
            surface.calculateSurfaceNormals();
        } else {
            std::printf("[lvr2gb_reconstruct] Using given normals.\n");
            surface.setNormals(given_normals.data());
        }
        double t1 = now_ms();
        lvr2gb::GridOptions g;
        g.voxelsize = o.voxelsize;
        g.intersections = o.intersections;
        g.extrude = o.extrude;
        g.decomposition = o.decomposition;
        lvr2gb::Mesh mesh = surface.reconstruct(g);
        // calcColorFromPointCloud (Main.cpp:868): only for clouds with colours
        if (rgb.size() == xyz.size()) mesh.vertexColors = surface.vertexColors(rgb);
        double t2 = now_ms();
        std::printf("[lvr2gb_reconstruct] Grid Cells: %lld\n", (long long)mesh.info.cells_valid);
        std::printf("[lvr2gb_reconstruct] Reconstructed mesh (vertices, faces): %lld, %lld\n",
                    (long long)mesh.info.vertices, (long long)mesh.info.faces);
        std::printf("[lvr2gb_reconstruct] normals %.2f ms, grid + distance + marching cubes %.2f ms\n", t1 - t0,
                    t2 - t1);
        write_mesh_ply(o.output, mesh);
        if (o.export_normals) write_point_normals_ply("pointnormals.ply", xyz, surface.normals());
        if (o.save_grid) {
            // HashGrid::saveGrid after the reconstruction (Main.cpp:604-607)
            std::vector<float> centers, tsdf;
            surface.cellTsdf(centers, tsdf);
            std::ofstream grid("fastgrid.grid", std::ios::out | std::ios::binary);
            lvr2gb::writeGrid(grid, centers, tsdf);
            if (!grid) throw std::runtime_error("cannot write fastgrid.grid");
        }
        std::printf("[lvr2gb_reconstruct] wrote %s\n", o.output.c_str());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "[lvr2gb_reconstruct] error: %s\n", e.what());
        return 1;
    }
    return 0;
}

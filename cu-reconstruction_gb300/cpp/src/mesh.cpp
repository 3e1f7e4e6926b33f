// cuphoto::Mesh and its PLY output (reference: mesh.cpp:1-64, utils.cpp:96-119).
#include "cuphoto/mesh.hpp"

#include <cstdint>
#include <cstdio>
#include <fstream>

namespace cuphoto {

Mesh::Mesh(const std::vector<NormalColorPoint>& data_pts) { set_vertices_data(data_pts); }

void Mesh::set_vertices_data(const std::vector<NormalColorPoint>& data_pts) {
    for (const auto& pt : data_pts) {
        mesh_vertices.emplace_back(pt(0), pt(1), pt(2));
        mesh_colors.emplace_back(pt(3), pt(4), pt(5));
        mesh_normals.emplace_back(pt(6), pt(7), pt(8), pt(9));
    }
}

std::vector<Mesh::Point> Mesh::vertices() const { return mesh_vertices; }
std::vector<Mesh::Color> Mesh::colors() const { return mesh_colors; }
std::vector<Mesh::Normal> Mesh::normals() const { return mesh_normals; }
void Mesh::vertices(const std::vector<Mesh::Point>& v) { mesh_vertices = v; }
void Mesh::colors(const std::vector<Mesh::Color>& c) { mesh_colors = c; }
void Mesh::normals(const std::vector<Mesh::Normal>& n) { mesh_normals = n; }
std::vector<Mesh::Triangle> Mesh::polygons() const { return mesh_polygons; }
void Mesh::polygons(const std::vector<Mesh::Triangle>& p) { mesh_polygons = p; }

bool write_mesh_to_ply(const std::string& file_name, const std::vector<Vec3f>& vertices,
                       const std::vector<Vec3i>& triangles) {
    std::ofstream of(file_name);
    if (!of.is_open()) return false;
    of << "ply" << '\n'
       << "format ascii 1.0" << '\n'
       << "element vertex " << vertices.size() << '\n'
       << "property float x" << '\n'
       << "property float y" << '\n'
       << "property float z" << '\n'
       << "element face " << triangles.size() << '\n'
       << "property list uchar int vertex_indices" << '\n'
       << "end_header\n";
    for (const auto& v : vertices) of << v.x() << " " << v.y() << " " << v.z() << "\n";
    for (const auto& t : triangles) of << "3 " << t.x() << " " << t.y() << " " << t.z() << "\n";
    return of.good();
}

namespace {

// Binary little-endian PLY with position, colour (0..1 floats scaled to
// uchar), normal and curvature, and the faces.
bool write_binary_ply(const std::string& file_name, const std::vector<Vec3f>& v, const std::vector<Vec3f>& c,
                      const std::vector<Vec4f>& n, const std::vector<Vec3i>& f) {
    std::ofstream of(file_name, std::ios::binary);
    if (!of.is_open()) return false;
    of << "ply\nformat binary_little_endian 1.0\nelement vertex " << v.size()
       << "\nproperty float x\nproperty float y\nproperty float z\n"
          "property uchar red\nproperty uchar green\nproperty uchar blue\n"
          "property float nx\nproperty float ny\nproperty float nz\nproperty float curvature\n"
       << "element face " << f.size() << "\nproperty list uchar int vertex_indices\nend_header\n";
    for (size_t i = 0; i < v.size(); ++i) {
        of.write(reinterpret_cast<const char*>(v[i].v), 12);
        for (int k = 0; k < 3; ++k) {
            const float x = i < c.size() ? c[i](k) : 0.f;
            const uint8_t b = (uint8_t)(x <= 0.f ? 0 : x >= 1.f ? 255 : x * 255.f + 0.5f);
            of.write(reinterpret_cast<const char*>(&b), 1);
        }
        const Vec4f nn = i < n.size() ? n[i] : Vec4f();
        of.write(reinterpret_cast<const char*>(nn.v), 16);
    }
    for (const auto& t : f) {
        const uint8_t three = 3;
        of.write(reinterpret_cast<const char*>(&three), 1);
        of.write(reinterpret_cast<const char*>(t.v), 12);
    }
    return of.good();
}

}  // namespace

void Mesh::store_to_ply(const std::string& ply_filepath) const {
    // mesh.cpp:59-64
    if (mesh_normals.empty())
        write_mesh_to_ply(ply_filepath, mesh_vertices, mesh_polygons);
    else
        write_binary_ply(ply_filepath, mesh_vertices, mesh_colors, mesh_normals, mesh_polygons);
}

}  // namespace cuphoto

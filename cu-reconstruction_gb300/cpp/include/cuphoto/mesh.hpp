// cuphoto::Mesh (reference: modules/include/mesh.hpp:12-47, mesh.cpp:1-64).
// store_to_ply writes the reference's ASCII PLY when the mesh has no normals
// (utils.cpp:96-119); with normals it writes a binary little-endian PLY with
// per-vertex colour and normal (the reference hands that case to PCL).
#ifndef CUPHOTO_GB300_MESH_HPP
#define CUPHOTO_GB300_MESH_HPP

#include <string>
#include <vector>

#include "geometry.hpp"

namespace cuphoto {

class Mesh {
public:
    using Point = Vec3f;
    using Color = Vec3f;
    using Normal = Vec4f;
    using ColorPoint = Vec6f;
    using NormalColorPoint = Vec10f;
    using Triangle = Vec3i;

public:
    Mesh() = default;
    Mesh(const std::vector<NormalColorPoint>& data_pts);

    void set_vertices_data(const std::vector<NormalColorPoint>& data_pts);

    std::vector<Mesh::Point> vertices() const;
    std::vector<Mesh::Color> colors() const;
    std::vector<Mesh::Normal> normals() const;

    void colors(const std::vector<Mesh::Color>& mesh_colors);
    void vertices(const std::vector<Mesh::Point>& mesh_vertices);
    void normals(const std::vector<Mesh::Normal>& mesh_normals);

    std::vector<Mesh::Triangle> polygons() const;
    void polygons(const std::vector<Mesh::Triangle>& mesh_faces);

    void store_to_ply(const std::string& ply_filepath) const;

private:
    std::vector<Point> mesh_vertices;
    std::vector<Color> mesh_colors;
    std::vector<Normal> mesh_normals;
    std::vector<Triangle> mesh_polygons;
};

// ASCII PLY of utils.cpp:96-119 ("element vertex / element face / property
// list uchar int vertex_indices").
bool write_mesh_to_ply(const std::string& file_name, const std::vector<Vec3f>& vertices,
                       const std::vector<Vec3i>& triangles);

}  // namespace cuphoto

#endif

// Stand-in for the header of the tinyobjloader library (an empty git submodule in the
// reference checkout), so that the reference's core/meshio.cc compiles for the oracle.
// It declares only what meshio.cc's loadOBJ touches, with the library's public names;
// LoadObj always fails (the oracle loads PLY files only).  Test infrastructure.
#pragma once

#include <string>
#include <vector>

namespace tinyobj {

struct index_t {
    int vertex_index = -1;
    int normal_index = -1;
    int texcoord_index = -1;
};

struct mesh_t {
    std::vector<index_t> indices;
};

struct shape_t {
    std::string name;
    mesh_t mesh;
};

struct attrib_t {
    std::vector<float> vertices, normals, texcoords;
};

struct material_t {};

inline bool LoadObj(attrib_t *, std::vector<shape_t> *, std::vector<material_t> *, std::string *err, const char *) {
    if (err) *err = "OBJ loading is not available in the oracle build";
    return false;
}

}  // namespace tinyobj

// ref_mesh_stub.cpp -- link stand-ins for the reference's triangle-mesh
// loader (mesh.cpp needs the unvendored miniScene library).  TEST
// INFRASTRUCTURE ONLY: the chopSuey tool is built from the reference sources
// for its raw-volume path (.raw -> .vol); its .obj path is out of scope and
// fails with an exception here.
#include <stdexcept>

#include "mesh.h"

namespace maui {

Mesh::SP Mesh::loadOBJ(std::string) { throw std::runtime_error("triangle meshes are not built"); }
Mesh::SP Mesh::loadMini(std::string) { throw std::runtime_error("triangle meshes are not built"); }
Mesh::SP Mesh::load(std::string) { throw std::runtime_error("triangle meshes are not built"); }

}  // namespace maui

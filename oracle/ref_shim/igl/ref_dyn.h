/* Test infrastructure: stand-ins for the sparse Eigen types and the libigl calls that the
 * reference's include/mesh_builder.h names besides marching cubes (mesh smoothing,
 * decimation), plus an OBJ writer that keeps the mesh in memory.  The oracle runs
 * MeshBuilder::computeMesh without smoothing or decimation, so every stand-in but
 * writeOBJ aborts if it is ever called. */
#pragma once
#include <string>
#include <vector>

#include <Eigen/Dense>

namespace Eigen {

template <class T>
using SparseMatrix = SparseStub;

enum ComputationInfo { Success = 0 };

template <class M>
struct SimplicialLLT {
  explicit SimplicialLLT(const SparseStub&) { shim_unsupported("SimplicialLLT"); }
  ComputationInfo info() const { return Success; }
  SparseStub solve(const SparseStub&) const { shim_unsupported("SimplicialLLT::solve"); }
};

}  // namespace Eigen

namespace igl {

enum MassMatrixType { MASSMATRIX_TYPE_BARYCENTRIC = 0 };

template <class... A>
void cotmatrix(A&&...) { Eigen::shim_unsupported("igl::cotmatrix"); }
template <class... A>
void grad(A&&...) { Eigen::shim_unsupported("igl::grad"); }
template <class... A>
void doublearea(A&&...) { Eigen::shim_unsupported("igl::doublearea"); }
template <class... A>
void massmatrix(A&&...) { Eigen::shim_unsupported("igl::massmatrix"); }
template <class... A>
void barycenter(A&&...) { Eigen::shim_unsupported("igl::barycenter"); }
template <class... A>
bool decimate(A&&...) { Eigen::shim_unsupported("igl::decimate"); }

// The mesh MeshBuilder::computeMesh hands to writeOBJ: V row-major (nv x 3), F (nf x 3).
struct WrittenMesh {
  std::string path;
  std::vector<double> V;
  std::vector<int> F;
};
inline WrittenMesh& written_mesh() {
  static WrittenMesh m;
  return m;
}

template <class DV, class DF>
bool writeOBJ(const std::string& path, const DV& V, const DF& F) {
  WrittenMesh& m = written_mesh();
  m.path = path;
  m.V.resize(V.rows() * 3);
  m.F.resize(F.rows() * 3);
  for (long i = 0; i < V.rows(); ++i)
    for (int c = 0; c < 3; ++c) m.V[3 * i + c] = V(i, c);
  for (long i = 0; i < F.rows(); ++i)
    for (int c = 0; c < 3; ++c) m.F[3 * i + c] = F(i, c);
  return true;
}

}  // namespace igl

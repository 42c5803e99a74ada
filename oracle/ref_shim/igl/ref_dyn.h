/* Test infrastructure: declaration-only stand-ins for the dynamic Eigen types and the
 * libigl calls that the reference's include/mesh_builder.h names in its mesh and
 * smoothing code.  They exist so that header compiles for the host; the oracle only
 * calls its fillVoxelGrid_distance, so none of these is ever executed (every operation
 * is a no-op returning an empty value). */
#pragma once
#include <cmath>
#include <string>

namespace Eigen {

struct Dyn {
  double v = 0.0;
  Dyn() {}
  Dyn(long) {}
  Dyn(long, long) {}
  double& operator()(long, long) { return v; }
  Dyn replicate(int, int) const { return Dyn(); }
  Dyn asDiagonal() const { return Dyn(); }
  Dyn transpose() const { return Dyn(); }
  Dyn eval() const { return Dyn(); }
  Dyn& array() { return *this; }
  double sum() const { return 0.0; }
  Dyn& operator/=(double) { return *this; }
  Dyn operator-() const { return Dyn(); }
  Dyn operator*(const Dyn&) const { return Dyn(); }
  Dyn operator*(double) const { return Dyn(); }
  Dyn operator-(const Dyn&) const { return Dyn(); }
};
inline Dyn operator*(double, const Dyn&) { return Dyn(); }

using MatrixXd = Dyn;
using MatrixXi = Dyn;
using VectorXd = Dyn;
using VectorXi = Dyn;
template <class T>
using SparseMatrix = Dyn;

enum ComputationInfo { Success = 0 };

template <class M>
struct SimplicialLLT {
  explicit SimplicialLLT(const Dyn&) {}
  ComputationInfo info() const { return Success; }
  Dyn solve(const Dyn&) const { return Dyn(); }
};

}  // namespace Eigen

namespace igl {

enum MassMatrixType { MASSMATRIX_TYPE_BARYCENTRIC = 0 };

template <class... A>
void cotmatrix(A&&...) {}
template <class... A>
void grad(A&&...) {}
template <class... A>
void doublearea(A&&...) {}
template <class... A>
void massmatrix(A&&...) {}
template <class... A>
void barycenter(A&&...) {}
template <class... A>
bool decimate(A&&...) { return false; }
template <class... A>
bool writeOBJ(A&&...) { return false; }

namespace copyleft {
template <class... A>
void marching_cubes(A&&...) {}
}  // namespace copyleft

}  // namespace igl

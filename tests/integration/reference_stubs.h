// Stand-ins for the reference types that the INTEGRATION.md shims touch
// (test infrastructure). Each declaration keeps the reference's name, member
// names and signature for the members the shims use:
//
//   scisim/Math/MathDefines.h:32-85      scalar, VectorXs, VectorXi, Vector2s,
//                                        Array2s, Array2u, Matrix2Xsc, Matrix22sc
//   mpmgrains2d/StaticPlane.h:6-22       MPMStaticPlane
//   mpmgrains2d/BasisFunctions.h:11-31   BasisFunctionType, BasisFunctions::type
//   mpmgrains2d/MaterialPoints.h:118-156 MaterialPoints fields
//   mpmgrains2d/PhysicsGrid.h:68-87      PhysicsGrid fields
//   mpmgrains2d/SimulationState.h:16-68  SimulationState fields
//   mpmgrains2d/ExplicitIntegrator.h:8-13  ExplicitIntegrator::flow*
//   scisim/ConstrainedMaps/ImpactFrictionMap.h:32-80  ImpactFrictionMap
//   rigidbody2d/RigidBody2DGeometry.h:8-16, CircleGeometry.h:6-24
//   rigidbody2d/RigidBody2DState.h:32-58, 108-109, 152-154  RigidBody2DState
//
// Eigen is not available here, so the dense types are plain arrays with the
// Eigen members the shims call (data(), size(), cols(), x(), y(),
// operator()); the storage orders are Eigen's (column-major 2 x N,
// column-major 2 x 2 blocks). The bodies of RigidBody2DState hold plain
// vectors and add a test-only builder (add_circle, remove_marked) that
// mirrors RigidBody2DState::addBody / removeBodies
// (RigidBody2DState.cpp:237-336, 645-660), including their calls into the
// impact map.
#ifndef HG_REFERENCE_STUBS_H
#define HG_REFERENCE_STUBS_H

#include <cmath>
#include <cstdint>
#include <iosfwd>
#include <limits>
#include <memory>
#include <string>
#include <vector>

using scalar = double;

struct VectorXs {
  std::vector<double> a;
  VectorXs() = default;
  explicit VectorXs(long n) : a((size_t)n, 0.0) {}
  long size() const { return (long)a.size(); }
  double *data() { return a.data(); }
  const double *data() const { return a.data(); }
  double &operator()(long i) { return a[(size_t)i]; }
  double operator()(long i) const { return a[(size_t)i]; }
  void resize(long n) { a.resize((size_t)n); }
};

struct VectorXi {
  std::vector<int> a;
  long size() const { return (long)a.size(); }
  int *data() { return a.data(); }
  const int *data() const { return a.data(); }
  void resize(long n) { a.resize((size_t)n); }
};

struct Vector2s {
  double v[2] = {0.0, 0.0};
  double &x() { return v[0]; }
  double &y() { return v[1]; }
  const double &x() const { return v[0]; }
  const double &y() const { return v[1]; }
};
using Array2s = Vector2s;

struct Array2u {
  unsigned v[2] = {0u, 0u};
  unsigned x() const { return v[0]; }
  unsigned y() const { return v[1]; }
};

// Eigen::Matrix<scalar, 2, Eigen::Dynamic, Eigen::ColMajor>
struct Matrix2Xsc {
  std::vector<double> a;
  long cols() const { return (long)a.size() / 2; }
  double *data() { return a.data(); }
  const double *data() const { return a.data(); }
  void resize(long rows, long cols) { (void)rows; a.resize(2 * (size_t)cols); }
};

// Eigen::Matrix<scalar, 2, 2, Eigen::ColMajor>
struct Matrix22sc {
  double a[4] = {1.0, 0.0, 0.0, 1.0};
  double *data() { return a; }
  const double *data() const { return a; }
};

// ---- mpmgrains2d -----------------------------------------------------------

struct MPMStaticPlane final {
  enum class BoundaryBehavior { SLIDING, STICKING };
  Vector2s x;
  Vector2s n;
  BoundaryBehavior boundary_behavior = BoundaryBehavior::STICKING;
  scalar lower_bound = -std::numeric_limits<scalar>::infinity();
};

enum class BasisFunctionType { Linear, ThirdOrder, uGIMPLinear };

struct BasisFunctions {
  virtual ~BasisFunctions() = default;
  virtual BasisFunctionType type() const = 0;
};

struct MaterialPoints {
  unsigned npoints = 0;
  Matrix2Xsc q0, q, v;
  VectorXs m, volume, m0, volume0, weight, hl;
  std::vector<Matrix22sc> be_bar;
  VectorXs J;
  std::vector<Matrix22sc> sigma, vel_grad;
  VectorXi just_homogenized;
  std::vector<bool> always_fixed;
  std::vector<bool> kinematically_scripted;
};

struct PhysicsGrid {
  Array2s min;
  Array2s max;
  scalar cell_width = 0.0;
  Array2u cell_count;
  VectorXs rasterized_mass;
  Matrix2Xsc velocity;
  Matrix2Xsc acceleration;
};

struct SimulationState final {
  MaterialPoints material_points;
  PhysicsGrid physics_grid;
  std::vector<MPMStaticPlane> static_planes;
  scalar shear_modulus = 0.0;
  scalar bulk_modulus = 0.0;
  scalar Drucker_Prager_alpha = 0.0;
  Vector2s near_earth_gravity;
  scalar alpha = 0.0;
  std::unique_ptr<BasisFunctions> basis_functions;
};

namespace ExplicitIntegrator {
void flow(const scalar &dt, SimulationState &state);
void flow_zero_phase(SimulationState &state);
void flow_first_phase(const scalar &dt, SimulationState &state);
void flow_second_phase(const scalar &dt, SimulationState &state);
} // namespace ExplicitIntegrator

// ---- scisim / rigidbody2d ----------------------------------------------------

class ScriptingCallback;
class FlowableSystem;
class ConstrainedSystem;
class UnconstrainedMap;
class FrictionSolver;
class HDF5File;
struct CollisionImpulses;

class ImpactFrictionMap {
public:
  ImpactFrictionMap(const ImpactFrictionMap &) = delete;
  ImpactFrictionMap &operator=(const ImpactFrictionMap &) = delete;
  virtual ~ImpactFrictionMap() = default;
  virtual void flow(ScriptingCallback &call_back, FlowableSystem &fsys,
                    ConstrainedSystem &csys, UnconstrainedMap &umap,
                    FrictionSolver &friction_solver, const unsigned iteration,
                    const scalar &dt, const scalar &CoR, const scalar &mu_default,
                    const bool reduce_bandwidth, const VectorXs &q0, const VectorXs &v0,
                    VectorXs &q1, VectorXs &v1) = 0;
  virtual void flowWithWeights(ScriptingCallback &call_back, FlowableSystem &fsys,
                               ConstrainedSystem &csys, UnconstrainedMap &umap,
                               FrictionSolver &friction_solver, const unsigned iteration,
                               const scalar &dt, const scalar &CoR, const scalar &mu_default,
                               const bool reduce_bandwidth, const VectorXs &q0,
                               const VectorXs &v0, const VectorXs &w, VectorXs &q1,
                               VectorXs &v1) = 0;
  virtual void resetCachedData() = 0;
  virtual void serialize(std::ostream &output_stream) const = 0;
  virtual std::string name() const = 0;
  virtual void exportForcesNextStep(HDF5File &output_file) = 0;
  virtual void saveImpulsesNextStep(CollisionImpulses &impulses) = 0;
  virtual std::unique_ptr<ImpactFrictionMap> clone() const = 0;
  virtual bool stabilize() const { return false; }
  virtual void enlargeCache(const int new_size) { (void)new_size; }
  virtual void deleteCacheEntries(const VectorXs &q) { (void)q; }

protected:
  ImpactFrictionMap() = default;
};

enum class RigidBody2DGeometryType { ANNULUS, CIRCLE, BOX };

class RigidBody2DGeometry {
public:
  virtual ~RigidBody2DGeometry() = default;
  virtual RigidBody2DGeometryType type() const = 0;
};

class CircleGeometry final : public RigidBody2DGeometry {
public:
  explicit CircleGeometry(const scalar &r) : m_r(r) {}
  RigidBody2DGeometryType type() const override { return RigidBody2DGeometryType::CIRCLE; }
  const scalar &r() const { return m_r; }

private:
  scalar m_r;
};

class RigidBody2DState {
public:
  unsigned nbodies() const { return (unsigned)(m_q.size() / 3); }
  VectorXs &q() { return m_q; }
  const VectorXs &q() const { return m_q; }
  VectorXs &v() { return m_v; }
  const VectorXs &v() const { return m_v; }
  const scalar &m(const unsigned bdy_idx) const { return m_M[3 * bdy_idx]; }
  const scalar &I(const unsigned bdy_idx) const { return m_M[3 * bdy_idx + 2]; }
  bool fixed(const int idx) const { return m_fixed[(size_t)idx] != 0; }
  const std::unique_ptr<RigidBody2DGeometry> &bodyGeometry(const unsigned bdy_idx) const {
    return m_geo[bdy_idx];
  }
  const VectorXs &massWeights() const { return m_w; }
  scalar &massWeight(const unsigned idx) { return m_w(idx); }

  // ---- test-only builders (not reference API) ----
  // addBody for a circle: M0 = M for every body afterwards, as in
  // RigidBody2DState.cpp:299, then ifmap->enlargeCache(nbodies()) (:333-335)
  void add_circle(const double q[3], const double v[3], double r, double m, double I,
                  bool fixed, ImpactFrictionMap *ifmap) {
    for (int c = 0; c < 3; ++c) {
      m_q.a.push_back(q[c]);
      m_v.a.push_back(v[c]);
    }
    m_M.push_back(m);
    m_M.push_back(m);
    m_M.push_back(I);
    m_fixed.push_back(fixed ? 1 : 0);
    m_w.a.push_back(1.0);
    m_geo.emplace_back(new CircleGeometry(r));
    if (ifmap) ifmap->enlargeCache((int)nbodies());
  }
  // removeBodies: the removed bodies' x marked NaN, ifmap->deleteCacheEntries(q)
  // (RigidBody2DState.cpp:651-658), then the arrays compacted
  void remove_marked(const std::vector<unsigned> &idx, ImpactFrictionMap *ifmap) {
    for (unsigned i : idx) m_q(3 * i) = std::numeric_limits<double>::quiet_NaN();
    if (ifmap) ifmap->deleteCacheEntries(m_q);
    const unsigned n = nbodies();
    unsigned k = 0;
    for (unsigned i = 0; i < n; ++i) {
      if (std::isnan(m_q(3 * i))) continue;
      for (int c = 0; c < 3; ++c) {
        m_q(3 * k + c) = m_q(3 * i + c);
        m_v(3 * k + c) = m_v(3 * i + c);
        m_M[3 * k + c] = m_M[3 * i + c];
      }
      m_fixed[k] = m_fixed[i];
      m_w(k) = m_w(i);
      m_geo[k] = std::move(m_geo[i]);
      ++k;
    }
    m_q.resize(3 * k);
    m_v.resize(3 * k);
    m_M.resize(3 * k);
    m_fixed.resize(k);
    m_w.resize(k);
    m_geo.resize(k);
  }

private:
  VectorXs m_q, m_v, m_w;
  std::vector<double> m_M;
  std::vector<uint8_t> m_fixed;
  std::vector<std::unique_ptr<RigidBody2DGeometry>> m_geo;
};

#endif

// KalmanFitter.hpp — header-only C++ drop-in for the reference fitter's API,
// over the gb300kf C ABI.
//
// A caller written against the reference's fitter compiles against this
// header with its includes changed: the type names, template parameters and
// call signatures are the reference's, and the fit runs on the GPU through
// kf_fit_batch_host.  Reference interfaces mirrored (paths relative to the
// reference project):
//   KalmanFitter<P, U, S, O>::fit           include/Fitter/KalmanFitter.hpp:716-768
//   KalmanFitterOptions<O>                  include/Fitter/KalmanFitter.hpp:48-96
//   KalmanFitterResult<SL, P, T>            include/Fitter/KalmanFitter.hpp:98-120
//   CudaKernelContainer<T>                  include/Utilities/CudaKernelContainer.hpp:18-71
//   TrackState<SL, P>                       include/EventData/TrackState.hpp:38-169
//   PixelSourceLink                         include/EventData/PixelSourceLink.hpp:22-75
//   SingleBoundTrackParameters / BoundParameters
//                                           include/EventData/SingleBoundTrackParameters.hpp:27-105
//   Propagator<S>, EigenStepper<B>          include/Propagator/Propagator.hpp, EigenStepper.hpp
//   GainMatrixUpdater, GainMatrixSmoother<P> include/Fitter/GainMatrixUpdater.hpp, GainMatrixSmoother.hpp
//   VoidOutlierFinder                       include/Fitter/detail/VoidKalmanComponents.hpp:67-80
//   PlaneSurface<InfiniteBounds>(center, normal[, material])
//                                           include/Surfaces/PlaneSurface.hpp:69-80
//   LineSurface(point)                      include/Surfaces/LineSurface.hpp:57
//   GeometryID set/get of its fields        include/Geometry/GeometryID.hpp:30-125
//   Material, MaterialSlab, HomogeneousSurfaceMaterial, Test::makeSilicon
//                                           include/Material/*, include/Test/Helper.hpp:25-29
//   Test::ConstantBField                    include/Test/Helper.hpp:17-22
//   InterpolatedBFieldMap from a text map   src/Plugins/BFieldOptions.cpp:33-61
//   Vector/matrix types with Eigen's comma initialiser (values << a, b;)
//   and the bound/free parameter indices    include/Utilities/Definitions.hpp,
//                                           ParameterDefinitions.hpp
//   units (Acts::units::_mm, UnitConstants) include/Utilities/Units.hpp
//
// So the typedefs of the reference driver (Run/Common/FitData.hpp:26-43) and
// its fit loop (Run/GPU/KalmanFitterGPUTest.cu:539-560, Run/GPU/Kernels.cu:
// 6-45) compile unchanged.  fit() fits one track per call, as the
// reference's does (thread-safe: concurrent calls from an OpenMP loop use one
// CUDA stream per host thread); fitBatch() takes the arrays the reference's
// GPU kernel takes and fits all tracks in one launch, the intended use.
//
// What a fitted TrackState holds: the source link, the geometry id, the
// measurement flag and the smoothed parameters with their covariance
// (parameter.smoothed).  The predicted and filtered parameters and the
// per-state Jacobian are not returned by the C ABI and stay default; the
// per-state chi2 is 0, as the reference's updater leaves it
// (GainMatrixUpdater.hpp:90-101).
//
// Names live in namespace gb300kf (and gb300kf::test for the reference's
// Test:: helpers); define GB300KF_ACTS_NAMESPACE before the include to also
// expose them as namespaces Acts and Test.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <bitset>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <ios>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../gb300kf.h"
#include "../gb300kf_fieldmap.h"
#include "../gb300kf_io.h"

namespace gb300kf {

using ActsScalar = double;

// ---------------------------------------------------------------------------
// Fixed-size matrices: the subset of the Eigen types the reference's API is
// written in (construction from coefficients, Zero/Identity, element access,
// the comma initialiser `m << a, b, ...;`, row-major order).
// ---------------------------------------------------------------------------
template <int R, int C> class Matrix {
public:
  static constexpr int RowsAtCompileTime = R, ColsAtCompileTime = C;
  Matrix() : m_a{} {}
  template <typename... T,
            typename = std::enable_if_t<(sizeof...(T) == R * C) && (R * C > 1) &&
                                        (std::is_arithmetic_v<T> && ...)>>
  Matrix(T... v) : m_a{static_cast<double>(v)...} {}
  static Matrix Zero() { return Matrix(); }
  static Matrix Identity() {
    Matrix m;
    for (int i = 0; i < (R < C ? R : C); ++i) m(i, i) = 1.;
    return m;
  }
  double &operator()(int r, int c) { return m_a[r * C + c]; }
  double operator()(int r, int c) const { return m_a[r * C + c]; }
  double &operator()(int i) { return m_a[i]; }
  double operator()(int i) const { return m_a[i]; }
  double &operator[](int i) { return m_a[i]; }
  double operator[](int i) const { return m_a[i]; }
  double x() const { return m_a[0]; }
  double y() const { return m_a[1]; }
  double z() const { return m_a[2]; }
  double *data() { return m_a; }
  const double *data() const { return m_a; }
  static constexpr int rows() { return R; }
  static constexpr int cols() { return C; }

  class CommaInitializer {
  public:
    CommaInitializer(Matrix &m, double v) : m_m(m) { put(v); }
    CommaInitializer &operator,(double v) {
      put(v);
      return *this;
    }
    ~CommaInitializer() noexcept(false) {
      if (m_i != R * C && !std::uncaught_exceptions())
        throw std::invalid_argument("comma initialiser: wrong number of coefficients");
    }

  private:
    void put(double v) {
      if (m_i >= R * C) throw std::invalid_argument("comma initialiser: too many coefficients");
      m_m.m_a[m_i++] = v;
    }
    Matrix &m_m;
    int m_i = 0;
  };
  CommaInitializer operator<<(double v) { return CommaInitializer(*this, v); }

  friend Matrix operator+(const Matrix &a, const Matrix &b) {
    Matrix r;
    for (int i = 0; i < R * C; ++i) r.m_a[i] = a.m_a[i] + b.m_a[i];
    return r;
  }
  friend Matrix operator-(const Matrix &a, const Matrix &b) {
    Matrix r;
    for (int i = 0; i < R * C; ++i) r.m_a[i] = a.m_a[i] - b.m_a[i];
    return r;
  }
  friend Matrix operator*(double s, const Matrix &a) {
    Matrix r;
    for (int i = 0; i < R * C; ++i) r.m_a[i] = s * a.m_a[i];
    return r;
  }
  double dot(const Matrix &b) const {
    double s = 0.;
    for (int i = 0; i < R * C; ++i) s += m_a[i] * b.m_a[i];
    return s;
  }
  double norm() const { return std::sqrt(dot(*this)); }

private:
  double m_a[R * C];
};

using Vector2D = Matrix<2, 1>;
using Vector3D = Matrix<3, 1>;
using SymMatrix2D = Matrix<2, 2>;
using BoundVector = Matrix<6, 1>;
using BoundSymMatrix = Matrix<6, 6>;
using BoundMatrix = Matrix<6, 6>;

inline Vector3D cross(const Vector3D &a, const Vector3D &b) {
  return Vector3D(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                  a[0] * b[1] - a[1] * b[0]);
}

/// Bound parameter order (loc0, loc1, phi, theta, q/p, t) and free order
/// (position, time, direction, q/p), Utilities/ParameterDefinitions.hpp.
enum BoundIndices : unsigned int {
  eBoundLoc0 = 0, eBoundLoc1 = 1, eBoundPhi = 2, eBoundTheta = 3, eBoundQOverP = 4,
  eBoundTime = 5, eBoundSize = 6
};
enum FreeIndices : unsigned int {
  eFreePos0 = 0, eFreePos1 = 1, eFreePos2 = 2, eFreeTime = 3, eFreeDir0 = 4, eFreeDir1 = 5,
  eFreeDir2 = 6, eFreeQOverP = 7, eFreeSize = 8
};

/// Native units: mm, GeV, e, time in mm (c = 1); the field in GeV/(e mm).
namespace UnitConstants {
constexpr double um = 1e-3, mm = 1.0, cm = 10.0, m = 1e3;
constexpr double cm3 = cm * cm * cm;
constexpr double s = 299792458000.0, ns = 1e-9 * s, ps = 1e-12 * s;
constexpr double mrad = 1e-3, rad = 1.0;
constexpr double eV = 1e-9, keV = 1e-6, MeV = 1e-3, GeV = 1.0;
constexpr double T = 0.000299792458, Gauss = 1e-4 * T;
constexpr double mol = 1.0;
} // namespace UnitConstants
namespace units {
constexpr double _um = UnitConstants::um, _mm = UnitConstants::mm, _cm = UnitConstants::cm,
                 _m = UnitConstants::m, _ns = UnitConstants::ns, _ps = UnitConstants::ps,
                 _MeV = UnitConstants::MeV, _GeV = UnitConstants::GeV, _T = UnitConstants::T,
                 _mrad = UnitConstants::mrad;
} // namespace units

constexpr double kTesla = UnitConstants::T;

// ---------------------------------------------------------------------------
// Contexts and identifiers
// ---------------------------------------------------------------------------
struct GeometryContext {
  GeometryContext(int = 0) {}
};
struct MagneticFieldContext {
  MagneticFieldContext(int = 0) {}
};

/// Surface identifier with the reference's fields (volume, boundary, layer,
/// approach, sensitive); only equality matters to the fit.
class GeometryID {
public:
  using Value = uint64_t;
  constexpr GeometryID() = default;
  constexpr GeometryID(Value encoded) : m_value(encoded) {}
  constexpr Value value() const { return m_value; }
  constexpr Value volume() const { return get(kVolume); }
  constexpr Value boundary() const { return get(kBoundary); }
  constexpr Value layer() const { return get(kLayer); }
  constexpr Value approach() const { return get(kApproach); }
  constexpr Value sensitive() const { return get(kSensitive); }
  constexpr GeometryID &setVolume(Value v) { return set(kVolume, v); }
  constexpr GeometryID &setBoundary(Value v) { return set(kBoundary, v); }
  constexpr GeometryID &setLayer(Value v) { return set(kLayer, v); }
  constexpr GeometryID &setApproach(Value v) { return set(kApproach, v); }
  constexpr GeometryID &setSensitive(Value v) { return set(kSensitive, v); }
  friend constexpr bool operator==(GeometryID a, GeometryID b) { return a.m_value == b.m_value; }
  friend constexpr bool operator!=(GeometryID a, GeometryID b) { return a.m_value != b.m_value; }

private:
  // (shift, width) of each field in a 64-bit word
  struct Field {
    int shift, bits;
  };
  static constexpr Field kVolume{48, 16}, kBoundary{40, 8}, kLayer{28, 12}, kApproach{20, 8},
      kSensitive{0, 20};
  static constexpr Value mask(Field f) { return ((Value(1) << f.bits) - 1) << f.shift; }
  constexpr Value get(Field f) const { return (m_value & mask(f)) >> f.shift; }
  constexpr GeometryID &set(Field f, Value v) {
    m_value = (m_value & ~mask(f)) | ((v << f.shift) & mask(f));
    return *this;
  }
  Value m_value = 0;
};

// ---------------------------------------------------------------------------
// Material (Material/Material.hpp, MaterialSlab.hpp,
// HomogeneousSurfaceMaterial.hpp): what the fit's material effects read.
// ---------------------------------------------------------------------------
class Material {
public:
  Material() = default;
  /// X0, L0 (mm), Ar, Z, molar density (mol/mm^3)
  static Material fromMolarDensity(double X0, double L0, double Ar, double Z,
                                   double molarDensity) {
    Material m;
    m.m_x0 = X0;
    m.m_l0 = L0;
    m.m_ar = Ar;
    m.m_z = Z;
    m.m_molarRho = molarDensity;
    return m;
  }
  double X0() const { return m_x0; }
  double L0() const { return m_l0; }
  double Ar() const { return m_ar; }
  double Z() const { return m_z; }
  double molarDensity() const { return m_molarRho; }
  explicit operator bool() const { return m_ar > 0.; }

private:
  double m_x0 = 0., m_l0 = 0., m_ar = 0., m_z = 0., m_molarRho = 0.;
};

class MaterialSlab {
public:
  MaterialSlab() = default;
  MaterialSlab(const Material &material, double thickness)
      : m_material(material), m_thickness(thickness) {}
  const Material &material() const { return m_material; }
  double thickness() const { return m_thickness; }

private:
  Material m_material;
  double m_thickness = 0.;
};

class HomogeneousSurfaceMaterial {
public:
  HomogeneousSurfaceMaterial() = default;
  explicit HomogeneousSurfaceMaterial(const MaterialSlab &slab) : m_slab(slab) {}
  const MaterialSlab &materialSlab() const { return m_slab; }

private:
  MaterialSlab m_slab;
};

// ---------------------------------------------------------------------------
// Surfaces.  Every concrete surface has the base's size, so that a surface
// sequence handed over as `const Surface *` (an array of one concrete type,
// as the reference's navigator steps through it) indexes correctly.
// ---------------------------------------------------------------------------
struct InfiniteBounds {};

class Surface {
public:
  enum SurfaceType { Plane = 0, Straw = 1 };
  const Vector3D &center(const GeometryContext & = GeometryContext()) const { return m_center; }
  /// rotation columns U, V, T (T the plane normal / the line axis), row-major
  const std::array<double, 9> &rotation() const { return m_rot; }
  SurfaceType type() const { return m_type; }
  GeometryID geoID() const { return m_id; }
  void assignGeoID(const GeometryID &id) { m_id = id; }
  const HomogeneousSurfaceMaterial &surfaceMaterial() const { return m_material; }

protected:
  Surface() = default;
  Vector3D m_center{0., 0., 0.};
  std::array<double, 9> m_rot{1., 0., 0., 0., 1., 0., 0., 0., 1.};
  HomogeneousSurfaceMaterial m_material;
  GeometryID m_id;
  SurfaceType m_type = Plane;
};

/// Boundless plane with the reference's frame: T = normal, U = z x T (x x T
/// when T is along z), V = T x U (PlaneSurface.ipp:24-46).
template <typename bounds_t = InfiniteBounds> class PlaneSurface : public Surface {
public:
  PlaneSurface() = default;
  PlaneSurface(const Vector3D &center, const Vector3D &normal,
               const HomogeneousSurfaceMaterial &material = HomogeneousSurfaceMaterial()) {
    m_type = Plane;
    m_center = center;
    m_material = material;
    const double n = normal.norm();
    const Vector3D T(normal[0] / n, normal[1] / n, normal[2] / n);
    const Vector3D a = std::fabs(T[2]) < 0.999995 ? Vector3D(0., 0., 1.) : Vector3D(1., 0., 0.);
    Vector3D U = cross(a, T);
    U = (1. / U.norm()) * U;
    const Vector3D V = cross(T, U);
    for (int r = 0; r < 3; ++r) {
      m_rot[3 * r + 0] = U[r];
      m_rot[3 * r + 1] = V[r];
      m_rot[3 * r + 2] = T[r];
    }
  }
  Vector3D normal(const GeometryContext & = GeometryContext()) const {
    return Vector3D(m_rot[2], m_rot[5], m_rot[8]);
  }
  /// global position to local (U, V) coordinates (PlaneSurface.ipp:215-223)
  bool globalToLocal(const GeometryContext &, const Vector3D &position, const Vector3D &,
                     Vector2D &local) const {
    const Vector3D d = position - m_center;
    local[0] = d[0] * m_rot[0] + d[1] * m_rot[3] + d[2] * m_rot[6];
    local[1] = d[0] * m_rot[1] + d[1] * m_rot[4] + d[2] * m_rot[7];
    return true;
  }
};
static_assert(sizeof(PlaneSurface<InfiniteBounds>) == sizeof(Surface),
              "a surface sequence is indexed as an array of Surface");

/// Line surface through a point with axis z (the perigee target).
class LineSurface : public Surface {
public:
  LineSurface() { m_type = Straw; }
  explicit LineSurface(const Vector3D &point) {
    m_type = Straw;
    m_center = point;
  }
};
static_assert(sizeof(LineSurface) == sizeof(Surface), "concrete surfaces add no data");

// ---------------------------------------------------------------------------
// Measurements and parameters
// ---------------------------------------------------------------------------
/// 2D pixel measurement on a surface (PixelSourceLink.hpp:22-75).
class PixelSourceLink {
public:
  using meas_par_t = Vector2D;
  using meas_cov_t = SymMatrix2D;
  PixelSourceLink() = default;
  PixelSourceLink(const Vector2D &values, const SymMatrix2D &cov, GeometryID gid)
      : m_values(values), m_cov(cov), m_geometryId(gid) {}
  const Vector2D &localPosition() const { return m_values; }
  const SymMatrix2D &covariance() const { return m_cov; }
  GeometryID geometryId() const { return m_geometryId; }

private:
  Vector2D m_values;
  SymMatrix2D m_cov;
  GeometryID m_geometryId;
};

/// Parameters (loc0, loc1, phi, theta, q/p, t) with covariance bound to a
/// surface (SingleBoundTrackParameters.hpp:27-105).
template <typename surface_t> class BoundParameters {
public:
  using ParametersVector = BoundVector;
  using CovarianceMatrix = BoundSymMatrix;
  using ReferenceSurfaceType = surface_t;
  BoundParameters() = default;
  BoundParameters(const GeometryContext &, const BoundSymMatrix &cov, const BoundVector &pars,
                  const Surface *surface)
      : m_pars(pars), m_cov(cov), m_surface(surface) {}
  const BoundVector &parameters() const { return m_pars; }
  const BoundSymMatrix *covariance() const { return &m_cov; }
  const Surface &referenceSurface() const { return *m_surface; }
  const Surface *referenceSurfacePtr() const { return m_surface; }
  double charge() const { return m_pars[eBoundQOverP] > 0 ? 1. : -1.; }
  double time() const { return m_pars[eBoundTime]; }
  template <unsigned int par> double get() const { return m_pars[par]; }
  /// global position: on a plane, centre + loc0 U + loc1 V
  /// (PlaneSurface.ipp:207-213); on a line, centre + loc1 along the axis +
  /// loc0 along axis x momentum (LineSurface.ipp:184-198)
  Vector3D position() const {
    const Surface &s = *m_surface;
    const auto &R = s.rotation();
    const Vector3D c = s.center();
    if (s.type() == Surface::Plane)
      return Vector3D(c[0] + m_pars[0] * R[0] + m_pars[1] * R[1],
                      c[1] + m_pars[0] * R[3] + m_pars[1] * R[4],
                      c[2] + m_pars[0] * R[6] + m_pars[1] * R[7]);
    const Vector3D axis(R[2], R[5], R[8]);
    Vector3D r = cross(axis, momentum());
    r = (1. / r.norm()) * r;
    return Vector3D(c[0] + m_pars[1] * axis[0] + m_pars[0] * r[0],
                    c[1] + m_pars[1] * axis[1] + m_pars[0] * r[1],
                    c[2] + m_pars[1] * axis[2] + m_pars[0] * r[2]);
  }
  /// momentum from the angles and q/p
  Vector3D momentum() const {
    const double p = std::fabs(1. / m_pars[eBoundQOverP]);
    const double st = std::sin(m_pars[eBoundTheta]);
    return Vector3D(p * st * std::cos(m_pars[eBoundPhi]), p * st * std::sin(m_pars[eBoundPhi]),
                    p * std::cos(m_pars[eBoundTheta]));
  }

private:
  BoundVector m_pars;
  BoundSymMatrix m_cov;
  const Surface *m_surface = nullptr;
};

/// Non-owning span (CudaKernelContainer.hpp:18-71).
template <typename T> struct CudaKernelContainer {
  using value_type = T;
  using pointer = T *;
  using const_pointer = T const *;
  using reference = T &;
  using const_reference = T const &;
  using iterator = pointer;
  using const_iterator = const_pointer;
  CudaKernelContainer() = default;
  CudaKernelContainer(T *array, size_t size) : m_array(array), m_size(size) {}
  pointer array() { return m_array; }
  pointer data() { return m_array; }
  const_pointer array() const { return m_array; }
  const_pointer data() const { return m_array; }
  size_t size() const { return m_size; }
  T &operator[](int i) { return m_array[i]; }
  T const &operator[](int i) const { return m_array[i]; }
  iterator begin() { return m_array; }
  const_iterator begin() const { return m_array; }
  iterator end() { return m_array + m_size; }
  const_iterator end() const { return m_array + m_size; }
  template <typename visitor_t> const_iterator find_if(visitor_t &&visitor) const {
    for (auto i = begin(); i != end(); ++i)
      if (visitor(*i)) return i;
    return end();
  }

private:
  T *m_array = nullptr;
  size_t m_size = 0;
};

enum TrackStateFlag {
  MeasurementFlag = 0, ParameterFlag = 1, OutlierFlag = 2, HoleFlag = 3, MaterialFlag = 4,
  NumTrackStateFlags = 5
};
using TrackStateType = std::bitset<TrackStateFlag::NumTrackStateFlags>;

/// One fitted state (TrackState.hpp:38-169).
template <typename source_link_t, typename parameters_t> class TrackState {
public:
  using SourceLink = source_link_t;
  using Parameters = parameters_t;
  using Jacobian = typename Parameters::CovarianceMatrix;
  TrackState() = default;
  explicit TrackState(SourceLink m) : m_geometryId(m.geometryId()) {
    measurement.uncalibrated = std::move(m);
  }
  const GeometryID &geometryId() const { return m_geometryId; }
  void setGeometryId(GeometryID id) { m_geometryId = id; }
  void setType(const TrackStateFlag &flag, bool status = true) { m_typeFlags.set(flag, status); }
  bool isType(const TrackStateFlag &flag) const { return m_typeFlags.test(flag); }
  TrackStateType type() const { return m_typeFlags; }
  struct {
    Parameters predicted;
    Parameters filtered;
    Parameters smoothed;
    Jacobian jacobian;
    ActsScalar pathLength = 0.;
    ActsScalar chi2 = 0;
  } parameter;
  struct {
    SourceLink uncalibrated;
  } measurement;

private:
  GeometryID m_geometryId;
  TrackStateType m_typeFlags;
};

// ---------------------------------------------------------------------------
// Fields, stepper, propagator, updater, smoother
// ---------------------------------------------------------------------------
namespace test {
/// Test::ConstantBField: 2 T along z (Test/Helper.hpp:17-22).
struct ConstantBField {
  Vector3D getField(const Vector3D & = Vector3D()) const { return Vector3D(0., 0., 2. * kTesla); }
};
/// Test::makeSilicon (Test/Helper.hpp:25-29).
inline Material makeSilicon() {
  return Material::fromMolarDensity(9.370 * units::_cm, 46.52 * units::_cm, 28.0855, 14,
                                    (2.329 / 28.0855) * UnitConstants::mol / UnitConstants::cm3);
}
struct VoidAborter {};
} // namespace test

/// A uniform field of any value.
struct ConstantBField {
  ConstantBField() = default;
  explicit ConstantBField(const Vector3D &value) : m_value(value) {}
  ConstantBField(double bx, double by, double bz) : m_value(bx, by, bz) {}
  Vector3D getField(const Vector3D & = Vector3D()) const { return m_value; }

private:
  Vector3D m_value{0., 0., 2. * kTesla};
};

/// Field map (MagneticField/InterpolatedBFieldMap.hpp, trilinear on an
/// equidistant 3D grid) read from a text file of "x y z bx by bz" lines as
/// Options::readBField reads the driver's map (src/Plugins/BFieldOptions.cpp:
/// 33-61: lengths in mm, field in tesla); the grid is copied to the current
/// device and shared by the copies of this object.  `scale` multiplies
/// every lookup (InterpolatedBFieldMap::Config::scale).
class InterpolatedBFieldMap {
public:
  explicit InterpolatedBFieldMap(const std::string &xyzFile, double lengthUnit = 1.,
                                 double bFieldUnit = kTesla, bool firstOctant = false,
                                 double scale = 1.) {
    float *host = nullptr;
    if (kf_field_map_read_xyz(xyzFile.c_str(), lengthUnit, bFieldUnit, firstOctant ? 1 : 0,
                              &m_field, &host) != 0)
      throw std::runtime_error(std::string("field map: ") + kf_last_error_string());
    const size_t bytes = (size_t)m_field.nx * m_field.ny * m_field.nz * 4 * sizeof(float);
    void *dev = nullptr;
    const bool ok = cudaMalloc(&dev, bytes) == cudaSuccess &&
                    cudaMemcpy(dev, host, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    kf_field_map_free(host);
    if (!ok) {
      if (dev) cudaFree(dev);
      throw std::runtime_error("field map: device copy failed");
    }
    m_grid = std::shared_ptr<void>(dev, [](void *q) { cudaFree(q); });
    m_field.grid = static_cast<const float *>(dev);
    m_field.scale = scale;
  }
  /// the grid as the C ABI takes it (device memory)
  const kf_field_t &field() const { return m_field; }

private:
  kf_field_t m_field{};
  std::shared_ptr<void> m_grid;
};

namespace detail {
inline kf_field_t abiField(const ConstantBField &b) {
  kf_field_t f{};
  f.kind = KF_FIELD_CONSTANT;
  f.scale = 1.;
  const Vector3D v = b.getField();
  for (int a = 0; a < 3; ++a) f.value[a] = v[a];
  return f;
}
inline kf_field_t abiField(const test::ConstantBField &b) {
  kf_field_t f{};
  f.kind = KF_FIELD_CONSTANT;
  f.scale = 1.;
  const Vector3D v = b.getField();
  for (int a = 0; a < 3; ++a) f.value[a] = v[a];
  return f;
}
inline kf_field_t abiField(const InterpolatedBFieldMap &b) { return b.field(); }
} // namespace detail

/// EigenStepper<BField> (EigenStepper.hpp): the field, and the overstep
/// limit the reference fixes at 0.01 mm (EigenStepper.hpp:370).
template <typename bfield_t> class EigenStepper {
public:
  using BField = bfield_t;
  EigenStepper(BField bField = BField(), double overstepLimit = 0.01)
      : m_bField(std::move(bField)), m_overstepLimit(overstepLimit) {}
  const BField &bField() const { return m_bField; }
  double overstepLimit() const { return m_overstepLimit; }

private:
  BField m_bField;
  double m_overstepLimit;
};

struct PropagatorResult {};

/// Propagator<Stepper> (Propagator.hpp): holds the stepper; the fit's
/// propagation options are the reference's defaults (Propagator.hpp:72-95).
template <typename stepper_t> class Propagator {
public:
  using Stepper = stepper_t;
  explicit Propagator(stepper_t stepper) : m_stepper(std::move(stepper)) {}
  const stepper_t &stepper() const { return m_stepper; }

private:
  stepper_t m_stepper;
};

struct GainMatrixUpdater {};
template <typename parameters_t> struct GainMatrixSmoother {};
struct VoidOutlierFinder {};
using VoidKalmanUpdater = GainMatrixUpdater;

template <typename outlier_finder_t = VoidOutlierFinder> struct KalmanFitterOptions {
  using OutlierFinder = outlier_finder_t;
  KalmanFitterOptions() = default;
  KalmanFitterOptions(const GeometryContext &gctx, const MagneticFieldContext &mctx,
                      bool rsmoothing = true,
                      const OutlierFinder &outlierFinder_ = OutlierFinder(),
                      const Surface *rSurface = nullptr, bool mScattering = true, bool eLoss = true)
      : geoContext(gctx), magFieldContext(mctx), outlierFinder(outlierFinder_),
        referenceSurface(rSurface), smoothing(rsmoothing), multipleScattering(mScattering),
        energyLoss(eLoss) {}
  GeometryContext geoContext;
  MagneticFieldContext magFieldContext;
  OutlierFinder outlierFinder;
  const Surface *referenceSurface = nullptr;
  bool smoothing = true;
  bool multipleScattering = true;
  bool energyLoss = true;
};

template <typename source_link_t, typename parameters_t, typename target_surface_t>
struct KalmanFitterResult {
  using TrackStateType = TrackState<source_link_t, parameters_t>;
  CudaKernelContainer<TrackStateType> fittedStates;
  BoundParameters<target_surface_t> fittedParameters;
  size_t measurementStates = 0;
  bool smoothed = false;
  bool finished = false;
  bool result = true;
};

namespace detail {
/// Device staging of one host thread for kf_fit_batch_host, grown on demand
/// and released when the thread ends.
struct ThreadStaging {
  void *ptr = nullptr;
  size_t bytes = 0;
  int device = -1;
  ~ThreadStaging() {
    if (ptr) cudaFree(ptr);
  }
  void *get(size_t need) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) throw std::runtime_error("no CUDA device");
    if (ptr && (bytes < need || dev != device)) {
      cudaFree(ptr);
      ptr = nullptr;
      bytes = 0;
    }
    if (!ptr) {
      if (cudaMalloc(&ptr, need) != cudaSuccess) {
        ptr = nullptr;
        throw std::runtime_error("cudaMalloc of the fit staging buffer failed");
      }
      bytes = need;
      device = dev;
    }
    return ptr;
  }
};
inline ThreadStaging &threadStaging() {
  thread_local ThreadStaging s;
  return s;
}
} // namespace detail

/// KalmanFitter<propagator_t, updater_t, smoother_t, outlier_finder_t>
/// (KalmanFitter.hpp:123-): the fit runs on the GPU; the updater, smoother
/// and outlier-finder types select the reference's algorithms
/// (gain-matrix update and smoother, no outlier rejection).
template <typename propagator_t, typename updater_t = GainMatrixUpdater,
          typename smoother_t = GainMatrixSmoother<BoundParameters<PlaneSurface<InfiniteBounds>>>,
          typename outlier_finder_t = VoidOutlierFinder>
class KalmanFitter {
public:
  explicit KalmanFitter(propagator_t pPropagator) : m_propagator(std::move(pPropagator)) {
    kf_config_default(&m_config);
    m_config.overstep_limit = m_propagator.stepper().overstepLimit();
    m_field = detail::abiField(m_propagator.stepper().bField());
  }

  /// The fit configuration beyond the reference's options (precision,
  /// kernel form, step limits, outlier cut); the reference's values by
  /// default.
  kf_config_t &config() { return m_config; }
  const kf_config_t &config() const { return m_config; }

  /// Fit one track (KalmanFitter.hpp:716-768).  Returns false when the fit
  /// failed or did not produce a measurement state on every surface of the
  /// sequence, as the reference does.
  template <typename source_link_t, typename start_parameters_t,
            typename parameters_t = BoundParameters<PlaneSurface<InfiniteBounds>>,
            typename target_surface_t = PlaneSurface<InfiniteBounds>>
  bool fit(const CudaKernelContainer<source_link_t> &sourcelinks,
           const start_parameters_t &sParameters,
           const KalmanFitterOptions<outlier_finder_t> &kfOptions,
           KalmanFitterResult<source_link_t, parameters_t, target_surface_t> &kfResult,
           const Surface *surfaceSequence = nullptr, size_t surfaceSequenceSize = 0) const {
    bool status = false;
    run(sourcelinks.data(), sourcelinks.size(), &sParameters, &kfOptions, &kfResult, nullptr,
        &status, 1, surfaceSequence, surfaceSequenceSize, cudaStreamPerThread);
    return status;
  }

  /// Fit nTracks tracks in one GPU launch, with the arrays the reference's
  /// GPU kernel takes (fitKernelThreadPerTrack, Run/GPU/Kernels.cu:6-45):
  /// sourcelinks [nTracks][surfaceSequenceSize], start parameters, fit options
  /// and, per track, nSurfaces fitted-state slots (or nullptr), the fitted
  /// parameters and the status.
  template <typename source_link_t, typename start_parameters_t, typename parameters_t,
            typename target_surface_t>
  void fitBatch(const source_link_t *sourcelinks, const start_parameters_t *startParameters,
                const KalmanFitterOptions<outlier_finder_t> *fitOptions,
                TrackState<source_link_t, parameters_t> *fittedStates,
                BoundParameters<target_surface_t> *fitPars, bool *fitStatus, size_t nTracks,
                const Surface *surfaceSequence, size_t surfaceSequenceSize,
                cudaStream_t stream = nullptr) const {
    using Result = KalmanFitterResult<source_link_t, parameters_t, target_surface_t>;
    std::vector<Result> results(nTracks);
    for (size_t i = 0; i < nTracks && fittedStates; ++i)
      results[i].fittedStates = CudaKernelContainer<TrackState<source_link_t, parameters_t>>(
          fittedStates + i * surfaceSequenceSize, surfaceSequenceSize);
    run(sourcelinks, surfaceSequenceSize, startParameters, fitOptions, results.data(), nullptr,
        fitStatus, nTracks, surfaceSequence, surfaceSequenceSize, stream);
    for (size_t i = 0; i < nTracks; ++i) fitPars[i] = results[i].fittedParameters;
  }

private:
  template <typename source_link_t, typename start_parameters_t, typename parameters_t,
            typename target_surface_t>
  void run(const source_link_t *sourcelinks, size_t linksPerTrack,
           const start_parameters_t *starts, const KalmanFitterOptions<outlier_finder_t> *opts,
           KalmanFitterResult<source_link_t, parameters_t, target_surface_t> *results,
           const void *, bool *status, size_t nTracks, const Surface *surfaces, size_t nSurfaces,
           cudaStream_t stream) const {
    if (!surfaces || nSurfaces == 0 || nSurfaces > KF_MAX_PLANES)
      throw std::invalid_argument("surface sequence must hold 1..64 surfaces");
    const int64_t n = static_cast<int64_t>(nTracks);
    const int S = static_cast<int>(nSurfaces);
    if (n == 0) return;
    std::vector<double> center(3 * S), rot(9 * S), mat(6 * S);
    bool anyMaterial = false;
    for (int k = 0; k < S; ++k) {
      const MaterialSlab &sl = surfaces[k].surfaceMaterial().materialSlab();
      const Material &m = sl.material();
      const double row[6] = {sl.thickness(), m.X0(), m.L0(), m.Ar(), m.Z(), m.molarDensity()};
      for (int e = 0; e < 6; ++e) mat[6 * k + e] = row[e];
      anyMaterial = anyMaterial || (sl.thickness() > 0. && m.Ar() > 0.);
      for (int r = 0; r < 3; ++r) center[3 * k + r] = surfaces[k].center()[r];
      for (int e = 0; e < 9; ++e) rot[9 * k + e] = surfaces[k].rotation()[e];
    }
    // per surface, the index of each track's source link on it (-1: none):
    // the reference's actor finds a surface's link by geometry id
    // (SurfaceFinder, KalmanFitter.hpp:31-38)
    std::vector<int32_t> link((size_t)n * S, -1);
    std::vector<double> meas((size_t)S * 5 * n, 0.), start(6 * n), scov(21 * n), per(3 * n);
    std::vector<uint64_t> mask(n, 0);
    for (int64_t i = 0; i < n; ++i) {
      const source_link_t *sl = sourcelinks + (size_t)i * linksPerTrack;
      for (int k = 0; k < S; ++k) {
        meas[((size_t)k * 5 + 2) * n + i] = 1.;
        meas[((size_t)k * 5 + 4) * n + i] = 1.;
        const GeometryID gid = surfaces[k].geoID();
        for (size_t j = 0; j < linksPerTrack; ++j) {
          if (!(sl[j].geometryId() == gid)) continue;
          link[(size_t)i * S + k] = (int32_t)j;
          mask[i] |= (1ull << k);
          const auto &v = sl[j].localPosition();
          const auto &c = sl[j].covariance();
          const double m[5] = {v[0], v[1], c(0, 0), c(0, 1), c(1, 1)};
          for (int e = 0; e < 5; ++e) meas[((size_t)k * 5 + e) * n + i] = m[e];
          break;
        }
      }
      const auto &p = starts[i].parameters();
      const auto &C = *starts[i].covariance();
      for (int e = 0; e < 6; ++e) start[e * n + i] = p[e];
      int e = 0;
      for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b) scov[(e++) * n + i] = C(a, b);
      // the perigee line: the options' reference surface (the reference
      // driver sets it to the start parameters' line), else the start
      // parameters' own surface
      const Surface *target = opts[i].referenceSurface ? opts[i].referenceSurface
                                                       : &starts[i].referenceSurface();
      for (int r = 0; r < 3; ++r) per[r * n + i] = target->center()[r];
    }
    kf_inputs_t in{};
    in.n_tracks = n;
    in.stride = n;
    in.n_surfaces = S;
    in.meas = meas.data();
    in.hit_mask = mask.data();
    in.n_planes = nullptr;
    in.start_params = start.data();
    in.start_cov = scov.data();
    in.perigee = per.data();
    std::vector<double> oPar(6 * n), oCov(21 * n), oChi(n), oSm((size_t)S * 27 * n);
    std::vector<int32_t> oSt(n), oNm(n);
    kf_outputs_t out{};
    out.params = oPar.data();
    out.cov = oCov.data();
    out.chi2 = oChi.data();
    out.status = oSt.data();
    out.n_meas = oNm.data();
    out.smoothed = oSm.data();
    kf_config_t cfg = m_config;
    // smoothing and material switches are per call in the reference; one
    // launch takes the first track's
    cfg.smoothing = opts[0].smoothing ? 1 : 0;
    cfg.material_effects = anyMaterial ? ((opts[0].multipleScattering ? 1 : 0) |
                                          (opts[0].energyLoss ? 2 : 0))
                                       : 0;
    const kf_geometry_t geo{S, 0, center.data(), rot.data(), anyMaterial ? mat.data() : nullptr};
    const size_t need = kf_host_staging_size(&cfg, n, S, 1);
    void *staging = detail::threadStaging().get(need);
    const int32_t rc =
        kf_fit_batch_host(&in, &out, &cfg, &geo, &m_field, staging, need, stream);
    if (rc != 0)
      throw std::runtime_error(std::string("kf_fit_batch_host: ") + kf_last_error_string());
    for (int64_t i = 0; i < n; ++i) {
      auto &r = results[i];
      r.measurementStates = (size_t)oNm[i];
      r.result = (oSt[i] == KF_TRACK_OK);
      r.smoothed = r.result && cfg.smoothing && r.measurementStates > 0;
      r.finished = r.result;
      BoundVector p;
      BoundSymMatrix C;
      for (int e = 0; e < 6; ++e) p[e] = oPar[e * n + i];
      int e = 0;
      for (int a = 0; a < 6; ++a)
        for (int b = a; b < 6; ++b) C(a, b) = C(b, a) = oCov[(e++) * n + i];
      const Surface *target = opts[i].referenceSurface ? opts[i].referenceSurface
                                                       : &starts[i].referenceSurface();
      r.fittedParameters = BoundParameters<target_surface_t>(GeometryContext(), C, p, target);
      // measurement state k lies on the k-th surface with a source link
      uint64_t bits = mask[i];
      const size_t slots = r.fittedStates.size();
      for (size_t k = 0; k < r.measurementStates && bits; ++k) {
        const int plane = __builtin_ctzll(bits);
        bits &= bits - 1;
        if (k >= slots) continue;
        auto &ts = r.fittedStates[(int)k];
        ts = typename std::remove_reference_t<decltype(ts)>(
            sourcelinks[(size_t)i * linksPerTrack + link[(size_t)i * S + plane]]);
        ts.setType(MeasurementFlag);
        BoundVector sp;
        BoundSymMatrix sc;
        for (int q = 0; q < 6; ++q) sp[q] = oSm[((size_t)k * 27 + q) * n + i];
        int f = 0;
        for (int a = 0; a < 6; ++a)
          for (int b = a; b < 6; ++b) sc(a, b) = sc(b, a) = oSm[((size_t)k * 27 + 6 + (f++)) * n + i];
        ts.parameter.smoothed = parameters_t(GeometryContext(), sc, sp, &surfaces[plane]);
      }
      // KalmanFitter.hpp:760-767
      status[i] = r.result && r.measurementStates == nSurfaces;
    }
  }

  propagator_t m_propagator;
  kf_config_t m_config{};
  kf_field_t m_field{};
};

/// writeParamsCsv (Run/Common/Writer.hpp:80-110): the fitted parameters of
/// the tracks whose status is true, one CSV row each (kf_write_params_csv).
template <typename parameters_t>
void writeParamsCsv(const parameters_t *params, const bool *status, unsigned int nTracks,
                    std::string fileName) {
  if (fileName.empty()) fileName = "params-fitted.obj"; // the reference's default name
  std::vector<double> p((size_t)6 * nTracks);
  std::vector<int32_t> st(nTracks);
  for (unsigned int i = 0; i < nTracks; ++i) {
    for (int e = 0; e < 6; ++e) p[(size_t)e * nTracks + i] = params[i].parameters()[e];
    st[i] = status[i] ? KF_TRACK_OK : KF_TRACK_NOT_FITTED;
  }
  if (kf_write_params_csv(fileName.c_str(), p.data(), st.data(), nTracks, nTracks) != 0)
    throw std::ios_base::failure(kf_last_error_string());
}

/// writeStatesObj (Run/Common/Writer.hpp:42-78) with parameters = "smoothed":
/// one obj polyline per successful fit through its smoothed states
/// (kf_write_states_obj); `states` is the reference's [nTracks][nSurfaces]
/// fitted-state array, every slot of a successful track filled (the fit's
/// status requires a state on every surface).
template <typename track_state_t>
void writeStatesObj(const track_state_t *states, const bool *status, unsigned int nTracks,
                    unsigned int nSurfaces, std::string fileName,
                    const std::string &parameters = "smoothed") {
  if (fileName.empty()) fileName = "tracks-fitted.obj";
  if (parameters != "smoothed")
    throw std::invalid_argument("writeStatesObj: the fit returns smoothed states only");
  if (nSurfaces == 0 || nSurfaces > KF_MAX_PLANES)
    throw std::invalid_argument("surface sequence must hold 1..64 surfaces");
  const size_t n = nTracks, S = nSurfaces;
  // the surface sequence, from the first successful track's states
  std::vector<const Surface *> planes;
  for (size_t i = 0; i < n && planes.empty(); ++i)
    if (status[i])
      for (size_t k = 0; k < S; ++k)
        planes.push_back(&states[i * S + k].parameter.smoothed.referenceSurface());
  std::vector<double> sm(S * 27 * n, 0.), center(3 * S, 0.), rot(9 * S, 0.);
  std::vector<int32_t> nm(n, 0), st(n);
  std::vector<uint64_t> mask(n, 0);
  for (size_t i = 0; i < n; ++i) {
    st[i] = status[i] ? KF_TRACK_OK : KF_TRACK_NOT_FITTED;
    if (!status[i]) continue;
    for (size_t k = 0; k < S; ++k) {
      const auto &ts = states[i * S + k];
      if (&ts.parameter.smoothed.referenceSurface() != planes[k])
        throw std::invalid_argument("writeStatesObj: tracks on different surface sequences");
      for (int q = 0; q < 6; ++q) sm[(k * 27 + q) * n + i] = ts.parameter.smoothed.parameters()[q];
    }
    nm[i] = (int32_t)S;
    mask[i] = S == 64 ? ~0ull : ((1ull << S) - 1);
  }
  for (size_t k = 0; k < planes.size(); ++k) {
    for (int r = 0; r < 3; ++r) center[3 * k + r] = planes[k]->center()[r];
    for (int e = 0; e < 9; ++e) rot[9 * k + e] = planes[k]->rotation()[e];
  }
  const kf_geometry_t geo{(int32_t)S, 0, center.data(), rot.data(), nullptr};
  if (kf_write_states_obj(fileName.c_str(), sm.data(), nm.data(), mask.data(), st.data(),
                          (int64_t)n, (int64_t)n, &geo) != 0)
    throw std::ios_base::failure(kf_last_error_string());
}

} // namespace gb300kf

#ifdef GB300KF_ACTS_NAMESPACE
namespace Acts = gb300kf;
namespace Test = gb300kf::test;
#endif

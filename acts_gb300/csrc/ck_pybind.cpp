// ck_pybind.cpp — pybind11 module acts_gb300._acts_gb300_ext, the binding
// the reference's Python layer has for the fit,
//   Python/Examples/src/TrackFitting.cpp:50-67 (makeKalmanFitterFunction
//   with its keyword arguments, returning a TrackFitterFunction),
// over the C ABI of include/cudakalman.h. The tracking geometry is the
// surface table (a buffer of ck_surface, e.g. a ctypes array), the magnetic
// field a buffer holding one ck_field; the function object fits a batch
// given as numpy arrays in the ck_batch_in layout and returns the results
// as numpy arrays in the ck_batch_out layout (flat, track index innermost).
// Built when pybind11 is importable at build time; acts_gb300.fitter and
// acts_gb300.track_fitting give the same through ctypes.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "cudakalman.h"

namespace py = pybind11;
using namespace py::literals;

namespace {

template <typename T>
using Arr = py::array_t<T, py::array::c_style | py::array::forcecast>;

class TrackFitterFunction {
 public:
  TrackFitterFunction(std::vector<ck_surface> surfaces, ck_field field, ck_options options)
      : m_surfaces(std::move(surfaces)), m_opt(options) {
    ck_config c{};
    c.device = 0;
    c.n_surfaces = static_cast<int32_t>(m_surfaces.size());
    c.surfaces = m_surfaces.data();
    c.field = field;
    c.use_graph = 0;
    if (ck_create(&c, &m_h) != CK_OK)
      throw std::runtime_error(std::string("ck_create: ") + ck_last_error());
  }
  ~TrackFitterFunction() {
    if (m_h) ck_destroy(m_h);
  }
  TrackFitterFunction(const TrackFitterFunction&) = delete;
  TrackFitterFunction& operator=(const TrackFitterFunction&) = delete;

  // Fits the batch; arrays as in ck_batch_in (CSR offsets of n + 1 entries),
  // results flat in the ck_batch_out layout (track index innermost) for the
  // CK_OUT_* components asked for; referenceSurface >= 0 (a line surface of
  // the table) adds the parameters there (track_params, track_cov).
  py::dict fit(Arr<int32_t> seqOffsets, Arr<int32_t> seqSurfaces, Arr<int32_t> measOffsets,
               Arr<int32_t> measSurfaces, Arr<double> measValues, Arr<double> measCov,
               Arr<double> startParams, Arr<double> startCov, Arr<double> startFrames,
               Arr<float> particle, Arr<int32_t> particlePdg, py::object measSubspace,
               int maxStates, uint32_t components, int referenceSurface) const {
    const py::ssize_t n = seqOffsets.size() - 1;
    if (n < 0 || measOffsets.size() != n + 1 || startParams.size() != 6 * n ||
        startCov.size() != 36 * n || startFrames.size() != 12 * n || particle.size() != 2 * n ||
        particlePdg.size() != n || maxStates < 1)
      throw std::invalid_argument("inconsistent batch array sizes");
    ck_batch_in in{};
    in.n_tracks = static_cast<int32_t>(n);
    in.memory = CK_MEM_HOST;
    in.seq_offsets = seqOffsets.data();
    in.seq_surfaces = seqSurfaces.data();
    in.meas_offsets = measOffsets.data();
    in.meas_surfaces = measSurfaces.data();
    in.meas_values = measValues.data();
    in.meas_cov = measCov.data();
    in.start_params = startParams.data();
    in.start_cov = startCov.data();
    in.start_frames = startFrames.data();
    in.particle = particle.data();
    in.particle_pdg = particlePdg.data();
    Arr<int32_t> sub;
    if (!measSubspace.is_none()) {
      sub = measSubspace.cast<Arr<int32_t>>();
      in.meas_subspace = sub.data();
    }
    ck_options opt = m_opt;
    opt.reference_surface = referenceSurface;
    if (referenceSurface >= 0) components |= CK_OUT_REFERENCE;
    else components &= ~static_cast<uint32_t>(CK_OUT_REFERENCE);
    const py::ssize_t S = n * maxStates;
    const py::ssize_t cc = (components & CK_OUT_PACKED_COV) ? 21 : 36;
    py::dict res;
    auto add = [&](const char* name, auto arr) {
      res[name] = arr;
      return arr.mutable_data();
    };
    ck_batch_out out{};
    out.max_states = maxStates;
    out.components = components;
    out.memory = CK_MEM_HOST;
    out.status = add("status", Arr<int32_t>(n));
    out.n_states = add("n_states", Arr<int32_t>(n));
    out.n_measurements = add("n_measurements", Arr<int32_t>(n));
    out.n_holes = add("n_holes", Arr<int32_t>(n));
    out.n_outliers = add("n_outliers", Arr<int32_t>(n));
    out.ndf = add("ndf", Arr<int32_t>(n));
    out.chi2_sum = add("chi2_sum", Arr<double>(n));
    out.state_surface = add("state_surface", Arr<int32_t>(S));
    out.state_flags = add("state_flags", Arr<uint32_t>(S));
    out.state_path_length = add("state_path_length", Arr<double>(S));
    out.state_chi2 = add("state_chi2", Arr<double>(S));
    if (components & CK_OUT_PREDICTED) {
      out.predicted = add("predicted", Arr<double>(S * 6));
      out.predicted_cov = add("predicted_cov", Arr<double>(S * cc));
    }
    if (components & CK_OUT_FILTERED) {
      out.filtered = add("filtered", Arr<double>(S * 6));
      out.filtered_cov = add("filtered_cov", Arr<double>(S * cc));
    }
    if (components & CK_OUT_SMOOTHED) {
      out.smoothed = add("smoothed", Arr<double>(S * 6));
      out.smoothed_cov = add("smoothed_cov", Arr<double>(S * cc));
    }
    if (components & CK_OUT_JACOBIAN) out.jacobian = add("jacobian", Arr<double>(S * 36));
    if (components & CK_OUT_REFERENCE) {
      out.track_params = add("track_params", Arr<double>(n * 6));
      out.track_cov = add("track_cov", Arr<double>(n * 36));
    }
    ck_status s;
    {
      py::gil_scoped_release release;
      s = ck_fit_batch(m_h, &opt, &in, &out, nullptr);
      if (s == CK_OK) s = ck_sync(m_h);
    }
    if (s != CK_OK) throw std::runtime_error(std::string("ck_fit_batch: ") + ck_last_error());
    res["max_states"] = maxStates;
    res["components"] = components;
    return res;
  }

 private:
  std::vector<ck_surface> m_surfaces;
  ck_options m_opt{};
  ck_handle* m_h = nullptr;
};

std::vector<ck_surface> surfacesFrom(const py::buffer& b) {
  const py::buffer_info info = b.request();
  const size_t bytes = static_cast<size_t>(info.size) * static_cast<size_t>(info.itemsize);
  if (bytes % sizeof(ck_surface) != 0)
    throw std::invalid_argument("trackingGeometry: not a buffer of ck_surface");
  std::vector<ck_surface> v(bytes / sizeof(ck_surface));
  std::memcpy(v.data(), info.ptr, bytes);
  return v;
}

ck_field fieldFrom(const py::buffer& b) {
  const py::buffer_info info = b.request();
  const size_t bytes = static_cast<size_t>(info.size) * static_cast<size_t>(info.itemsize);
  if (bytes != sizeof(ck_field)) throw std::invalid_argument("magneticField: not a ck_field");
  ck_field f;
  std::memcpy(&f, info.ptr, sizeof(f));
  return f;
}

}  // namespace

PYBIND11_MODULE(_acts_gb300_ext, m) {
  m.doc() = "pybind11 binding of the batched Kalman fitter (makeKalmanFitterFunction)";
  py::class_<TrackFitterFunction>(m, "TrackFitterFunction")
      .def("__call__", &TrackFitterFunction::fit, "seq_offsets"_a, "seq_surfaces"_a,
           "meas_offsets"_a, "meas_surfaces"_a, "meas_values"_a, "meas_cov"_a,
           "start_params"_a, "start_cov"_a, "start_frames"_a, "particle"_a, "particle_pdg"_a,
           "meas_subspace"_a = py::none(), "max_states"_a = 24,
           "components"_a = static_cast<uint32_t>(CK_OUT_SMOOTHED | CK_OUT_PACKED_COV),
           "reference_surface"_a = -1);
  m.def(
      "makeKalmanFitterFunction",
      [](py::buffer trackingGeometry, py::buffer magneticField, bool multipleScattering,
         bool energyLoss, double reverseFilteringMomThreshold,
         double reverseFilteringCovarianceScaling, bool freeToBoundCorrection, double chi2Cut,
         bool useJosephFormulation, int level, int precision) {
        static_cast<void>(level);  // (the fitter has no logger)
        ck_options o;
        ck_options_default(&o);
        o.multiple_scattering = multipleScattering ? 1 : 0;
        o.energy_loss = energyLoss ? 1 : 0;
        o.reverse_filtering_mom_threshold = reverseFilteringMomThreshold;
        o.reverse_filtering_cov_scaling = reverseFilteringCovarianceScaling;
        o.free_to_bound_correction = freeToBoundCorrection ? 1 : 0;
        o.outlier_chi2_cut = chi2Cut;
        o.use_joseph = useJosephFormulation ? 1 : 0;
        o.smoother = CK_SMOOTHER_MBF;  // (the function object's smoother)
        o.reference_strategy = CK_EXTRAPOLATE_FIRST;
        o.precision = precision;
        return new TrackFitterFunction(surfacesFrom(trackingGeometry), fieldFrom(magneticField), o);
      },
      "trackingGeometry"_a, "magneticField"_a, "multipleScattering"_a = true,
      "energyLoss"_a = true, "reverseFilteringMomThreshold"_a = 0.0,
      "reverseFilteringCovarianceScaling"_a = 100.0, "freeToBoundCorrection"_a = false,
      "chi2Cut"_a = std::numeric_limits<double>::infinity(), "useJosephFormulation"_a = false,
      "level"_a = 0, "precision"_a = static_cast<int>(CK_PRECISION_FP64),
      py::return_value_policy::take_ownership);
}

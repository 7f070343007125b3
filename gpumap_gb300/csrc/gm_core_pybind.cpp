// Python module gpumap_gb300._core: the same classes, attributes and keyword
// names as the reference's pybind11 module (cpp/bindings/binding.cu:45-115),
// implemented on top of the C ABI in include/gpumap_gb300.h only.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <cctype>
#include <stdexcept>
#include <string>

#include "../../include/gpumap_gb300.h"

namespace py = pybind11;

namespace {

[[noreturn]] void raise_status(int rc) {
  const std::string msg = gm_last_error();
  switch (rc) {
    case GM_ERR_INVALID: throw py::value_error(msg);
    case GM_ERR_OOM: throw std::bad_alloc();
    default: throw std::runtime_error(msg.empty() ? "gpumap_gb300 error " + std::to_string(rc) : msg);
  }
}

inline void check(int rc) {
  if (rc != GM_OK) raise_status(rc);
}

struct Params {
  gm_params p;
  Params() { gm_params_default(&p); }
};

struct Result {
  gm_result r{};
};

std::string metric_name(int m) { return m == GM_METRIC_COSINE ? "cosine" : "euclidean"; }

// Accepts "euclidean"/"cosine" (any case), an int or an IntEnum
// (reference binding.cu:28-41).
int metric_from(const py::object &v) {
  if (py::isinstance<py::str>(v)) {
    std::string s = v.cast<std::string>();
    for (char &c : s) c = (char)std::tolower((unsigned char)c);
    if (s == "euclidean") return GM_METRIC_EUCLIDEAN;
    if (s == "cosine") return GM_METRIC_COSINE;
    throw py::value_error("Unknown metric '" + s + "' -- expected 'euclidean' or 'cosine'");
  }
  return v.cast<int>();
}

// ---- result views ---------------------------------------------------------
// The reference returns a bare object carrying __cuda_array_interface__ v3
// (cpp/bindings/utils/cai_wrapper.cuh:39-62: read-only, full capacity, no
// stream, borrowing the engine's memory).  DeviceView keeps those fields and
// adds the producing stream to the interface, plus the DLPack protocol
// (__dlpack__ / __dlpack_device__) whose consumer stream is made to wait for
// the session's queued work on the device.  A view holds a reference to its
// model, so the memory stays valid while the view lives.

// DLPack ABI (the data-interchange format's C structs, version 0.8 layout).
struct DLDevice {
  int32_t device_type;  // 2 = CUDA
  int32_t device_id;
};
struct DLDataType {
  uint8_t code;  // 1 = unsigned int, 2 = float
  uint8_t bits;
  uint16_t lanes;
};
struct DLTensor {
  void *data;
  DLDevice device;
  int32_t ndim;
  DLDataType dtype;
  int64_t *shape;
  int64_t *strides;  // in elements
  uint64_t byte_offset;
};
struct DLManagedTensor {
  DLTensor dl_tensor;
  void *manager_ctx;
  void (*deleter)(DLManagedTensor *self);
};

struct ViewCtx {
  int64_t shape[2];
  int64_t strides[2];
  PyObject *owner;  // the model, kept alive while a consumer holds the tensor
};

void dl_delete(DLManagedTensor *t) {
  auto *ctx = static_cast<ViewCtx *>(t->manager_ctx);
  {
    py::gil_scoped_acquire gil;
    Py_XDECREF(ctx->owner);
  }
  delete ctx;
  delete t;
}

void dl_capsule_destructor(PyObject *cap) {
  // a capsule nobody consumed still owns its tensor
  if (PyCapsule_IsValid(cap, "dltensor")) {
    auto *t = static_cast<DLManagedTensor *>(PyCapsule_GetPointer(cap, "dltensor"));
    if (t) t->deleter(t);
  }
}

struct DeviceView {
  gm_view v{};
  gm_session *s = nullptr;
  int device = 0;
  py::object owner;

  py::dict cai() const {
    py::dict d;
    d["version"] = 3;
    d["shape"] = py::make_tuple(v.rows, v.cols);
    d["typestr"] = v.dtype == GM_DTYPE_U32 ? "<u4" : "<f4";
    d["strides"] = py::make_tuple(v.row_stride_bytes, (uint64_t)4);
    d["data"] = py::make_tuple(reinterpret_cast<uintptr_t>(v.ptr), true);
    void *st = nullptr;
    check(gm_get_stream(s, &st));
    // the values are complete on this stream; 0 would mean "no stream"
    // (CUDA Array Interface v3), so the default stream is given as 1
    d["stream"] = st ? reinterpret_cast<uintptr_t>(st) : (uintptr_t)1;
    return d;
  }

  py::object dlpack(const py::object &stream) const {
    if (!stream.is_none()) {
      const auto h = stream.cast<intptr_t>();
      if (h != -1) check(gm_stream_wait(s, reinterpret_cast<void *>(h)));
    }
    auto *ctx = new ViewCtx;
    ctx->shape[0] = (int64_t)v.rows;
    ctx->shape[1] = (int64_t)v.cols;
    ctx->strides[0] = (int64_t)(v.row_stride_bytes / 4);
    ctx->strides[1] = 1;
    ctx->owner = owner.ptr();
    Py_XINCREF(ctx->owner);
    auto *t = new DLManagedTensor;
    t->dl_tensor.data = v.ptr;
    t->dl_tensor.device = DLDevice{2, device};
    t->dl_tensor.ndim = 2;
    t->dl_tensor.dtype = DLDataType{(uint8_t)(v.dtype == GM_DTYPE_U32 ? 1 : 2), 32, 1};
    t->dl_tensor.shape = ctx->shape;
    t->dl_tensor.strides = ctx->strides;
    t->dl_tensor.byte_offset = 0;
    t->manager_ctx = ctx;
    t->deleter = dl_delete;
    PyObject *cap = PyCapsule_New(t, "dltensor", dl_capsule_destructor);
    if (!cap) {
      dl_delete(t);
      throw py::error_already_set();
    }
    return py::reinterpret_steal<py::object>(cap);
  }
};

class Model {
 public:
  explicit Model(const Params &cfg) : p_(cfg.p) { check(gm_create(&p_, &s_)); }
  ~Model() { gm_destroy(s_); }
  Model(const Model &) = delete;
  Model &operator=(const Model &) = delete;

  void initialize(uint64_t n_instances, uint64_t n_features) {
    check(gm_initialize(s_, n_instances, n_features));
  }

  // Reference checks (numpy_utils.cuh:16-48, gpumap_wrapper.cuh:29-40).
  void append_data(py::array x) {
    py::buffer_info info = x.request();
    if (info.ndim != 2) throw std::runtime_error("Expected 2D numpy array.");
    if (info.format != py::format_descriptor<float>::format())
      throw std::runtime_error("Only float32 numpy arrays are supported.");
    if (info.strides[1] != (py::ssize_t)sizeof(float) ||
        info.strides[0] != (py::ssize_t)sizeof(float) * info.shape[1])
      throw std::runtime_error("Require C-contiguous numpy array (row-major float32).");
    if ((uint64_t)info.shape[1] != p_.n_features)
      throw std::runtime_error("n_features mismatch with numpy array second dimension.");
    if (info.shape[0] <= 0) return;
    check(gm_append(s_, static_cast<const float *>(info.ptr), (uint64_t)info.shape[0],
                    (uint64_t)info.shape[1]));
  }

  Result run(uint32_t ni, uint32_t nu, uint32_t ne) {
    Result r;
    int rc;
    {
      py::gil_scoped_release nogil;
      rc = gm_run(s_, ni, nu, ne, &r.r);
    }
    check(rc);
    return r;
  }

  void close() { check(gm_close(s_)); }

  // which: 0 embedding, 1 neighbor indices, 2 neighbor distances
  DeviceView view(int which, const py::object &self) const {
    DeviceView dv;
    const int rc = which == 0   ? gm_get_embedding(s_, &dv.v)
                   : which == 1 ? gm_get_neighbor_indices(s_, &dv.v)
                                : gm_get_neighbor_dists(s_, &dv.v);
    check(rc);
    int32_t dev = 0;
    check(gm_get_device(s_, &dev));
    dv.s = s_;
    dv.device = dev;
    dv.owner = self;
    return dv;
  }
  uintptr_t session_ptr() const { return reinterpret_cast<uintptr_t>(s_); }

 private:
  gm_params p_;
  gm_session *s_ = nullptr;
};

}  // namespace

PYBIND11_MODULE(_core, m) {
  m.doc() = "gpumap_gb300 GB300 progressive UMAP engine (C ABI binding)";

#define GM_RW(name, field) \
  .def_property(name, [](const Params &p) { return p.p.field; }, [](Params &p, decltype(gm_params::field) v) { p.p.field = v; })

  py::class_<Params>(m, "GPUMAPParams")
      .def(py::init<>())
      GM_RW("n_neighbors", n_neighbors)
      GM_RW("n_components", n_components)
      GM_RW("min_dist", min_dist)
      GM_RW("negative_sample_rate", negative_sample_rate)
      GM_RW("max_epoch", max_epoch)
      GM_RW("a", a)
      GM_RW("b", b)
      GM_RW("alpha", alpha)
      .def_property("verbose", [](const Params &p) { return p.p.verbose != 0; },
                    [](Params &p, bool v) { p.p.verbose = v ? 1 : 0; })
      .def_property("metric", [](const Params &p) { return metric_name(p.p.metric); },
                    [](Params &p, const py::object &v) { p.p.metric = metric_from(v); })
      GM_RW("n_instances", n_instances)
      GM_RW("n_features", n_features)
      GM_RW("precision", precision)
      GM_RW("overlap", overlap)
      GM_RW("device", device);
#undef GM_RW

#define GM_RO(name, field) .def_property_readonly(name, [](const Result &r) { return r.r.field; })
  py::class_<Result>(m, "GPUMAPResult")
      GM_RO("n_insertion_ops", n_insertion_ops)
      GM_RO("n_update_ops", n_update_ops)
      GM_RO("n_embedding_ops", n_embedding_ops)
      GM_RO("insertion_time", insertion_time)
      GM_RO("update_time", update_time)
      GM_RO("embedding_time", embedding_time)
      .def_property_readonly("insertion_completed", [](const Result &r) { return r.r.insertion_completed != 0; })
      .def_property_readonly("update_completed", [](const Result &r) { return r.r.update_completed != 0; })
      .def_property_readonly("embedding_completed", [](const Result &r) { return r.r.embedding_completed != 0; })
      GM_RO("n_inserted_instances", n_inserted_instances)
      GM_RO("n_update_changed_edges", n_update_changed_edges)
      GM_RO("embedding_pending_edges", embedding_pending_edges)
      GM_RO("insertion_queue_size", insertion_queue_size)
      GM_RO("update_queue_size", update_queue_size)
      GM_RO("embedding_queue_size", embedding_queue_size);
#undef GM_RO

  py::class_<DeviceView>(m, "DeviceView")
      .def_property_readonly("__cuda_array_interface__", &DeviceView::cai)
      .def("__dlpack__", &DeviceView::dlpack, py::arg("stream") = py::none())
      .def("__dlpack_device__", [](const DeviceView &v) { return py::make_tuple(2, v.device); })
      .def_property_readonly("shape", [](const DeviceView &v) { return py::make_tuple(v.v.rows, v.v.cols); });

  py::class_<Model>(m, "GPUMAP")
      .def(py::init<const Params &>(), py::arg("config"))
      .def("initialize", &Model::initialize, py::arg("n_instances"), py::arg("n_features"))
      .def("append_data", &Model::append_data, py::arg("x"))
      .def("run", &Model::run, py::arg("n_jobs_insertion"), py::arg("n_jobs_update"),
           py::arg("n_jobs_embedding"))
      .def("close", &Model::close)
      .def("get_embedding", [](py::object self) { return self.cast<const Model &>().view(0, self); })
      .def("get_neighbor_indices", [](py::object self) { return self.cast<const Model &>().view(1, self); })
      .def("get_neighbor_dists", [](py::object self) { return self.cast<const Model &>().view(2, self); })
      .def("_session_ptr", &Model::session_ptr);
}

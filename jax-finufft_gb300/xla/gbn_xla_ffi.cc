// gbn_xla_ffi.cc -- XLA typed-FFI handlers for jax-finufft's 18 GPU targets,
// implemented on libgbnufft's C ABI.
//
// Replaces lib/jax_finufft_gpu.cc:28-422 + lib/kernels.cc.cu of the reference: the
// same target names (nufft{1,2,3}d{1,2,3}{f,}), the same attributes in the
// same order (eps as f32 for the single-precision targets and f64 otherwise,
// then iflag, n_tot, n_transf, n_j, n_k_1, n_k_2, n_k_3, modeord as int64,
// upsampfac as f64, gpu_method, gpu_sort, gpu_kerevalmeth, gpu_maxbatchsize,
// debug as int64), the same buffers (source, the d point arrays in the
// backend order src/jax_finufft/lowering.py produces, for type 3 the d
// target arrays, then the output) and the same Python module interface
// (module jax_finufft_gpu, function registrations() -> {name: capsule}), so
// lowering.py registers these handlers unchanged.
//
// Differences from the reference's handlers: no host synchronisation (work
// stays ordered on XLA's stream), plans are cached across calls by the
// library, and a tolerance warning (status 1) is not an error.
//
// Built only where the XLA FFI headers are available (jaxlib), e.g.
//   c++ -O2 -std=c++17 -shared -fPIC -I<jax.ffi.include_dir()> -I<pybind11 include>
//       -I<python include> -I include -I<cuda include> gbn_xla_ffi.cc
//       -L<dir of libgbnufft.so> -lgbnufft -o jax_finufft_gpu<ext suffix>
#include <cuda_runtime.h>
#include <pybind11/pybind11.h>

#include <cstdint>
#include <string>

#include "gbnufft.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;
namespace py = pybind11;

namespace {

// The attributes every target carries after eps (lib/jax_finufft_gpu.cc:28-60,
// filled by src/jax_finufft/lowering.py:28-178).
struct Attrs {
  int64_t iflag, n_tot, n_transf, n_j, n_k[3], modeord;
  double upsampfac;
  int64_t gpu_method, gpu_sort, gpu_kerevalmeth, gpu_maxbatchsize, debug;
};

ffi::Error run(int type, int dim, bool single, cudaStream_t stream, double eps, const Attrs& a,
               const void* source, const void* const* pts, const void* const* tgts, void* out) {
  gbn_opts o;
  gbn_default_opts(&o);
  o.modeord = (int)a.modeord;
  o.upsampfac = a.upsampfac;
  o.gpu_method = (int)a.gpu_method;
  o.gpu_sort = (int)a.gpu_sort;
  o.gpu_kerevalmeth = (int)a.gpu_kerevalmeth;
  o.gpu_maxbatchsize = (int)a.gpu_maxbatchsize;
  o.debug = (int)a.debug;
  const int rc = gbn_run(type, dim, single ? 1 : 0, (void*)stream, eps, (int)a.iflag, a.n_tot,
                         a.n_transf, a.n_j, a.n_k, &o, source, pts, tgts, out);
  if (rc >= 2) return ffi::Error::Internal(std::string("jax_finufft_gb300: ") + gbn_last_error());
  return ffi::Error::Success();
}

template <int DIM, int TYPE, typename EPS>
struct Target {
  static ffi::Error call(cudaStream_t stream, EPS eps, int64_t iflag, int64_t n_tot,
                         int64_t n_transf, int64_t n_j, int64_t n_k_1, int64_t n_k_2,
                         int64_t n_k_3, int64_t modeord, double upsampfac, int64_t gpu_method,
                         int64_t gpu_sort, int64_t gpu_kerevalmeth, int64_t gpu_maxbatchsize,
                         int64_t debug, ffi::RemainingArgs args, ffi::Result<ffi::AnyBuffer> out) {
    const Attrs a{iflag,   n_tot,      n_transf,   n_j,
                  {n_k_1, n_k_2, n_k_3}, modeord, upsampfac, gpu_method,
                  gpu_sort, gpu_kerevalmeth, gpu_maxbatchsize, debug};
    const size_t want = 1 + DIM + (TYPE == 3 ? DIM : 0);
    if (args.size() != want) return ffi::Error::InvalidArgument("wrong number of buffers");
    auto buf = [&](size_t i) -> const void* {
      auto b = args.get<ffi::AnyBuffer>(i);
      return b.has_value() ? b.value().untyped_data() : nullptr;
    };
    const void* pts[3] = {nullptr, nullptr, nullptr};
    const void* tgts[3] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < DIM; ++d) pts[d] = buf(1 + d);
    if (TYPE == 3)
      for (int d = 0; d < DIM; ++d) tgts[d] = buf(1 + DIM + d);
    return run(TYPE, DIM, sizeof(EPS) == 4, stream, (double)eps, a, buf(0), pts, tgts,
               out->untyped_data());
  }
};

template <int DIM, int TYPE, typename EPS>
constexpr auto binding() {
  return ffi::Ffi::Bind()
      .Ctx<ffi::PlatformStream<cudaStream_t>>()
      .template Attr<EPS>("eps")
      .template Attr<int64_t>("iflag")
      .template Attr<int64_t>("n_tot")
      .template Attr<int64_t>("n_transf")
      .template Attr<int64_t>("n_j")
      .template Attr<int64_t>("n_k_1")
      .template Attr<int64_t>("n_k_2")
      .template Attr<int64_t>("n_k_3")
      .template Attr<int64_t>("modeord")
      .template Attr<double>("upsampfac")
      .template Attr<int64_t>("gpu_method")
      .template Attr<int64_t>("gpu_sort")
      .template Attr<int64_t>("gpu_kerevalmeth")
      .template Attr<int64_t>("gpu_maxbatchsize")
      .template Attr<int64_t>("debug")
      .RemainingArgs()
      .template Ret<ffi::AnyBuffer>();
}

}  // namespace

#define GBN_TARGET(NAME, DIM, TYPE, EPS)                                         \
  XLA_FFI_DEFINE_HANDLER_SYMBOL(NAME, (Target<DIM, TYPE, EPS>::call),            \
                                (binding<DIM, TYPE, EPS>()));
GBN_TARGET(nufft1d1f, 1, 1, float)
GBN_TARGET(nufft1d1, 1, 1, double)
GBN_TARGET(nufft2d1f, 2, 1, float)
GBN_TARGET(nufft2d1, 2, 1, double)
GBN_TARGET(nufft3d1f, 3, 1, float)
GBN_TARGET(nufft3d1, 3, 1, double)
GBN_TARGET(nufft1d2f, 1, 2, float)
GBN_TARGET(nufft1d2, 1, 2, double)
GBN_TARGET(nufft2d2f, 2, 2, float)
GBN_TARGET(nufft2d2, 2, 2, double)
GBN_TARGET(nufft3d2f, 3, 2, float)
GBN_TARGET(nufft3d2, 3, 2, double)
GBN_TARGET(nufft1d3f, 1, 3, float)
GBN_TARGET(nufft1d3, 1, 3, double)
GBN_TARGET(nufft2d3f, 2, 3, float)
GBN_TARGET(nufft2d3, 2, 3, double)
GBN_TARGET(nufft3d3f, 3, 3, float)
GBN_TARGET(nufft3d3, 3, 3, double)
#undef GBN_TARGET

// jax_finufft_gpu.registrations(): target name -> handler capsule, as
// src/jax_finufft/lowering.py:15-19 consumes it.
PYBIND11_MODULE(jax_finufft_gpu, m) {
  m.def("registrations", []() {
    py::dict d;
#define GBN_REG(NAME) d[#NAME] = py::capsule(reinterpret_cast<void*>(NAME));
    GBN_REG(nufft1d1f) GBN_REG(nufft1d1) GBN_REG(nufft2d1f) GBN_REG(nufft2d1)
    GBN_REG(nufft3d1f) GBN_REG(nufft3d1) GBN_REG(nufft1d2f) GBN_REG(nufft1d2)
    GBN_REG(nufft2d2f) GBN_REG(nufft2d2) GBN_REG(nufft3d2f) GBN_REG(nufft3d2)
    GBN_REG(nufft1d3f) GBN_REG(nufft1d3) GBN_REG(nufft2d3f) GBN_REG(nufft2d3)
    GBN_REG(nufft3d3f) GBN_REG(nufft3d3)
#undef GBN_REG
    return d;
  });
}

// dtrt_gb300 — render kernels and orchestration instantiated for nder = 3.
#include "dt_render.cuh"

namespace dt {
template int render_n<3>(dtrt_scene *, const dtrt_render_options *, float *, int, cudaStream_t);
template int render_n_noalloc<3>(dtrt_scene *, const dtrt_render_options *, float *, int, cudaStream_t,
                                  unsigned char *, size_t);
}

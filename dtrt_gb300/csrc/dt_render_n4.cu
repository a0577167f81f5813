// dtrt_gb300 — render kernels and orchestration instantiated for nder = 4.
#include "dt_render.cuh"

namespace dt {
template int render_n<4>(dtrt_scene *, const dtrt_render_options *, float *, int, cudaStream_t);
template int render_n_noalloc<4>(dtrt_scene *, const dtrt_render_options *, float *, int, cudaStream_t,
                                  unsigned char *, size_t);
}

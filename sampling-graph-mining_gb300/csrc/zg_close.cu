// zg_close.cu — ZGraphInstance::conditional_close with the found edge ids written back
// (src/ZGraphInstance.cpp:410-441) as a device primitive: one query per thread.
//
// The reference scans the edge-id-ordered list of every sampled vertex for each edge to wait.  On
// a simple graph (the build rejects duplicate edges) the edge (x, y) appears in exactly two lists,
// x's and y's, so the scan finds it iff one of x, y is a sampled vertex and the edge exists with an
// id >= min_valid; the cuckoo table answers the second part in one or two sector reads, and its
// answer is the edge's id, which is what the reference writes back.
#include "zg_programs.cuh"

namespace {

constexpr int kCloseBlock = 128;

__global__ void __launch_bounds__(kCloseBlock) k_close(ZgDevGraph g, const zg_close_query* __restrict__ q, uint32_t n,
                                                       zg_close_result* __restrict__ out) {
  const uint32_t i = blockIdx.x * kCloseBlock + threadIdx.x;
  if (i >= n) return;
  const zg_close_query& x = q[i];
  zg_close_result r;
  r.closed = 0;
  r.found = 0;
  for (int k = 0; k < ZG_MAX_LIST; ++k) r.edge_ids[k] = 0;
  const uint32_t nv = x.num_vertices < ZG_MAX_LIST ? x.num_vertices : ZG_MAX_LIST;
  const uint32_t ne = x.num_edges < ZG_MAX_LIST ? x.num_edges : ZG_MAX_LIST;
  bool all = true;
  for (uint32_t k = 0; k < ne && all; ++k) {
    const uint32_t a = x.edges[2 * k], b = x.edges[2 * k + 1];
    bool sampled = false;  // the edge lies in some sampled vertex's list only if an endpoint is sampled
    for (uint32_t j = 0; j < nv; ++j) sampled |= x.vertices[j] == a || x.vertices[j] == b;
    int64_t id = -1;
    if (sampled && a < g.nv && b < g.nv && a != b) id = edge_confirm(g, edge_candidate(g, a, b));
    if (id >= 0 && (uint64_t)id >= x.min_valid_edge_id) {
      r.edge_ids[k] = (uint64_t)id;
      r.found = k + 1;
    } else {
      all = false;
    }
  }
  r.closed = all ? 1u : 0u;
  out[i] = r;
}

}  // namespace

extern "C" int zg_conditional_close(const zg_graph* g, const zg_close_query* queries, uint32_t n, void* cuda_stream,
                                    zg_close_result* results) {
  if (!g || (n && (!queries || !results)))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_conditional_close: null argument"), ZG_ERR_INVALID_ARG;
  for (uint32_t i = 0; i < n; ++i)
    if (queries[i].num_vertices > ZG_MAX_LIST || queries[i].num_edges > ZG_MAX_LIST)
      return zg_set_error(ZG_ERR_INVALID_ARG, "zg_conditional_close: query %u has more than %d vertices or edges", i,
                          ZG_MAX_LIST),
             ZG_ERR_INVALID_ARG;
  if (n == 0) return ZG_OK;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  zg_close_query* dq = nullptr;
  zg_close_result* dr = nullptr;
  ZG_CUDA(zg_malloc_async((void**)&dq, sizeof(zg_close_query) * (size_t)n, s));
  cudaError_t e = zg_malloc_async((void**)&dr, sizeof(zg_close_result) * (size_t)n, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dq, queries, sizeof(zg_close_query) * (size_t)n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    ZgDevGraph d = g->d;
    k_close<<<(n + kCloseBlock - 1) / kCloseBlock, kCloseBlock, 0, s>>>(d, dq, n, dr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(results, dr, sizeof(zg_close_result) * (size_t)n, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(dq, s);
  if (dr) cudaFreeAsync(dr, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return zg_check_cuda(e, "zg_conditional_close");
  return ZG_OK;
}

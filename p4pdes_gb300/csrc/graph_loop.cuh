// graph_loop.cuh -- an iterative solver's loop body repeated on the device.
//
// The body (the kernels of a few solver iterations, captured once) sits in
// a graph as the child of a conditional WHILE node; a one-thread kernel at
// the end of the body sets the condition from the solver's own stop flag.
// One graph launch then runs the whole solve, with no host round trip per
// body (the host used to read the flag back after every body).  The body
// count is capped: after `cap` bodies the loop ends whatever the flag says,
// and the caller reports the unfinished solve.
#pragma once

#include <cuda_runtime.h>

namespace fg {

// Continue while (done == NULL or *done == 0) and (ndone == NULL or
// *ndone < nneed) and fewer than `cap` bodies have run; *count counts them.
static __global__ void k_loop_while(cudaGraphConditionalHandle h, const int *done, const unsigned int *ndone,
                                    unsigned int nneed, unsigned int *count, unsigned int cap) {
  const unsigned int c = *count + 1;
  *count = c;
  bool stop = c >= cap;
  if (done && __ldcg(done) != 0) stop = true;
  if (ndone && __ldcg(ndone) >= nneed) stop = true;
  cudaGraphSetConditional(h, stop ? 0u : 1u);
}

// Kernel nodes of a graph (for the launch count)
static inline long long graph_kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
  cudaGraphNode_t *nodes = new cudaGraphNode_t[n];
  long long k = 0;
  if (cudaGraphGetNodes(g, nodes, &n) == cudaSuccess)
    for (size_t q = 0; q < n; q++) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nodes[q], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
    }
  delete[] nodes;
  return k;
}

// Builds the loop graph: `enq` enqueues one body on `s` (captured into the
// WHILE node's child graph), followed by the condition kernel.  On success
// *exec is instantiated and *nbody holds the body's kernel nodes (condition
// kernel included).  Returns false if the driver refuses the construction.
template <typename F>
static bool build_loop_graph(cudaStream_t s, F enq, const int *done, const unsigned int *ndone, unsigned int nneed,
                             unsigned int *count, unsigned int cap, cudaGraphExec_t *exec, long long *nbody) {
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  bool ok = false;
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams p = {};
  cudaGraphNode_t node;
  if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess) {
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p) == cudaSuccess) {
      cudaGraph_t body = p.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
          cudaSuccess) {
        enq();
        k_loop_while<<<1, 1, 0, s>>>(h, done, ndone, nneed, count, cap);
        const cudaError_t e = cudaStreamEndCapture(s, &body);
        if (e == cudaSuccess) {
          *nbody = graph_kernel_nodes(body);
          ok = cudaGraphInstantiate(exec, g, 0) == cudaSuccess;
        }
      }
    }
  }
  cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();
    *exec = nullptr;
  }
  return ok;
}

}  // namespace fg

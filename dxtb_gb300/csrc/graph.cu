// CUDA graphs of whole single points.
//
// A caller that repeats the same packed batch with new positions (geometry
// optimisation, molecular dynamics, the repeated calls of a calculator)
// captures the sequence of this library's launches once and replays it:
// the geometry kernels, the integrals, every size class's SCF (and
// gradient) launch on its forked stream and the joins. Replays cost one
// graph launch instead of one host call per kernel.
//
// The capture is thread-local: other host threads of the process keep
// working, and any allocating or synchronising call made by this thread
// while it captures invalidates the capture (dxtb_graph_end then fails).
// The graph is instantiated with node priorities, so the priorities that
// the SCF sets on its class launches (larger classes first: their CTAs need
// whole SMs and bound the batch's makespan) hold on replay.

#include "common.cuh"

extern "C" int32_t dxtb_graph_begin(void *stream) {
  if (stream == nullptr) return DXTB_ERR_ARGS;  // the legacy stream cannot be captured
  if (cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return DXTB_ERR_LAUNCH;
  }
  return DXTB_OK;
}

extern "C" int32_t dxtb_graph_end(void *stream, void **exec) {
  if (stream == nullptr || exec == nullptr) return DXTB_ERR_ARGS;
  *exec = nullptr;
  cudaGraph_t graph = nullptr;
  if (cudaStreamEndCapture((cudaStream_t)stream, &graph) != cudaSuccess || graph == nullptr) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    return DXTB_ERR_LAUNCH;
  }
  cudaGraphExec_t ge = nullptr;
  const cudaError_t e = cudaGraphInstantiateWithFlags(&ge, graph, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess || ge == nullptr) {
    cudaGetLastError();
    return DXTB_ERR_LAUNCH;
  }
  *exec = ge;
  return DXTB_OK;
}

extern "C" int32_t dxtb_graph_launch(void *exec, void *stream) {
  if (exec == nullptr) return DXTB_ERR_ARGS;
  if (cudaGraphLaunch((cudaGraphExec_t)exec, (cudaStream_t)stream) != cudaSuccess) {
    cudaGetLastError();
    return DXTB_ERR_LAUNCH;
  }
  return DXTB_OK;
}

extern "C" int32_t dxtb_graph_destroy(void *exec) {
  if (exec == nullptr) return DXTB_OK;
  return cudaGraphExecDestroy((cudaGraphExec_t)exec) == cudaSuccess ? DXTB_OK : DXTB_ERR_LAUNCH;
}

// CUDA-graph capture of library calls.
//
// A graph recorded on one stream replays every library call made on it
// during the capture (kernels, the ragged work-counter reset, stream-ordered
// scratch allocations) with one launch, which removes the per-call host cost
// of short launches.  Per-device state that a call creates on first use (the
// device error word, the scratch pool, default resample taps, tensor maps'
// driver entry point) must exist before the capture: call scir_init() and
// make one call of each operation with the same shapes first.  The capture
// uses cudaStreamCaptureModeThreadLocal, so other host threads are not
// restricted while this one records.
#include "common.cuh"
#include "kernels.cuh"

struct scir_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int device = -1;
};

using namespace scir;

extern "C" {

SCIR_API int scir_graph_capture_begin(void* stream) {
    clear_error();
    SCIR_REQUIRE(stream != nullptr, SCIR_ERR_INVALID_ARG,
                 "capture needs a created stream (not the legacy default stream)");
    SCIR_CUDA_TRY(cudaStreamBeginCapture(as_stream(stream), cudaStreamCaptureModeThreadLocal));
    return SCIR_OK;
}

SCIR_API int scir_graph_capture_end(void* stream, scir_graph** out) {
    clear_error();
    SCIR_REQUIRE(stream != nullptr && out != nullptr, SCIR_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    cudaGraph_t g = nullptr;
    SCIR_CUDA_TRY(cudaStreamEndCapture(as_stream(stream), &g));
    cudaGraphExec_t e = nullptr;
    const cudaError_t ce = cudaGraphInstantiate(&e, g, 0);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        return set_error(SCIR_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ce));
    }
    auto* r = new scir_graph();
    r->graph = g;
    r->exec = e;
    SCIR_CUDA_TRY(cudaGetDevice(&r->device));
    *out = r;
    return SCIR_OK;
}

SCIR_API int scir_graph_launch(const scir_graph* graph, void* stream) {
    clear_error();
    SCIR_REQUIRE(graph != nullptr, SCIR_ERR_INVALID_ARG, "graph is NULL");
    int dev = -1;
    SCIR_CUDA_TRY(cudaGetDevice(&dev));
    SCIR_REQUIRE(dev == graph->device, SCIR_ERR_INVALID_ARG,
                 "graph was captured on device %d, current device is %d", graph->device, dev);
    SCIR_CUDA_TRY(cudaGraphLaunch(graph->exec, as_stream(stream)));
    return SCIR_OK;
}

SCIR_API int scir_graph_destroy(scir_graph* graph) {
    if (!graph) return SCIR_OK;
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    delete graph;
    return SCIR_OK;
}

}  // extern "C"

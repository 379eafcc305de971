#include "event.cuh"
struct EventEngine::Impl {};
EventEngine::EventEngine() : impl_(nullptr) {}
EventEngine::~EventEngine() {}
int EventEngine::init(const nraps_problem&, const nraps_opts&, GenState*, double*, SiteSink, nraps_site*,
                      nraps_site*, cudaStream_t, std::string& err) {
    err = "WOODCOCK tracking is not available in this build";
    return NRAPS_ERR_INVALID;
}
int EventEngine::enqueue_generation(cudaStream_t) { return -1; }
uint64_t EventEngine::launches_per_generation() const { return 0; }

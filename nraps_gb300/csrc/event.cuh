/*
 * event.cuh — the event-based Woodcock (delta-tracking) transport engine.
 */
#ifndef NRAPS_EVENT_CUH
#define NRAPS_EVENT_CUH
#include <string>

#include "engine.cuh"

class EventEngine {
public:
    EventEngine();
    ~EventEngine();
    /* Build device tables and particle queues for one problem. */
    int init(const nraps_problem& p, const nraps_opts& o, GenState* st, double* tally,
             SiteSink sink, nraps_site* bank0, nraps_site* bank1, cudaStream_t s, std::string& err);
    /* Enqueue one generation's transport; returns kernels launched, <0 on error. */
    int enqueue_generation(cudaStream_t s);
    uint64_t launches_per_generation() const;

private:
    struct Impl;
    Impl* impl_;
};
#endif

// Test scaffolding, not product code.
//
// A C wrapper around the MassiveMDS reference CPU engine, compiled straight
// from the reference's own sources (see oracle/Makefile) into
// oracle/_ref/libmdsref.so. Tests and the golden-fixture script load it with
// ctypes to pin the oracle restatement (oracle/mds_oracle.c) and the CUDA
// engine against the reference's own arithmetic. Nothing in the product links
// or loads this library.
//
// Engines reachable through mds::factory (src/factory.cpp:32-118) without
// HAVE_OPENCL / USE_SIMD: DoubleNoParallelNoSimd, DoubleTbbNoSimd,
// FloatNoParallelNoSimd, FloatTbbNoSimd (TBB = std::thread stand-in).
#include <cstddef>
#include <exception>
#include <memory>

// Defines the construct* factory functions (src/NewMultiDimensionalScaling.hpp:786-824),
// which src/factory.cpp references.
#include "NewMultiDimensionalScaling.hpp"

namespace {
struct Handle {
    mds::SharedPtr engine;
};
}  // namespace

extern "C" {

void* mdsref_create(int embeddingDimension, int locationCount, long flags, int threads) {
    try {
        auto* h = new Handle;
        h->engine = mds::factory(embeddingDimension, locationCount, flags, -1, threads);
        return h;
    } catch (const std::exception&) {
        return nullptr;
    }
}

void mdsref_destroy(void* h) { delete static_cast<Handle*>(h); }

void mdsref_set_pairwise_data(void* h, double* data, size_t length) {
    static_cast<Handle*>(h)->engine->setPairwiseData(data, length);
}

void mdsref_update_locations(void* h, int index, double* x, size_t length) {
    static_cast<Handle*>(h)->engine->updateLocations(index, x, length);
}

void mdsref_set_parameters(void* h, double* p, size_t length) {
    static_cast<Handle*>(h)->engine->setParameters(p, length);
}

double mdsref_get_sum_of_increments(void* h) {
    return static_cast<Handle*>(h)->engine->getSumOfIncrements();
}

void mdsref_get_log_likelihood_gradient(void* h, double* out, size_t length) {
    static_cast<Handle*>(h)->engine->getLogLikelihoodGradient(out, length);
}

void mdsref_store_state(void* h) { static_cast<Handle*>(h)->engine->storeState(); }
void mdsref_restore_state(void* h) { static_cast<Handle*>(h)->engine->restoreState(); }
void mdsref_accept_state(void* h) { static_cast<Handle*>(h)->engine->acceptState(); }
void mdsref_make_dirty(void* h) { static_cast<Handle*>(h)->engine->makeDirty(); }
int mdsref_get_internal_dimension(void* h) {
    return static_cast<Handle*>(h)->engine->getInternalDimension();
}

}  // extern "C"

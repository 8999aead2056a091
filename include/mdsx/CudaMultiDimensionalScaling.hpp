// Header-only drop-in engine: mds::CudaMultiDimensionalScaling implements the
// MassiveMDS engine interface (src/AbstractMultiDimensionalScaling.hpp:38-73)
// on top of the C ABI of libmdsx.so (include/mdsx.h).
//
// Callers that hold an mds::SharedPtr (the reference benchmark,
// src/benchmark.cpp:167; the Rcpp glue, src/MassiveMDS.cpp:97; the JNI
// singleton, src/jni/...NativeMDSSingleton.cpp:13-24) use it unchanged. The
// reference signals errors with assert/exit (src/NewMultiDimensionalScaling.hpp:140,
// src/backend/opencl/OpenCLMultiDimensionalScaling.hpp:128-131); this class
// throws mds::CudaEngineError carrying the C-ABI status and message instead.
//
// Build against the reference header: -DMDSX_USE_REFERENCE_HEADER -I<reference>/src
// Otherwise the restated interface in include/mdsx/ is used.
#ifndef MDSX_CUDA_MULTIDIMENSIONAL_SCALING_HPP
#define MDSX_CUDA_MULTIDIMENSIONAL_SCALING_HPP

#ifdef MDSX_USE_REFERENCE_HEADER
#include "AbstractMultiDimensionalScaling.hpp"
#else
#include "mdsx/AbstractMultiDimensionalScaling.hpp"
#endif

#include <memory>
#include <stdexcept>
#include <string>

#include "mdsx.h"

namespace mds {

class CudaEngineError : public std::runtime_error {
public:
    CudaEngineError(int status, const std::string& what) : std::runtime_error(what), status(status) {}
    int status;
};

class CudaMultiDimensionalScaling : public AbstractMultiDimensionalScaling {
public:
    CudaMultiDimensionalScaling(int embeddingDimension, int locationCount, long flags, int device)
        : AbstractMultiDimensionalScaling(embeddingDimension, locationCount, flags) {
        check(mdsx_create(embeddingDimension, locationCount, flags, device, &engine_), "mdsx_create");
        isLeftTruncated = (flags & MDSX_FLAG_LEFT_TRUNCATION) != 0;
    }

    ~CudaMultiDimensionalScaling() override {
        if (engine_) mdsx_destroy(engine_);
    }

    CudaMultiDimensionalScaling(const CudaMultiDimensionalScaling&) = delete;
    CudaMultiDimensionalScaling& operator=(const CudaMultiDimensionalScaling&) = delete;

    void updateLocations(int locationIndex, double* location, size_t length) override {
        check(mdsx_update_locations(engine_, locationIndex, location, length), "updateLocations");
        updatedLocation = locationIndex;
        sumOfIncrementsKnown = false;
    }

    double getSumOfIncrements() override {
        double out = 0.0;
        check(mdsx_get_sum_of_increments(engine_, &out), "getSumOfIncrements");
        sumOfIncrementsKnown = true;
        return out;
    }

    void getLogLikelihoodGradient(double* result, size_t length) override {
        check(mdsx_get_log_likelihood_gradient(engine_, result, length), "getLogLikelihoodGradient");
    }

    void storeState() override { check(mdsx_store_state(engine_), "storeState"); }

    void restoreState() override {
        check(mdsx_restore_state(engine_), "restoreState");
        sumOfIncrementsKnown = true;
    }

    void acceptState() override { check(mdsx_accept_state(engine_), "acceptState"); }

    void setPairwiseData(double* data, size_t length) override {
        check(mdsx_set_pairwise_data(engine_, data, length), "setPairwiseData");
    }

    void setParameters(double* data, size_t length) override {
        check(mdsx_set_parameters(engine_, data, length), "setParameters");
    }

    void makeDirty() override {
        check(mdsx_make_dirty(engine_), "makeDirty");
        sumOfIncrementsKnown = false;
        incrementsKnown = false;
    }

    int getInternalDimension() override {
        int out = 0;
        check(mdsx_get_internal_dimension(engine_, &out), "getInternalDimension");
        return out;
    }

    // Not in the reference interface: the R layer's log-likelihood (R/mds.R:24-28).
    double getLogLikelihood() {
        double out = 0.0;
        check(mdsx_get_log_likelihood(engine_, &out), "getLogLikelihood");
        return out;
    }

    mdsx_engine* handle() { return engine_; }

private:
    void check(int status, const char* what) {
        if (status != MDSX_OK) {
            throw CudaEngineError(status, std::string(what) + ": " + mdsx_last_error(engine_));
        }
    }

    mdsx_engine* engine_ = nullptr;
};

// The CUDA branch of mds::factory (src/factory.cpp:32-118): flags with OPENCL
// or CUDA set select this engine; FLOAT selects the FP32 sweep.
inline SharedPtr constructCudaMultiDimensionalScaling(int embeddingDimension, int locationCount, long flags,
                                                      int device) {
    return std::make_shared<CudaMultiDimensionalScaling>(embeddingDimension, locationCount, flags, device);
}

}  // namespace mds

#endif  // MDSX_CUDA_MULTIDIMENSIONAL_SCALING_HPP

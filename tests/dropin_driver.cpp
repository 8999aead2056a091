// Test driver (not product code): runs the C++ drop-in engine
// mds::CudaMultiDimensionalScaling (include/mdsx/CudaMultiDimensionalScaling.hpp)
// through the call sequence of the reference benchmark (src/benchmark.cpp:167-309
// of MassiveMDS): mds::factory, setPairwiseData, the initial locations one at
// a time, setParameters, makeDirty, getSumOfIncrements, getLogLikelihoodGradient,
// then per iteration storeState, updateLocations(-1), getSumOfIncrements,
// restoreState or acceptState, getLogLikelihoodGradient.
//
// The factory below is the reference factory's dispatch with its CUDA branch
// (OPENCL or CUDA bit -> the drop-in); the reference's CPU engines are not
// linked here, so other flags are an error.
//
// It also checks, through a subclass that can read them, the protected flags
// the reference's callers and subclasses rely on (updatedLocation,
// sumOfIncrementsKnown, isLeftTruncated) and that a wrong length throws
// mds::CudaEngineError with MDSX_EINVAL instead of asserting.
//
// usage: dropin_driver <input> <output>
//   input : int32 n, p, iterations; int64 flags; double tau; delta[n*n];
//           x0[n*p]; xs[iterations][n*p]; uint8 restore[iterations]
//   output: double sums[iterations + 1]; double gradients[iterations + 1][n*p]
// Exit status 0 on success; a message on stderr otherwise.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "mdsx/CudaMultiDimensionalScaling.hpp"

namespace mds {

// src/factory.cpp:32-118 with the CUDA branch; no CPU engines in this binary.
SharedPtr factory(int dim1, int dim2, long flags, int device, int /*threads*/) {
    if (flags & (Flags::OPENCL | MDSX_FLAG_CUDA)) return constructCudaMultiDimensionalScaling(dim1, dim2, flags, device);
    throw std::runtime_error("factory: this test binary provides the GPU engine only");
}

}  // namespace mds

namespace {

// Reads the protected state the reference's interface keeps.
class Probe : public mds::CudaMultiDimensionalScaling {
public:
    using mds::CudaMultiDimensionalScaling::CudaMultiDimensionalScaling;
    int updated() const { return updatedLocation; }
    bool sumKnown() const { return sumOfIncrementsKnown; }
    bool truncated() const { return isLeftTruncated; }
};

void require(bool ok, const std::string& what) {
    if (!ok) throw std::runtime_error("check failed: " + what);
}

template <typename T>
void read(FILE* f, T* dst, size_t count) {
    if (fread(dst, sizeof(T), count, f) != count) throw std::runtime_error("short input file");
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
        return 2;
    }
    try {
        FILE* in = fopen(argv[1], "rb");
        if (!in) throw std::runtime_error("cannot open input");
        int32_t hdr[3];
        int64_t flags = 0;
        double tau = 0.0;
        read(in, hdr, 3);
        read(in, &flags, 1);
        read(in, &tau, 1);
        const int n = hdr[0], p = hdr[1], iters = hdr[2];
        std::vector<double> delta((size_t)n * n), x0((size_t)n * p), xs((size_t)iters * n * p);
        std::vector<uint8_t> restore(iters);
        read(in, delta.data(), delta.size());
        read(in, x0.data(), x0.size());
        read(in, xs.data(), xs.size());
        read(in, restore.data(), restore.size());
        fclose(in);

        mds::SharedPtr instance = mds::factory(p, n, (long)flags, 0, 1);
        require(instance->getInternalDimension() == p, "getInternalDimension() == P");
        instance->setPairwiseData(delta.data(), delta.size());
        for (int i = 0; i < n; ++i) instance->updateLocations(i, &x0[(size_t)i * p], p);
        instance->setParameters(&tau, 1);
        instance->makeDirty();

        std::vector<double> sums, grads((size_t)(iters + 1) * n * p);
        sums.push_back(instance->getSumOfIncrements());
        instance->getLogLikelihoodGradient(&grads[0], (size_t)n * p);
        for (int it = 0; it < iters; ++it) {
            instance->storeState();
            instance->updateLocations(-1, &xs[(size_t)it * n * p], (size_t)n * p);
            sums.push_back(instance->getSumOfIncrements());
            if (restore[it])
                instance->restoreState();
            else
                instance->acceptState();
            instance->getLogLikelihoodGradient(&grads[(size_t)(it + 1) * n * p], (size_t)n * p);
        }

        // The interface's protected state, as the reference's engines keep it
        // (src/AbstractMultiDimensionalScaling.hpp:63-72).
        Probe probe(p, n, (long)flags, 0);
        require(probe.truncated() == ((flags & mds::Flags::LEFT_TRUNCATION) != 0), "isLeftTruncated");
        probe.setPairwiseData(delta.data(), delta.size());
        probe.updateLocations(-1, x0.data(), x0.size());
        require(probe.updated() == -1 && !probe.sumKnown(), "updateLocations(-1) marks the sum unknown");
        probe.setParameters(&tau, 1);
        const double s0 = probe.getSumOfIncrements();
        require(probe.sumKnown(), "getSumOfIncrements marks the sum known");
        probe.storeState();
        probe.updateLocations(3 % n, &xs[0], p);
        require(probe.updated() == 3 % n && !probe.sumKnown(), "updateLocations(i) records i");
        probe.restoreState();
        require(probe.sumKnown() && probe.getSumOfIncrements() == s0, "restoreState brings the stored sum back");
        probe.makeDirty();
        require(!probe.sumKnown(), "makeDirty marks the sum unknown");
        bool threw = false;
        try {
            std::vector<double> small(1);
            probe.getLogLikelihoodGradient(small.data(), small.size());
        } catch (const mds::CudaEngineError& e) {
            threw = e.status == MDSX_EINVAL;
        }
        require(threw, "a wrong gradient length throws CudaEngineError(MDSX_EINVAL)");

        FILE* out = fopen(argv[2], "wb");
        if (!out) throw std::runtime_error("cannot open output");
        fwrite(sums.data(), sizeof(double), sums.size(), out);
        fwrite(grads.data(), sizeof(double), grads.size(), out);
        fclose(out);
    } catch (const std::exception& e) {
        fprintf(stderr, "dropin_driver: %s\n", e.what());
        return 1;
    }
    return 0;
}

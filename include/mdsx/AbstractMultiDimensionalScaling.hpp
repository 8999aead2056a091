// The MassiveMDS engine interface, restated so code can build against this
// engine without the reference tree.
//
// Class name, namespace, method names, order, signatures and protected members
// are those of mds::AbstractMultiDimensionalScaling
// (src/AbstractMultiDimensionalScaling.hpp:38-77 of MassiveMDS): a drop-in has
// to present the same virtual interface. When the reference's own header is
// on the include path, define MDSX_USE_REFERENCE_HEADER and
// CudaMultiDimensionalScaling.hpp includes that instead of this file.
#ifndef MDSX_ABSTRACT_MULTIDIMENSIONAL_SCALING_HPP
#define MDSX_ABSTRACT_MULTIDIMENSIONAL_SCALING_HPP

#include <cstddef>
#include <memory>

namespace mds {

enum Flags {
    FLOAT = 1 << 2,
    TBB = 1 << 3,
    OPENCL = 1 << 4,
    LEFT_TRUNCATION = 1 << 5,
    SSE = 1 << 7,
    AVX = 1 << 8,
    AVX512 = 1 << 9
};

class AbstractMultiDimensionalScaling {
public:
    AbstractMultiDimensionalScaling(int embeddingDimension, int locationCount, long flags)
        : embeddingDimension(embeddingDimension), locationCount(locationCount),
          observationCount(locationCount * (locationCount - 1) / 2), flags(flags) {}

    virtual ~AbstractMultiDimensionalScaling() = default;

    virtual void updateLocations(int, double*, size_t) = 0;
    virtual double getSumOfIncrements() = 0;
    virtual void getLogLikelihoodGradient(double*, size_t) = 0;
    virtual void storeState() = 0;
    virtual void restoreState() = 0;
    virtual void acceptState() = 0;
    virtual void setPairwiseData(double*, size_t) = 0;
    virtual void setParameters(double*, size_t) = 0;
    virtual void makeDirty() = 0;
    virtual int getInternalDimension() = 0;

protected:
    int embeddingDimension;
    int locationCount;
    int observationCount;
    long flags;

    int updatedLocation = -1;
    bool incrementsKnown = false;
    bool sumOfIncrementsKnown = false;
    bool isLeftTruncated = false;
};

typedef std::shared_ptr<mds::AbstractMultiDimensionalScaling> SharedPtr;

}  // namespace mds

#endif  // MDSX_ABSTRACT_MULTIDIMENSIONAL_SCALING_HPP

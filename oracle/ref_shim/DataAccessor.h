/*
 * DataAccessor.h - in-memory stand-in for ISCE's image line accessor, used
 * only to build the reference's C++ CPU ampcor as a timed baseline (test
 * infrastructure, never shipped).
 *
 * The reference CPU port reads image lines through
 * iscesys/ImageApi/DataAccessor (components/zerodop/GPUampcor/src/
 * Ampcor.cpp:13,106-107,574-597: getLineBand(buffer, line, band) with a
 * 0-based line, DataAccessorNoCaster.cpp:13-18) and writes its tables with
 * setLineSequential (Ampcor.cpp:64-81).  This class keeps those two calls and
 * serves lines from a row-major image already in host memory; lines outside
 * the image read as zeros.  Written lines are discarded (the caller reads the
 * results from the Ampcor object's arrays).
 */
#ifndef AMPCOR_REF_SHIM_DATAACCESSOR_H
#define AMPCOR_REF_SHIM_DATAACCESSOR_H

#include <cstddef>
#include <cstdint>
#include <cstring>

class DataAccessor {
public:
    DataAccessor(const char* data, int width, int height, int pixel_bytes)
        : data_(data), width_(width), height_(height), pixel_(pixel_bytes) {}

    int getLineBand(char* buf, int pos, int band)
    {
        (void)band;
        const size_t row = (size_t)width_ * (size_t)pixel_;
        if (data_ == nullptr || pos < 0 || pos >= height_) {
            std::memset(buf, 0, row);
            return 0;
        }
        std::memcpy(buf, data_ + (size_t)pos * row, row);
        return 0;
    }

    void setLineSequential(char* buf) { (void)buf; }

private:
    const char* data_;
    int width_;
    int height_;
    int pixel_;
};

#endif

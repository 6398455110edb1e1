/*
 * GDALImage.h - GDAL-free stand-in used only to build the reference
 * PyCuAmpcor as a parity checker (test infrastructure, never shipped).
 *
 * The reference opens its images through GDAL's virtual-memory reader
 * (contrib/PyCuAmpcor/src/GDALImage.h:21-80, GDALImage.cpp:23-153).  GDAL is
 * not installed on either machine, so this header replaces that class with
 * one of the same interface (constructor from a file name, getters, and
 * loadToDevice with the same argument meaning) that reads a raw row-major
 * file instead.  The image shape comes from a side file "<name>.shape"
 * holding "height width bytes_per_pixel".  Only the interface is kept; the
 * body is this project's.
 */
#ifndef AMPCOR_REF_SHIM_GDALIMAGE_H
#define AMPCOR_REF_SHIM_GDALIMAGE_H

#include <cuda_runtime.h>
#include <driver_types.h>

#include <cstdio>
#include <cstdlib>
#include <string>
/* GDAL's headers bring in the standard library headers below; the reference's
 * chunk header relies on them (std::unique_ptr, cuAmpcorChunk.h:75-76). */
#include <memory>
#include <vector>

/* The reference's controller registers GDAL's drivers before opening files
 * (cuAmpcorController.cpp:42); there is nothing to register here. */
inline void GDALAllRegister() {}

class GDALImage {
public:
    using size_t = std::size_t;

    GDALImage() = delete;
    GDALImage(std::string fn, int band = 1, int cacheSizeInGB = 0, int useMmap = 1);
    ~GDALImage();

    void* getmemPtr() { return mem_; }
    int getHeight() { return height_; }
    int getWidth() { return width_; }
    int getPixelSize() { return pixel_; }
    bool isComplex() { return pixel_ == 8; }

    /* Copies the h_tile x w_tile tile at (h_offset, w_offset) to dArray
     * (row pitch w_tile pixels) on `stream`, as GDALImage.cpp:107-124 does
     * from its memory map. */
    void loadToDevice(void* dArray, size_t h_offset, size_t w_offset, size_t h_tile, size_t w_tile,
                      cudaStream_t stream);

private:
    int height_ = 0;
    int width_ = 0;
    int pixel_ = 0;
    char* mem_ = nullptr;
};

#endif

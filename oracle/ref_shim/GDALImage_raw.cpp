/*
 * Raw-file body of the GDAL-free GDALImage stand-in (see GDALImage.h in this
 * directory).  Test infrastructure for the reference build only.
 */
#include "GDALImage.h"

#include <fstream>
#include <stdexcept>

static void fail(const std::string& what)
{
    std::fprintf(stderr, "GDALImage stand-in: %s\n", what.c_str());
    std::exit(EXIT_FAILURE);
}

GDALImage::GDALImage(std::string fn, int band, int cacheSizeInGB, int useMmap)
{
    (void)band;
    (void)cacheSizeInGB;
    (void)useMmap;
    std::ifstream shp(fn + ".shape");
    if (!(shp >> height_ >> width_ >> pixel_) || height_ <= 0 || width_ <= 0 || (pixel_ != 4 && pixel_ != 8))
        fail("cannot read " + fn + ".shape");
    const size_t bytes = (size_t)height_ * (size_t)width_ * (size_t)pixel_;
    mem_ = static_cast<char*>(std::malloc(bytes));
    if (!mem_) fail("out of host memory");
    std::ifstream in(fn, std::ios::binary);
    if (!in.read(mem_, (std::streamsize)bytes)) fail("cannot read " + fn);
}

GDALImage::~GDALImage() { std::free(mem_); }

void GDALImage::loadToDevice(void* dArray, size_t h_offset, size_t w_offset, size_t h_tile, size_t w_tile,
                             cudaStream_t stream)
{
    if (h_offset + h_tile > (size_t)height_ || w_offset + w_tile > (size_t)width_)
        fail("tile outside the image");
    const char* src = mem_ + (h_offset * (size_t)width_ + w_offset) * (size_t)pixel_;
    cudaError_t e = cudaMemcpy2DAsync(dArray, w_tile * pixel_, src, (size_t)width_ * pixel_, w_tile * pixel_,
                                      h_tile, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) fail(cudaGetErrorString(e));
}

/*
 * Volume.h -- binary mask container, source-compatible with the public API of
 * the reference's Volume (forBench/Volume.h:7-26): one byte per voxel,
 * zero-initialised, linear index x + W*y + W*H*z (forBench/Volume.h:51-54),
 * 3D and 2D constructors, dispose() frees.  Written for this library; the
 * storage is uint8_t so it can be handed to the C ABI as is.
 */
#ifndef HD_VOLUME_H
#define HD_VOLUME_H

#include <stdint.h>
#include <stdlib.h>

typedef unsigned char uchar;
typedef unsigned int uint;

class Volume {
public:
    Volume(int width, int height, int depth) : width_(width), height_(height), depth_(depth) {
        data_ = (bool*)calloc((size_t)width * height * depth, sizeof(bool));
    }
    Volume(int width, int height) : Volume(width, height, 1) {}

    bool getVoxelValue(int x, int y, int z) { return data_[index(x, y, z)]; }
    bool getPixelValue(int x, int y) { return data_[index(x, y, 0)]; }
    void setVoxelValue(bool value, int x, int y, int z) { data_[index(x, y, z)] = value; }
    void setPixelValue(bool value, int x, int y) { data_[index(x, y, 0)] = value; }
    uint getWidth() { return (uint)width_; }
    uint getHeight() { return (uint)height_; }
    uint getDepth() { return (uint)depth_; }
    bool* getVolume() { return data_; }
    /* The mask as bytes for the C ABI (bool is one byte on every supported target). */
    const uint8_t* bytes() const { return reinterpret_cast<const uint8_t*>(data_); }
    void dispose() {
        free(data_);
        data_ = nullptr;
    }

private:
    size_t index(int x, int y, int z) const {
        return (size_t)x + (size_t)width_ * y + (size_t)width_ * height_ * z;
    }
    bool* data_;
    int width_, height_, depth_;
};

static_assert(sizeof(bool) == 1, "Volume hands its bool storage to the C ABI as bytes");

#endif /* HD_VOLUME_H */

// hd_hdf5.cpp -- HDF5 mask loader, the counterpart of loadHDFIntoBoolArr
// (forBench/hdf5Manag.cu:44-86): open the file, open the dataset, read its
// rank-1 extent, read it as native booleans into a malloc'd byte array.
// Built only when HDF5's C library is available (-DHD_WITH_HDF5 and
// -lhdf5); otherwise the entry point reports HD_ERR_UNSUPPORTED.
#include <cstdlib>

#include "hd/hd.h"

#ifdef HD_WITH_HDF5
#include <hdf5.h>
#endif

extern "C" hd_status hd_load_hdf5_bool(const char* path, const char* dataset, uint8_t** out, size_t* n) {
    if (!path || !dataset || !out || !n) return HD_ERR_BAD_ARG;
    *out = nullptr;
    *n = 0;
#ifdef HD_WITH_HDF5
    hid_t f = H5Fopen(path, H5F_ACC_RDONLY, H5P_DEFAULT);
    if (f < 0) return HD_ERR_BAD_ARG;
    hid_t d = H5Dopen2(f, dataset, H5P_DEFAULT);
    if (d < 0) {
        H5Fclose(f);
        return HD_ERR_BAD_ARG;
    }
    hid_t sp = H5Dget_space(d);
    hsize_t dims[8] = {0};
    const int rank = H5Sget_simple_extent_dims(sp, dims, nullptr);
    hd_status st = HD_OK;
    size_t count = 1;
    if (rank < 1 || rank > 8) st = HD_ERR_BAD_ARG;
    for (int i = 0; i < rank && st == HD_OK; ++i) count *= (size_t)dims[i];
    uint8_t* buf = nullptr;
    if (st == HD_OK) {
        buf = (uint8_t*)std::calloc(count ? count : 1, 1);
        if (!buf) st = HD_ERR_OOM;
    }
    if (st == HD_OK && H5Dread(d, H5T_NATIVE_HBOOL, H5S_ALL, H5S_ALL, H5P_DEFAULT, buf) < 0) st = HD_ERR_BAD_ARG;
    H5Sclose(sp);
    H5Dclose(d);
    H5Fclose(f);
    if (st != HD_OK) {
        std::free(buf);
        return st;
    }
    *out = buf;
    *n = count;
    return HD_OK;
#else
    return HD_ERR_UNSUPPORTED;
#endif
}

extern "C" void hd_free(void* p) { std::free(p); }

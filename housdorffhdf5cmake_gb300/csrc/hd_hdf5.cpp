// hd_hdf5.cpp -- HDF5 host entry.
//
// hd_load_hdf5_bool is the counterpart of loadHDFIntoBoolArr
// (forBench/hdf5Manag.cu:44-86): open the file, open the dataset, read its
// extent, read it as native booleans into a malloc'd byte array.
// hd_compute_hdf5 is the reference's whole host path for one pair: loadHDF
// (:196-214) loads two flat boolean datasets and benchmarkOliviera (:93-111)
// lays them out as Volumes (x + W*y + W*H*z, the flat order the datasets are
// stored in) and calls computeDistance; here the two byte arrays go straight
// to hd_compute_u8.
// Built only when HDF5's C library is available (-DHD_WITH_HDF5 and
// -lhdf5); otherwise both entry points report HD_ERR_UNSUPPORTED.
#include <cstdlib>
#include <cstring>

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
    // The reference reads NATIVE_HBOOL (the C library's boolean, one byte on
    // current builds).  A build whose boolean is wider reads into a buffer of
    // that element size and narrows to one byte per voxel (nonzero = 1).
    const size_t esz = H5Tget_size(H5T_NATIVE_HBOOL);
    if (st == HD_OK && esz == 1) {
        if (H5Dread(d, H5T_NATIVE_HBOOL, H5S_ALL, H5S_ALL, H5P_DEFAULT, buf) < 0) st = HD_ERR_BAD_ARG;
    } else if (st == HD_OK) {
        unsigned char* wide = esz ? (unsigned char*)std::calloc(count ? count : 1, esz) : nullptr;
        if (!wide) {
            st = esz ? HD_ERR_OOM : HD_ERR_BAD_ARG;
        } else {
            if (H5Dread(d, H5T_NATIVE_HBOOL, H5S_ALL, H5S_ALL, H5P_DEFAULT, wide) < 0) st = HD_ERR_BAD_ARG;
            for (size_t i = 0; i < count && st == HD_OK; ++i) {
                unsigned char nz = 0;
                for (size_t k = 0; k < esz; ++k) nz |= wide[i * esz + k];
                buf[i] = nz ? 1 : 0;
            }
            std::free(wide);
        }
    }
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

extern "C" hd_status hd_compute_hdf5(hd_context* ctx, const char* path_a, const char* dataset_a, const char* path_b,
                                     const char* dataset_b, int32_t W, int32_t H, int32_t D, hd_metric metric,
                                     hd_result* out) {
#ifdef HD_WITH_HDF5
    if (!ctx || !path_a || !dataset_a || !path_b || !dataset_b || !out) return HD_ERR_BAD_ARG;
    if (W <= 0 || H <= 0 || D <= 0) return HD_ERR_BAD_ARG;
    uint8_t *a = nullptr, *b = nullptr;
    size_t na = 0, nb = 0;
    hd_status st = hd_load_hdf5_bool(path_a, dataset_a, &a, &na);
    if (st == HD_OK) st = hd_load_hdf5_bool(path_b, dataset_b, &b, &nb);
    // the flat datasets must hold exactly one W x H x D volume each (the
    // reference trusts its hard-coded 512 x 512 x 826, hdf5Manag.cu:197-199)
    const size_t n = (size_t)W * H * D;
    if (st == HD_OK && (na != n || nb != n)) st = HD_ERR_BAD_ARG;
    if (st == HD_OK) st = hd_compute_u8(ctx, a, b, W, H, D, metric, out);
    std::free(a);
    std::free(b);
    return st;
#else
    (void)ctx, (void)path_a, (void)dataset_a, (void)path_b, (void)dataset_b, (void)W, (void)H, (void)D, (void)metric,
        (void)out;
    return HD_ERR_UNSUPPORTED;
#endif
}

extern "C" void hd_free(void* p) { std::free(p); }

/*
 * HausdorffDistance.h -- C++ drop-in for the reference's class
 * (forBench/HausdorffDistance.cuh:11-19):
 *
 *     HausdorffDistance hd;
 *     int d = hd.computeDistance(&img1, &img2);
 *
 * computeDistance keeps the reference's signature and return value (the
 * Hausdorff distance as a dilation count; the reference returns it at
 * forBench/HausdorffDistance.cu:185).  It runs on the GB300 library through
 * the C ABI of hd.h.  Differences, all on purpose: errors return -1 instead
 * of exiting the process, exactly one empty mask returns -1 at once instead of
 * looping forever, and the device is not reset.
 *
 * The structuring element follows the reference's compile-time switches
 * (forBench/HausdorffDistance.cuh:5-8): CHEBYSHEV 1 (the reference's default)
 * selects its 18-neighbour element, CHEBYSHEV 0 the 6-neighbour one.  IS_3D 0
 * is supported for 2D volumes (depth 1).  CUDA_DEVICE_INDEX picks the GPU.
 * computeDistances() adds the average HD.
 */
#ifndef HD_HAUSDORFF_DISTANCE_H
#define HD_HAUSDORFF_DISTANCE_H

#include "hd.h"
#include "Volume.h"

#ifndef CUDA_DEVICE_INDEX
#define CUDA_DEVICE_INDEX 0
#endif
#ifndef IS_3D
#define IS_3D 1
#endif
#ifndef CHEBYSHEV
#define CHEBYSHEV 1
#endif

class HausdorffDistance {
public:
    HausdorffDistance() : metric_(CHEBYSHEV ? HD_SE18_FORBENCH : HD_SE6) {}
    explicit HausdorffDistance(hd_metric metric) : metric_(metric) {}

    /* Max HD between the two masks (sizes of img1 are used for both, as in
     * forBench/HausdorffDistance.cu:103), or -1 on error / one empty mask. */
    int computeDistance(Volume* img1, Volume* img2) {
        hd_result r;
        return run(img1, img2, &r) == HD_OK ? r.hd : -1;
    }

    /* Max HD as above; *avgHd receives the average HD. */
    int computeDistances(Volume* img1, Volume* img2, double* avgHd) {
        hd_result r;
        const hd_status st = run(img1, img2, &r);
        if (avgHd) *avgHd = st == HD_OK ? r.avg_hd : -1.0;
        return st == HD_OK ? r.hd : -1;
    }

    /* Full result of the last kind (status, sums, counts, robust HD). */
    hd_status computeResult(Volume* img1, Volume* img2, hd_result* out) { return run(img1, img2, out); }

    /* The reference's HDF5 host path (loadHDF -> loadHDFIntoBoolArr x 2 ->
     * Volumes -> computeDistance, forBench/hdf5Manag.cu:196-214, 93-111):
     * max HD of two flat boolean datasets of width x height x depth
     * elements, or -1 on error (missing file or dataset, size mismatch, a
     * library built without HDF5, one empty mask). */
    int computeDistanceHdf5(const char* pathA, const char* datasetA, const char* pathB, const char* datasetB,
                            int width, int height, int depth) {
        hd_context* ctx = context();
        if (!ctx) return -1;
        hd_result r;
        return hd_compute_hdf5(ctx, pathA, datasetA, pathB, datasetB, width, height, depth, metric_, &r) == HD_OK
                   ? r.hd
                   : -1;
    }

private:
    static hd_context* context() {
        static hd_context* ctx = [] {
            hd_context* c = nullptr;
            if (hd_context_create(CUDA_DEVICE_INDEX, nullptr, &c) != HD_OK) c = nullptr;
            return c;
        }();
        return ctx;
    }
    hd_status run(Volume* img1, Volume* img2, hd_result* out) {
        if (!img1 || !img2 || !out) return HD_ERR_BAD_ARG;
        hd_context* ctx = context();
        if (!ctx) return HD_ERR_CUDA;
        const int W = (int)img1->getWidth(), H = (int)img1->getHeight(), D = (int)img1->getDepth();
        if (!IS_3D && D != 1) return HD_ERR_BAD_ARG;
        return hd_compute_u8(ctx, img1->bytes(), img2->bytes(), W, H, D, metric_, out);
    }
    hd_metric metric_;
};

#endif /* HD_HAUSDORFF_DISTANCE_H */

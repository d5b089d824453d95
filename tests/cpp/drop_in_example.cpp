// The reference's call site, unchanged in shape (forBench/hdf5Manag.cu:94-111):
// fill two Volumes voxel by voxel, construct HausdorffDistance, call
// computeDistance.  Prints "HD: <n> AVG: <x>" for the test to compare.
#include <cstdio>

#include "hd/HausdorffDistance.h"

int main() {
    const int W = 70, H = 50, D = 40;
    Volume img1 = Volume(W, H, D), img2 = Volume(W, H, D);
    for (int x = 0; x < W; x++)
        for (int y = 0; y < H; y++)
            for (int z = 0; z < D; z++) {
                const int dx = x - 30, dy = y - 25, dz = z - 20;
                img1.setVoxelValue(dx * dx + dy * dy + dz * dz <= 100, x, y, z);
                const int ex = x - 37, ey = y - 22, ez = z - 18;
                img2.setVoxelValue(ex * ex + ey * ey + ez * ez <= 64, x, y, z);
            }
    HausdorffDistance* hd = new HausdorffDistance();
    int dist = (*hd).computeDistance(&img1, &img2);
    double avg = 0;
    int dist2 = hd->computeDistances(&img1, &img2, &avg);
    printf("HD: %d AVG: %.17g\n", dist, avg);
    delete hd;
    img1.dispose();
    img2.dispose();
    return dist == dist2 ? 0 : 1;
}

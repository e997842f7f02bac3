// Host check of the z-chunk chooser of the chunked stencil kernels (wave_zchunk in
// spatialops-threadfix_gb300/csrc/common.cuh): over a sweep of tile counts, resident-slot
// counts, plane counts, halo overheads and alignments, the chosen chunk
//   - is a positive multiple of `align` whose chunks cover every plane;
//   - is at least min_planes, or covers nz in one chunk when nz is smaller;
//   - gives six or more waves whenever some admissible chunk does, and among those the
//     smallest rounds * (chunk + overhead).
// Prints "cases N" and "bad M"; M must be 0.
#include <cstdio>

#include "common.cuh"

int main() {
  const long tiles_list[] = {1, 2, 3, 4, 7, 16, 64, 128, 144, 256, 1024, 4096};
  const long slots_list[] = {152, 304, 456, 608, 760, 912, 1216};
  long cases = 0, bad = 0;
  for (long tiles : tiles_list)
    for (long slots : slots_list)
      for (int nz = 1; nz <= 600; nz += (nz < 40 ? 1 : 7))
        for (int overhead : {1, 4})
          for (int align : {1, 5}) {
            const int minp = 8;
            const int zc = nebo::wave_zchunk(tiles, slots, nz, overhead, minp, align);
            ++cases;
            const long chunks = zc > 0 ? (nz + zc - 1) / zc : 0;
            const int lo = minp < nz ? minp : nz;
            bool ok = zc >= 1 && zc % align == 0 && chunks >= 1 && (long)zc * chunks >= nz && zc >= lo;
            // the best admissible chunk with >= 6 waves, if any
            const int top = (nz + align - 1) / align * align;
            long best6 = -1;
            for (int c = top; c >= lo && c >= 1; c -= align) {
              const long ch = (nz + c - 1) / c, r = (tiles * ch + slots - 1) / slots;
              if (r >= 6 && (best6 < 0 || r * (c + overhead) < best6)) best6 = r * (c + overhead);
            }
            if (ok && best6 >= 0) {
              const long r = (tiles * chunks + slots - 1) / slots;
              ok = r >= 6 && r * (zc + overhead) == best6;
            }
            if (!ok) {
              if (bad < 10)
                std::printf("mismatch tiles=%ld slots=%ld nz=%d overhead=%d align=%d -> %d\n", tiles, slots, nz,
                            overhead, align, zc);
              ++bad;
            }
          }
  std::printf("cases %ld\nbad %ld\n", cases, bad);
  return 0;
}

// Device indices and storage modes (drop-in for spatialops/structured/MemoryTypes.h).
// Fields of this build always hold their values in GPU memory; CPU_INDEX names the host mirror.
#ifndef SpatialOps_MemoryTypes_h
#define SpatialOps_MemoryTypes_h

#define CPU_INDEX (-1)
#define GPU_INDEX 0
#define IS_CPU_INDEX(i) ((i) == CPU_INDEX)
#define IS_GPU_INDEX(i) ((i) >= 0)
#define IS_VALID_INDEX(i) ((i) >= -1)

namespace SpatialOps {
enum StorageMode { InternalStorage, ExternalStorage };
}
#endif

// The expression catalog (tests/cpp/catalog_cases.inc) compiled against the drop-in headers:
// every case becomes one fused sm_103a kernel.  Writes the same record file as the
// reference-built generator, so tests/test_gpu_catalog.py compares the two record by record.
//
//   catalog_gpu <domain> <out.bin>
#include <spatialops/structured/FVStaggered.h>
#include <spatialops/structured/stencil/StencilBuilder.h>

#include "catalog_ctx.h"

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: catalog_gpu <domain> <out.bin>\n");
    return 1;
  }
  const int id = std::atoi(argv[1]);
  if (id < 0 || id > 2) return 1;
  Out o(argv[2]);
  CatalogCtx C(id, o);
  nebo_catalog(C);
  return 0;
}

/* Empty stand-in for the CUDA samples header that the reference's generated
 * CUDA source includes (StringResources.h: `#include <helper_cuda.h>`, found
 * through `-I../../data/` in its nvcc command).  The generated code defines its
 * own error-check macro and uses nothing from that header, so an empty file on
 * the include path lets it compile unchanged. */
#pragma once

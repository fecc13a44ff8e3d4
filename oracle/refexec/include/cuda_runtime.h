/* Empty stand-in for <cuda_runtime.h> when the reference's kernel sources are compiled for the
 * CPU (test infrastructure): refexec_shim.h provides the few runtime names they use. */
#pragma once

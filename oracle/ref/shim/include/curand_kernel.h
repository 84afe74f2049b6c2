/* Test infrastructure: empty stand-in for <curand_kernel.h>; oracle/ref/shim/lts_ref_shim.h supplies the host definitions. */
#pragma once

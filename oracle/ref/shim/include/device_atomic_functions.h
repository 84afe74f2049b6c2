/* Test infrastructure: empty stand-in for <device_atomic_functions.h>; oracle/ref/shim/lts_ref_shim.h supplies the host definitions. */
#pragma once

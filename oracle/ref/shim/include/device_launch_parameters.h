/* Test infrastructure: empty stand-in for <device_launch_parameters.h>; oracle/ref/shim/lts_ref_shim.h supplies the host definitions. */
#pragma once

/* Test infrastructure: empty stand-in for <thrust/execution_policy.h>; oracle/ref/shim/lts_ref_shim.h supplies the host definitions. */
#pragma once

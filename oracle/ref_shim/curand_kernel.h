// CPU stand-in for <curand_kernel.h>: the reference's kernel header includes it but
// uses no device-side cuRAND API.  Test infrastructure only.
#pragma once

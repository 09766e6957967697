// generic_bicgstab.h -- forwards to ref_standin.h (the reference interface the shim compiles against; test
// infrastructure for running the shim where the reference checkout is absent).
#pragma once
#include "ref_standin.h"

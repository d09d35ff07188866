// common/umbrella.h of the headless engine (the reference's libs/common/include/common/umbrella.h without the
// GUI thread controls): the configuration constants and CUDACHECK. <initializer_list> is needed by graph
// helpers written against the reference (its cuda-internal.cuh:60-81 uses it without including it).
#pragma once
#include <initializer_list>
#include <stdint.h>

#include "constants.h"
#include "macros.h"

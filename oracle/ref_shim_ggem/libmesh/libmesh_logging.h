#pragma once
#include "libmesh/libmesh_common.h"

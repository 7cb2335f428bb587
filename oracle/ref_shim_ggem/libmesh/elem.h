// (the reference's GGEM headers include libMesh's elem.h; nothing of it is used)
#pragma once
#include "libmesh/point.h"

// bem2d C++ API, GB300 build: the public interface of the reference library's
// lib/bem2d.h (same header and class names), with assembly and dense solves
// on the GPU.  Programs written against the reference include this header
// and link bem2d.a plus libbem2d_gpu.so.
#ifndef BEM2D_H
#define BEM2D_H

#include "bem2d_basis.h"
#include "bem2d_basistypes.h"
#include "bem2d_curve.h"
#include "bem2d_curvetypes.h"
#include "bem2d_defs.h"
#include "bem2d_element.h"
#include "bem2d_exceptions.h"
#include "bem2d_fun.h"
#include "bem2d_geometry.h"
#include "bem2d_kernel.h"
#include "bem2d_mathroutines.h"
#include "bem2d_outputhandler.h"
#include "bem2d_outputroutines.h"
#include "bem2d_point.h"
#include "bem2d_pnpoly.h"
#include "bem2d_quadpoints.h"
#include "bem2d_quadrature.h"
#include "bem2d_shape.h"
#include "bem2d_soundsoftscattering.h"

#endif

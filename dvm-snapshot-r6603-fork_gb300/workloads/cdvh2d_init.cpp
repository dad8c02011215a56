// The module initialiser of cdvh2d.c as cdvmh writes it for a C source with
// global regular variables (cdvmh/src/c_dvmh.cpp:214-230: a C++ object in the
// tail of the converted file set): the runtime calls the init function (data
// enter of `coef`) when it initialises and the finish function at exit.
#include "dvmhlib2.h"

extern "C" void initCdvmhGlobals_cdvh2d_c();
extern "C" void finishCdvmhGlobals_cdvh2d_c();
static DvmhModuleInitializer initCdvmhGlobals_cdvh2d_c_initializer(initCdvmhGlobals_cdvh2d_c,
                                                                   finishCdvmhGlobals_cdvh2d_c);

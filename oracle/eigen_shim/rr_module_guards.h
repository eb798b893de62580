// ORACLE build support (test infrastructure only).
// Force-included (-include) when compiling the reference sources: marks the
// Dense sub-modules other than Core as already included, so that only the
// self-written "Core" shim next to this file is parsed.
#pragma once
#define EIGEN_LU_MODULE_H
#define EIGEN_CHOLESKY_MODULE_H
#define EIGEN_QR_MODULE_H
#define EIGEN_SVD_MODULE_H
#define EIGEN_GEOMETRY_MODULE_H
#define EIGEN_EIGENVALUES_MODULE_H
#include <cmath>

// Shadow of pa/math/types.hpp (types.hpp:1-33) for the oracle build.
// The reference header forces EIGEN_USE_MKL_ALL (types.hpp:4-6); MKL is absent
// here, and the fixed-size Eigen types the hot path uses never dispatch to MKL,
// so this shadow keeps the same aliases without the MKL macros.
#ifndef PA_MATH_TYPES_HPP
#define PA_MATH_TYPES_HPP

#include <cstdint>

#include <Eigen/Core>

namespace pa
{
using scalar   = float          ;
using vector2  = Eigen::Vector2f;
using vector3  = Eigen::Vector3f;
using vector4  = Eigen::Vector4f;

using integer  = std::int32_t   ;
using ivector2 = Eigen::Vector2i;
using ivector3 = Eigen::Vector3i;
using ivector4 = Eigen::Vector4i;

using matrix2  = Eigen::Matrix2f;
using matrix3  = Eigen::Matrix3f;
using matrix4  = Eigen::Matrix4f;

using imatrix2 = Eigen::Matrix2i;
using imatrix3 = Eigen::Matrix3i;
using imatrix4 = Eigen::Matrix4i;
}

#endif

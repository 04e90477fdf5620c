// ref_geometry.cpp - the reference's own reset-case lattice generators (utils/Geometry.cpp,
// copied with utils/Geometry.hpp and utils/Math.hpp into oracle/_ref/geometry/ by
// build_ref.py, with a generated Logging.hpp that turns LOG_ERROR into nothing), behind C
// entry points, so that the cases the library's rtp_reset generates can be compared with
// them bit for bit.
//
// TEST INFRASTRUCTURE ONLY.  Only the uniform distributions are exposed: the random ones
// call rand(), which the reference never seeds.
#if __has_include("geometry/Geometry.cpp")
#include "geometry/Geometry.cpp"

namespace {
void store(const std::vector<Math::float3>& v, float* out) {
  for (size_t i = 0; i < v.size(); ++i) {
    out[3 * i + 0] = v[i].x;
    out[3 * i + 1] = v[i].y;
    out[3 * i + 2] = v[i].z;
  }
}
}  // namespace

extern "C" {

// Geometry::Generate3DGrid(shape, res, start, end, Uniform); shape 0 = Box, 1 = Sphere.
// out: res[0] * res[1] * res[2] x 3 floats.  Returns the vertex count.
int ref_generate_3d_grid(int shape, const int* res, const float* s, const float* e, float* out) {
  const auto v = Geometry::Generate3DGrid(shape ? Geometry::Shape3D::Sphere : Geometry::Shape3D::Box,
                                          Math::int3({res[0], res[1], res[2]}), Math::float3({s[0], s[1], s[2]}),
                                          Math::float3({e[0], e[1], e[2]}));
  store(v, out);
  return (int)v.size();
}

// Geometry::Generate2DGrid(shape, YZ, res, start, end, Uniform); shape 0 = Rectangle, 1 = Circle.
int ref_generate_2d_grid_yz(int shape, const int* res, const float* s, const float* e, float* out) {
  const auto v = Geometry::Generate2DGrid(shape ? Geometry::Shape2D::Circle : Geometry::Shape2D::Rectangle,
                                          Geometry::Plane::YZ, Math::int2({res[0], res[1]}),
                                          Math::float3({s[0], s[1], s[2]}), Math::float3({e[0], e[1], e[2]}));
  store(v, out);
  return (int)v.size();
}

}  // extern "C"
#endif

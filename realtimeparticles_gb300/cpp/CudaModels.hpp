// Physics::Model subclasses over the C ABI of librtp_gb300.so (include/rtp.h): the drop-in a
// maintainer adds beside physics/ocl/ in the reference tree (physics/cuda/CudaModels.hpp)
// together with one `case` per model in Physics::CreateModel (physics/Model.cpp:10-24):
//
//   case ModelType::FLUIDS: return std::make_unique<Physics::Cuda::Fluids>(params);
//
// Each class keeps the reference model's contract (physics/Model.hpp:81-216):
// - the constructor creates the model, resets it to params.pCase and applies the JSON inputs
//   it was given (Fluids.cpp:76-98);
// - update() is one Model::update step unless paused (Fluids.cpp:400-457, Boids.cpp:323-384,
//   Clouds.cpp:503-627); the base class's non-virtual setters (setNbParticles, setBoundary,
//   setCase) only store their value, so update() and reset() hand the stored values to the
//   library first, as the reference's models read them at those points;
// - updateModelWithInputJson() reads the reference's JSON paths (Fluids.cpp:218-251,
//   Boids.cpp:177-210, Clouds.cpp:279-329) into the library's parameter structs;
// - errors: a failing library call throws std::runtime_error carrying rtp_last_error(), as
//   the reference's JSON transfer throws on a bad path.
// Positions for a renderer: rtp_device_ptr(handle(), RTP_BUF_POS, &p) (a float4 device buffer
// of maxNbParticles entries) in place of the GL VBOs of ModelParams.
#pragma once

#include <stdexcept>
#include <string>

#include "Model.hpp"
#include "rtp.h"

namespace Physics::Cuda
{
inline void check(int status, const char* what)
{
  if (status != RTP_OK)
    throw std::runtime_error(std::string(what) + ": " + rtp_last_error());
}

// Common part: the handle, and the base class's stored state handed to the library.
template <int MODEL>
class RtpModel : public Physics::Model
{
  public:
  RtpModel(ModelParams p, json js)
      : Model(p, js)
  {
    rtp_model_params mp {};
    mp.currNbParticles = p.currNbParticles;
    mp.maxNbParticles = p.maxNbParticles;
    mp.boxSize[0] = (float)p.boxSize.x;
    mp.boxSize[1] = (float)p.boxSize.y;
    mp.boxSize[2] = (float)p.boxSize.z;
    mp.gridRes[0] = (uint32_t)p.gridRes.x;
    mp.gridRes[1] = (uint32_t)p.gridRes.y;
    mp.gridRes[2] = (uint32_t)p.gridRes.z;
    mp.velocity = p.velocity;
    mp.dimension = dimOf(p.dimension);
    mp.pCase = (int32_t)p.pCase;
    mp.maxNbPartsInCell = 0; // the reference's constant for the model
    check(rtp_create(MODEL, &mp, &m_h), "rtp_create");
    m_init = true;
  }
  ~RtpModel() override { rtp_destroy(m_h); }
  RtpModel(const RtpModel&) = delete;
  RtpModel& operator=(const RtpModel&) = delete;

  void update() override
  {
    if (!m_init || m_pause)
      return;
    pushState();
    check(rtp_update(m_h, 1), "rtp_update");
  }

  // The case's particles (the library's reset also restores the default parameters), then
  // the model's stored JSON inputs again.
  void reset() override
  {
    if (!m_init)
      return;
    check(rtp_set_case(m_h, (int)m_case), "rtp_set_case");
    pushState();
    check(rtp_set_dimension(m_h, dimOf(m_dimension)), "rtp_set_dimension"); // stores, then resets
    json js = getInputJson();
    if (!js.empty())
      updateModelWithInputJson(js);
  }

  bool isProfilingEnabled() const override
  {
    int e = 0;
    rtp_is_profiling_enabled(m_h, &e);
    return e != 0;
  }
  void enableProfiling(bool enable) override { check(rtp_enable_profiling(m_h, enable ? 1 : 0), "rtp_enable_profiling"); }

  void* handle() const { return m_h; }

  protected:
  static uint32_t dimOf(Geometry::Dimension d) { return d == Geometry::Dimension::dim2D ? 2u : 3u; }

  void pushState()
  {
    check(rtp_set_nb_particles(m_h, m_currNbParticles), "rtp_set_nb_particles");
    check(rtp_set_boundary(m_h, m_boundary == Boundary::CyclicWall ? RTP_BOUNDARY_CYCLIC_WALL : RTP_BOUNDARY_BOUNCING_WALL),
          "rtp_set_boundary");
  }

  static rtp_fluid_params fluidParams(json& js, uint32_t dim)
  {
    auto& f = js["Fluids"];
    rtp_fluid_params fp {};
    fp.restDensity = f["Rest Density"][0].template get<float>();
    fp.relaxCFM = f["Relax CFM"][0].template get<float>();
    fp.timeStep = f["Time Step"][0].template get<float>();
    fp.dim = dim;
    auto& ap = f["Artificial Pressure"];
    fp.isArtPressureEnabled = ap["Enable##Pressure"] == true ? 1u : 0u;
    fp.artPressureCoeff = ap["Coefficient##Pressure"][0].template get<float>();
    fp.artPressureRadius = ap["Radius"][0].template get<float>();
    fp.artPressureExp = ap["Exp"][0].template get<uint32_t>();
    auto& vc = f["Vorticity Confinement"];
    fp.isVorticityConfEnabled = vc["Enable##Vorticity"] == true ? 1u : 0u;
    fp.vorticityConfCoeff = vc["Coefficient##Vorticity"][0].template get<float>();
    fp.xsphViscosityCoeff = vc["xSPH Viscosity Coefficient"][0].template get<float>();
    return fp;
  }

  void* m_h = nullptr;
};

// Physics::CL::Fluids (physics/ocl/Fluids.hpp).
class Fluids : public RtpModel<RTP_MODEL_FLUIDS>
{
  public:
  explicit Fluids(ModelParams p, json js = {})
      : RtpModel(p, js)
  {
    reset();
  }
  void updateModelWithInputJson(json& js) override
  {
    const rtp_fluid_params fp = fluidParams(js, dimOf(m_dimension));
    check(rtp_set_fluid_params(m_h, &fp), "rtp_set_fluid_params");
    check(rtp_set_jacobi_iterations(m_h, js["Fluids"]["Nb Jacobi Iterations"][0].template get<uint32_t>()),
          "rtp_set_jacobi_iterations");
  }
};

// Physics::CL::Boids (physics/ocl/Boids.hpp), with its target (physics/Target.hpp).
class Boids : public RtpModel<RTP_MODEL_BOIDS>
{
  public:
  explicit Boids(ModelParams p, json js = {})
      : RtpModel(p, js)
  {
    reset();
  }
  void updateModelWithInputJson(json& js) override
  {
    auto& b = js["Boids"];
    rtp_boids_params bp {};
    bp.velocityScale = b["Velocity"][0].template get<float>();
    bp.alignmentScale = b["Alignment"]["Enable##Alignment"].template get<bool>() ? b["Alignment"]["Scale##Alignment"][0].template get<float>() : 0.0f;
    bp.separationScale = b["Separation"]["Enable##Separation"].template get<bool>() ? b["Separation"]["Scale##Separation"][0].template get<float>() : 0.0f;
    bp.cohesionScale = b["Cohesion"]["Enable##Cohesion"].template get<bool>() ? b["Cohesion"]["Scale##Cohesion"][0].template get<float>() : 0.0f;
    check(rtp_set_boids_params(m_h, &bp), "rtp_set_boids_params");
    auto& t = b["Target"];
    rtp_target_params tp {};
    check(rtp_target_params_default(&tp), "rtp_target_params_default");
    tp.enabled = t["Enable##Target"].template get<bool>() ? 1 : 0;
    tp.visible = t["Show"].template get<bool>() ? 1 : 0;
    tp.radiusEffect = t["Radius"][0].template get<float>();
    tp.signEffect = t["Attract"].template get<bool>() ? 1 : 0; // (int)"Attract"
    check(rtp_set_target(m_h, &tp), "rtp_set_target");
  }
  Math::float3 targetPos() const override
  {
    float p[3] = { 0.0f, 0.0f, 0.0f };
    int a = 0, v = 0;
    rtp_get_target(m_h, p, &a, &v);
    return { p[0], p[1], p[2] };
  }
  bool isTargetActivated() const override
  {
    float p[3];
    int a = 0, v = 0;
    rtp_get_target(m_h, p, &a, &v);
    return a != 0;
  }
  bool isTargetVisible() const override
  {
    float p[3];
    int a = 0, v = 0;
    rtp_get_target(m_h, p, &a, &v);
    return v != 0;
  }
};

// Physics::CL::Clouds (physics/ocl/Clouds.hpp).  The environment (clouds.cl:72-89) is the
// reference's unless rtp_set_cloud_environment sets another on handle().
class Clouds : public RtpModel<RTP_MODEL_CLOUDS>
{
  public:
  explicit Clouds(ModelParams p, json js = {})
      : RtpModel(p, js)
  {
    reset();
  }
  void updateModelWithInputJson(json& js) override
  {
    const uint32_t dim = dimOf(m_dimension);
    const rtp_fluid_params fp = fluidParams(js, dim);
    auto& c = js["Clouds"];
    rtp_cloud_params cp {};
    check(rtp_cloud_params_default(&cp), "rtp_cloud_params_default");
    cp.restDensity = fp.restDensity; // Clouds.cpp:309-313: shared with the fluid inputs
    cp.timeStep = fp.timeStep;
    cp.dim = dim;
    cp.relaxCFM = fp.relaxCFM;
    cp.isTempSmoothingEnabled = c["Enable Temperature Smoothing"].template get<bool>() ? 1u : 0u;
    cp.groundHeatCoeff = c["Ground Heat Coefficient"][0].template get<float>();
    cp.buoyancyCoeff = c["Buoyancy Heat Coefficient"][0].template get<float>();
    cp.gravCoeff = c["Gravity Coefficient"][0].template get<float>();
    cp.adiabaticLapseRate = c["Adiabatic Lapse Rate"][0].template get<float>();
    cp.phaseTransitionRate = c["Phase Transition Rate"][0].template get<float>();
    cp.latentHeatCoeff = c["Latent Heat Coefficient"][0].template get<float>();
    cp.windCoeff = c["Wind Coefficient"][0].template get<float>();
    check(rtp_set_fluid_params(m_h, &fp), "rtp_set_fluid_params");
    check(rtp_set_cloud_params(m_h, &cp), "rtp_set_cloud_params");
    check(rtp_set_jacobi_iterations(m_h, js["Fluids"]["Nb Jacobi Iterations"][0].template get<uint32_t>()),
          "rtp_set_jacobi_iterations");
  }
};

// Physics::CreateModel (physics/Model.cpp:10-24) for the GB300 models.
inline std::unique_ptr<Model> CreateModel(ModelType type, ModelParams params)
{
  switch (type)
  {
    case ModelType::BOIDS:
      return std::make_unique<Boids>(params);
    case ModelType::FLUIDS:
      return std::make_unique<Fluids>(params);
    case ModelType::CLOUDS:
      return std::make_unique<Clouds>(params);
  }
  return nullptr;
}
} // namespace Physics::Cuda

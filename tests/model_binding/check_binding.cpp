// Compiles the Physics::Model subclasses of realtimeparticles_gb300/cpp/CudaModels.hpp against
// the reference's physics/Model.hpp (with the nlohmann/json stand-in beside this file) and
// links them with librtp_gb300.so.  TEST INFRASTRUCTURE ONLY.
//
//   check_binding json   - reads the fluids, boids and clouds JSON paths of the subclasses
//                          from a tree built like the reference's initial JSON (no device)
//   check_binding create - creates each model through Physics::Cuda::CreateModel, resets and
//                          steps it; prints "created <model> <n>" or the library's error
#include <cstdio>
#include <cstring>

#include "CudaModels.hpp"

namespace
{
// Trees with the reference's JSON paths and shapes (Fluids.cpp:52-75, Boids.cpp:30-52,
// Clouds.cpp:47-89: scalars as [value, min, max]); the values are samples.
json fluidsJson()
{
  return json { { "Fluids",
                  { { "Rest Density", { 450.0f, 10.0f, 1000.0f } },
                    { "Relax CFM", { 600.0f, 100.0f, 1000.0f } },
                    { "Time Step", { 0.010f, 0.0001f, 0.020f } },
                    { "Nb Jacobi Iterations", { 2, 1, 6 } },
                    { "Artificial Pressure",
                      { { "Enable##Pressure", true },
                        { "Coefficient##Pressure", { 0.001f, 0.0f, 0.001f } },
                        { "Radius", { 0.006f, 0.001f, 0.015f } },
                        { "Exp", { 4, 1, 6 } } } },
                    { "Vorticity Confinement",
                      { { "Enable##Vorticity", true },
                        { "Coefficient##Vorticity", { 0.0004f, 0.0f, 0.001f } },
                        { "xSPH Viscosity Coefficient", { 0.0001f, 0.0f, 0.001f } } } } } } };
}

json boidsJson()
{
  return json { { "Boids",
                  { { "Velocity", { 2.0f, 0.0f, 5.0f } },
                    { "Alignment", { { "Enable##Alignment", true }, { "Scale##Alignment", { 1.5f, 0.0f, 3.0f } } } },
                    { "Separation", { { "Enable##Separation", false }, { "Scale##Separation", { 1.2f, 0.0f, 3.0f } } } },
                    { "Cohesion", { { "Enable##Cohesion", true }, { "Scale##Cohesion", { 0.7f, 0.0f, 3.0f } } } },
                    { "Target",
                      { { "Enable##Target", true }, { "Show", true }, { "Radius", { 2.0f, 0.0f, 5.0f } }, { "Attract", true } } } } } };
}

json cloudsJson()
{
  json js = fluidsJson();
  js.merge_patch(json { { "Clouds",
                          { { "Enable Temperature Smoothing", true },
                            { "Ground Heat Coefficient", { 0.11f, 0.0f, 0.5f } },
                            { "Buoyancy Heat Coefficient", { 0.5f, 0.0f, 1.0f } },
                            { "Gravity Coefficient", { 0.0005f, 0.0f, 0.001f } },
                            { "Adiabatic Lapse Rate", { 5.0f, 0.0f, 10.0f } },
                            { "Phase Transition Rate", { 0.5f, 0.0f, 1.0f } },
                            { "Latent Heat Coefficient", { 0.1f, 0.0f, 1.0f } },
                            { "Wind Coefficient", { 0.3f, 0.0f, 1.0f } } } } });
  return js;
}

// A subclass whose library calls are not made: reads the JSON paths the way the models do.
struct Reader : Physics::Cuda::RtpModel<RTP_MODEL_FLUIDS>
{
  static void readAll()
  {
    json f = fluidsJson();
    const rtp_fluid_params fp = fluidParams(f, 3);
    std::printf("fluids %.4f %.1f %.4f %u %u %.4f %.4f %u %u %.5f %.5f iters %u\n", fp.restDensity, fp.relaxCFM,
                fp.timeStep, fp.dim, fp.isArtPressureEnabled, fp.artPressureRadius, fp.artPressureCoeff,
                fp.artPressureExp, fp.isVorticityConfEnabled, fp.vorticityConfCoeff, fp.xsphViscosityCoeff,
                f["Fluids"]["Nb Jacobi Iterations"][0].get<uint32_t>());
    json c = cloudsJson();
    std::printf("clouds smoothing %d wind %.2f rho0 %.1f\n", c["Clouds"]["Enable Temperature Smoothing"] == true ? 1 : 0,
                c["Clouds"]["Wind Coefficient"][0].get<float>(), fluidParams(c, 3).restDensity);
    json b = boidsJson();
    std::printf("boids %.2f %.2f %d\n", b["Boids"]["Velocity"][0].get<float>(),
                b["Boids"]["Alignment"]["Scale##Alignment"][0].get<float>(),
                b["Boids"]["Separation"]["Enable##Separation"].get<bool>() ? 1 : 0);
  }
};
} // namespace

int main(int argc, char** argv)
{
  const char* mode = argc > 1 ? argv[1] : "json";
  if (std::strcmp(mode, "json") == 0)
  {
    Reader::readAll();
    return 0;
  }
  struct Case
  {
    Physics::ModelType type;
    const char* name;
    Utils::PhysicsCase pcase;
    json js;
  };
  const Case cases[] = { { Physics::ModelType::FLUIDS, "fluids", Utils::FLUIDS_DAM, fluidsJson() },
                         { Physics::ModelType::BOIDS, "boids", Utils::BOIDS_SMALL, boidsJson() },
                         { Physics::ModelType::CLOUDS, "clouds", Utils::CLOUDS_CUMULUS, cloudsJson() } };
  for (const Case& c : cases)
  {
    Physics::ModelParams p;
    p.currNbParticles = 4096;
    p.maxNbParticles = 4096;
    p.boxSize = { 1, 1, 1 };
    p.gridRes = { 16, 16, 16 };
    p.velocity = 1.0f;
    p.dimension = Geometry::Dimension::dim3D;
    p.pCase = c.pcase;
    try
    {
      auto m = Physics::Cuda::CreateModel(c.type, p);
      json js = c.js;
      m->updateModelWithInputJson(js);
      m->reset();
      m->update();
      m->setBoundary(Physics::Boundary::CyclicWall);
      m->update();
      std::printf("created %s %zu\n", c.name, m->nbParticles());
    }
    catch (const std::runtime_error& e)
    {
      std::printf("error %s: %s\n", c.name, e.what());
      return 3;
    }
  }
  return 0;
}

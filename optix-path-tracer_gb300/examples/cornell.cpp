// The reference's Cornell scene (host_includes/scenes.hpp:188-260) written
// against pt_scene.hpp exactly as the reference writes it against OptiX,
// rendered progressively like main.cpp's sample loop.  Usage:
//   cornell W H SPP out.pfm   (writes the accumulator as a float RGB PFM)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pt_scene.hpp"

using namespace pt;

struct App_State {  // host_includes/host_common.hpp:21-45 (subset)
  Context context = Context::create();
  int W = 500, H = 500, samples = 500;
};

void Cornell(App_State& app) {
  Light_Sampler lights;
  Rectangle_PDF rect_pdf(213.f, 343.f, 227.f, 332.f, 554.f, Y_AXIS);
  lights.pdf.push_back(rect_pdf.createPDF(app.context));
  lights.sample.push_back(rect_pdf.createSample(app.context));
  lights.emissions.push_back(make_float3(7.f));

  setRayGenerationProgram(app.context, lights);
  setMissProgram(app.context, CONSTANT);
  setExceptionProgram(app.context);
  Group group;

  Texture* redTx = new Constant_Texture(0.65f, 0.05f, 0.05f);
  Texture* whiteTx = new Constant_Texture(0.73f);
  Texture* greenTx = new Constant_Texture(0.12f, 0.45f, 0.15f);
  Texture* lightTx = new Constant_Texture(7.f);

  BRDF* redMt = new Lambertian(redTx);
  BRDF* whiteMt = new Lambertian(whiteTx);
  BRDF* greenMt = new Lambertian(greenTx);
  BRDF* lightMt = new Diffuse_Light(lightTx);

  Hitable_List list;
  list.push(new AARect(0.f, 555.f, 0.f, 555.f, 555.f, true, X_AXIS, redMt));
  list.push(new AARect(0.f, 555.f, 0.f, 555.f, 0.f, false, X_AXIS, greenMt));
  list.push(new AARect(213.f, 343.f, 227.f, 332.f, 554.f, true, Y_AXIS, lightMt));
  list.push(new AARect(0.f, 555.f, 0.f, 555.f, 555.f, true, Y_AXIS, whiteMt));
  list.push(new AARect(0.f, 555.f, 0.f, 555.f, 0.f, false, Y_AXIS, whiteMt));
  list.push(new AARect(0.f, 555.f, 0.f, 555.f, 555.f, true, Z_AXIS, whiteMt));

  Box* box0 = new Box(make_float3(0.f), make_float3(165.f, 330.f, 165.f), greenMt);
  box0->translate(make_float3(265.f, 0.f, 295.f));
  box0->rotate(15.f, Y_AXIS);
  list.push(box0);

  list.addElementsTo(group, app.context);

  Camera camera(make_float3(278.f, 278.f, -800.f), make_float3(278.f, 278.f, 0.f),
                make_float3(0.f, 1.f, 0.f), 40.f, float(app.W) / float(app.H), 0.f, 10.f, 0.f,
                1.f);
  camera.set(app.context);
}

int main(int argc, char** argv) {
  App_State app;
  app.W = argc > 1 ? atoi(argv[1]) : 256;
  app.H = argc > 2 ? atoi(argv[2]) : 256;
  app.samples = argc > 3 ? atoi(argv[3]) : 16;
  const char* out = argc > 4 ? argv[4] : "cornell.pfm";
  try {
    Cornell(app);
    std::vector<float> acc((size_t)app.W * app.H * 4, 0.f);
    // one call per batch of frames, as main.cpp's loop advances "frame"
    int batch = 4;
    for (int f = 0; f < app.samples; f += batch)
      renderFrame(app.context, app.W, app.H, f, std::min(batch, app.samples - f), acc.data());
    FILE* fp = fopen(out, "wb");
    if (!fp) return 2;
    fprintf(fp, "PF\n%d %d\n-1.0\n", app.W, app.H);
    for (int y = app.H - 1; y >= 0; y--)  // PFM rows run bottom to top
      for (int x = 0; x < app.W; x++) fwrite(&acc[((size_t)y * app.W + x) * 4], 4, 3, fp);
    fclose(fp);
    printf("rendered %d spp at %dx%d -> %s\n", app.samples, app.W, app.H, out);
  } catch (const Error& e) {
    fprintf(stderr, "error %d: %s\n", e.code, e.what());
    return 1;
  }
  return 0;
}

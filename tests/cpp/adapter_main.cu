// Links the gpuvmem plugin adapter (gpuvmem_gb300/adapter/gvgb_plugins.cu,
// compiled against gpuvmem's own headers) with libgpuvmem_gb300 and checks,
// without a GPU, that gpuvmem's factories hand out the adapter's classes
// under gpuvmem's ids: main.cu's createObject<Fi, std::string>("Chi2") and
// createObject<Optimizer, std::string>("CG-FRPRMN") wiring.
//
// The globals below are the ones src/mfs.cu and src/main.cu define in a
// gpuvmem build; linkAddToDPhi stands in for src/functions.cu's.
#include <cstdio>
#include <string>
#include <vector>

#include "framework.cuh"
#include "functions.cuh"

long M = 64, N = 64;
int image_count = 2;
float* penalizators = nullptr;
int nPenalizators = 0;
std::vector<MSDataset> datasets;
std::vector<float> initial_values;
float eta = -1.0f, threshold = 0.0f, nu_0 = 230e9f;
double DELTAX = -1e-5, DELTAY = 1e-5;
bool nopositivity = false;
Vars variables;

__host__ void linkAddToDPhi(float* dphi, float* dgi, int index) {}

int main() {
  int fails = 0;
  const char* fis[] = {"Chi2", "Entropy", "TotalSquaredVariation", "TotalVariation", "L1-Norm",
                       "Laplacian"};
  for (const char* id : fis) {
    Fi* f = createObject<Fi, std::string>(id);
    const bool ok = f && f->getName() == id && f->getPenalizationFactor() == 1.0f;
    std::printf("%-22s -> %s %s\n", id, f ? f->getName().c_str() : "null", ok ? "ok" : "WRONG");
    fails += ok ? 0 : 1;
  }
  Fi* e0 = createObject<Fi, int>(0);
  fails += (e0 && e0->getName() == "Entropy") ? 0 : 1;
  const char* opts[] = {"CG-FRPRMN", "CG-LBFGS"};
  for (const char* id : opts) {
    Optimizer* o = createObject<Optimizer, std::string>(id);
    o->setK(15);
    const bool ok = o != nullptr && o->getK() == 15 && o->getFtol() == 1e-12f;
    std::printf("%-22s -> %s\n", id, ok ? "ok" : "WRONG");
    fails += ok ? 0 : 1;
  }
  ObjectiveFunction* of = createObject<ObjectiveFunction, std::string>("ObjectiveFunction");
  fails += of ? 0 : 1;
  std::printf("%s\n", fails ? "FAILED" : "adapter factory wiring ok");
  return fails ? 1 : 0;
}

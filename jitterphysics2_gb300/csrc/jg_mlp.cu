// Placeholder translation unit for the learned warm start; filled in below.
#include "jg_world.cuh"
int jg_mlp_alloc(WorldDev& w) { (void)w; return JG_OK; }
int jg_mlp_launch_warmstart(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm) { (void)w; (void)p; (void)s; (void)nsm; return JG_OK; }
extern "C" {
int jg_mlp_load(jg_world*, const float*, int32_t) { return JG_ERR_NOT_SUPPORTED; }
int jg_mlp_predict(jg_world*, const float*, int32_t, float*) { return JG_ERR_NOT_SUPPORTED; }
int jg_mlp_train_step(jg_world*, const float*, const float*, int32_t, float, float*) { return JG_ERR_NOT_SUPPORTED; }
int jg_mlp_export(jg_world*, float*, int32_t, int32_t*) { return JG_ERR_NOT_SUPPORTED; }
int jg_mlp_gradients(jg_world*, const float*, const float*, int32_t, float*, int32_t, float*) { return JG_ERR_NOT_SUPPORTED; }
int jg_collect_training(jg_world*, float*, float*, int32_t, int32_t*) { return JG_ERR_NOT_SUPPORTED; }
}

// Models compiled into libopenabl_cuda (written by regenerate.py).
#include "abl_model.h"

extern "C" {
const abl_model_desc *abl_model_desc_circle(void);
const abl_model_desc *abl_model_desc_circle3d(void);
const abl_model_desc *abl_model_desc_boids2d(void);
const abl_model_desc *abl_model_desc_game_of_life(void);
const abl_model_desc *abl_model_desc_boids2d_float(void);
const abl_model_desc *abl_model_desc_predator_prey(void);
const abl_model_desc *abl_model_desc_circle_float(void);
const abl_model_desc *abl_model_desc_circle3d_float(void);
const abl_model_desc *abl_model_desc_predator_prey_float(void);
const abl_model_desc *abl_model_desc_boids3d(void);
const abl_model_desc *abl_model_desc_boids2d_mixed(void);
const abl_model_desc *abl_model_desc_boids3d_mixed(void);
const abl_model_desc *abl_model_desc_sugarscape(void);
const abl_model_desc *abl_model_desc_boids2d_devinit(void);
const abl_model_desc *abl_model_desc_kinds(void);
const abl_model_desc *abl_model_desc_grazers(void);
const abl_model_desc *abl_model_desc_ants(void);
const abl_model_desc *abl_model_desc_boids2d_flockers(void);
const abl_model_desc *abl_model_desc_keratinocyte(void);
extern const abl_model_desc *const abl_builtin_models[];
const abl_model_desc *const abl_builtin_models[] = {
    abl_model_desc_circle(),
    abl_model_desc_circle3d(),
    abl_model_desc_boids2d(),
    abl_model_desc_game_of_life(),
    abl_model_desc_boids2d_float(),
    abl_model_desc_predator_prey(),
    abl_model_desc_circle_float(),
    abl_model_desc_circle3d_float(),
    abl_model_desc_predator_prey_float(),
    abl_model_desc_boids3d(),
    abl_model_desc_boids2d_mixed(),
    abl_model_desc_boids3d_mixed(),
    abl_model_desc_sugarscape(),
    abl_model_desc_boids2d_devinit(),
    abl_model_desc_kinds(),
    abl_model_desc_grazers(),
    abl_model_desc_ants(),
    abl_model_desc_boids2d_flockers(),
    abl_model_desc_keratinocyte(),
    nullptr};
}

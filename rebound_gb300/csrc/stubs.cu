// Temporary: modules not yet built.
#include "rgpu_internal.cuh"
int tree_accel(rgpu_sim* s) { return set_error(s, RGPU_ERR_UNSUPPORTED, "tree gravity not built"); }
int tree_collisions(rgpu_sim* s, rgpu_collision*, size_t, size_t*, bool) { return set_error(s, RGPU_ERR_UNSUPPORTED, "tree collisions not built"); }
void tree_free(rgpu_sim*) {}
int direct_collisions(rgpu_sim* s, rgpu_collision*, size_t, size_t*, bool) { return set_error(s, RGPU_ERR_UNSUPPORTED, "direct collisions not built"); }
int resolve_collisions_device(rgpu_sim* s) { return set_error(s, RGPU_ERR_UNSUPPORTED, "resolve not built"); }

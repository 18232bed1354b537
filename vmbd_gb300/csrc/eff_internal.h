// Internal helpers shared between the C-ABI translation units.
#pragma once
#include <string>

struct EffPlan;

namespace eff {
// Record `msg` as the calling thread's eff_last_error() and return `code`.
int set_error(int code, const std::string& msg);
// Device the plan was created on (-1 for a null plan).
int plan_device(const EffPlan* plan);
// EFF_OK when the plan's device is the current device, else an
// EFF_ERR_INVALID / EFF_ERR_CUDA status with the message recorded.
int check_plan_device(const EffPlan* plan);
// The plan was created with EFF_GEOM_DETERMINISTIC.
bool plan_deterministic(const EffPlan* plan);
}  // namespace eff

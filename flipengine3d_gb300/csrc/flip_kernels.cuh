// Kernel launch interface; see flip_device.cuh.
#pragma once
#include "flip_device.cuh"

// Stand-in for c2h/vector.h: with THRUST_DEVICE_SYSTEM=CPP both vectors live in host memory.
#pragma once
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>
namespace c2h
{
template <class T>
using host_vector = thrust::host_vector<T>;
template <class T>
using device_vector = thrust::device_vector<T>;
} // namespace c2h

// dp/culling/cuda/Manager.h -- the Mode::CUDA culling backend for nvpro-pipeline.
//
// Drop-in for the reference tree: it sits beside dp/culling/cpu and dp/culling/opengl,
// derives from dp::culling::ManagerBitSet as they do (dp/culling/cpu/Manager.h:37-44),
// and culls on a GB300 through the dpcull C ABI (include/dpcull.h of the GB300
// backend).  Selected by the Mode switch of dp/sg/xbar/culling/src/CullingImpl.cpp:52-63.
#pragma once

#include <dp/culling/Config.h>
#include <dp/culling/ManagerBitSet.h>

namespace dp
{
  namespace culling
  {
    namespace cuda
    {

      class Manager : public dp::culling::ManagerBitSet
      {
      public:
        // device: CUDA ordinal of the GPU to cull on.
        DP_CULLING_API static Manager* create( int device = 0 );

        // Culls the group against `count` world matrices already in device memory (16-byte
        // aligned, 16 floats each, for instance the output of a GPU transform tree) instead
        // of the host array of groupSetMatrices: no host round trip, the matrices are read
        // at every cull.  nullptr returns the group to its host matrices.
        DP_CULLING_API virtual void groupSetDeviceMatrices( GroupSharedPtr const& group, float const* matrices,
                                                            size_t count ) = 0;
      };

    } // namespace cuda
  } // namespace culling
} // namespace dp

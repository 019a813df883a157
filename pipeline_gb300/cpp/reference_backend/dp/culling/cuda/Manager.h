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
      };

    } // namespace cuda
  } // namespace culling
} // namespace dp

// dp/culling/cuda/src/ManagerImpl.cpp -- Mode::CUDA backend over the dpcull C ABI.
//
// Object, group and result state are the reference's own BitSet classes; only the cull
// and the bounding box run on the GPU:
//   * GroupCUDA keeps a device copy of its objects and matrices and rebuilds it exactly
//     when cpu::GroupCPU rebuilds its OBB cache (dp/culling/cpu/src/ManagerImpl.cpp:
//     114-162), so stale-cache behaviour matches the CPU backend call for call;
//   * cull() computes the visibility words on the GPU (bit-exact with the CPU manager's
//     isVisible) and hands them to the reference's ResultBitSet::updateChanged, which
//     builds the changed list and applies its resize rules unchanged;
//   * calculateBoundingBox() folds the world-space corners on the GPU in group order
//     from a separate device copy of the current objects and matrices.
#include <dp/culling/cuda/Manager.h>
#include <dp/culling/GroupBitSet.h>
#include <dp/culling/ObjectBitSet.h>
#include <dp/culling/ResultBitSet.h>
#include <dp/util/FrameProfiler.h>

#include <dpcull.h>

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace dp
{
  namespace culling
  {
    namespace cuda
    {
      namespace
      {
        void check( int rc, char const* what )
        {
          if ( rc != DPCULL_OK )
          {
            throw std::runtime_error( std::string( what ) + ": " + dpcull_last_error() );
          }
        }

        struct Context
        {
          dpcull_ctx ctx = nullptr;
          ~Context() { if ( ctx ) { dpcull_ctx_destroy( ctx ); } }
        };
        typedef std::shared_ptr<Context> ContextSharedPtr;

        DEFINE_PTR_TYPES( GroupCUDA );

        class GroupCUDA : public GroupBitSet
        {
        public:
          static GroupCUDASharedPtr create( ContextSharedPtr const& context )
          {
            return std::shared_ptr<GroupCUDA>( new GroupCUDA( context ) );
          }

          virtual ~GroupCUDA()
          {
            dpcull_result_destroy( m_context->ctx, m_result );
            dpcull_group_destroy( m_context->ctx, m_group );
            if ( m_haveBox ) { dpcull_group_destroy( m_context->ctx, m_boxGroup ); }
          }

          // Uploads the current objects and matrices into `group`.
          void upload( dpcull_group group ) const
          {
            size_t const n = m_objects.size();
            std::vector<float> lower( 3 * n ), extent( 3 * n );
            std::vector<uint32_t> xform( n );
            for ( size_t i = 0; i < n; ++i )
            {
              ObjectBitSetSharedPtr const& o = m_objects[i];
              for ( int c = 0; c < 3; ++c )
              {
                lower[c * n + i] = o->getLowerLeft()[c];
                extent[c * n + i] = o->getExtent()[c];
              }
              if ( o->getTransformIndex() > 0xFFFFFFFFull )
              {
                throw std::runtime_error( "transform index does not fit the device index type" );
              }
              xform[i] = uint32_t( o->getTransformIndex() );
            }
            dpcull_ctx ctx = m_context->ctx;
            check( dpcull_group_set_objects( ctx, group, n, lower.data(), extent.data(), xform.data() ), "set objects" );
            check( dpcull_group_set_matrices( ctx, group, getMatricesCount() ? getMatrices() : nullptr, getMatricesCount(),
                                              getMatricesCount() ? getMatricesStride() : 64 ), "set matrices" );
          }

          // GroupCPU::updateOBBs: rebuild only when dirty or when objects were added/removed.
          void update()
          {
            m_obbDirty |= ( m_incarnationDevice != m_objectIncarnation );
            if ( m_obbDirty )
            {
              upload( m_group );
              m_incarnationDevice = m_objectIncarnation;
              m_obbDirty = false;
            }
          }

          // Visibility words of the current objects under `vp` (ResultBitSet layout).
          uint32_t const* cull( dp::math::Mat44f const& vp )
          {
            update();
            dpcull_ctx ctx = m_context->ctx;
            check( dpcull_cull( ctx, m_group, m_result, vp.getPtr() ), "cull" );
            size_t bits = 0;
            m_words.resize( ( m_objects.size() + 31 ) / 32 + 1 );
            check( dpcull_result_bits( ctx, m_result, m_words.data(), m_words.size(), &bits ), "result bits" );
            return m_words.data();
          }

          dp::math::Box3f box()
          {
            dpcull_ctx ctx = m_context->ctx;
            if ( !m_haveBox )
            {
              check( dpcull_group_create( ctx, &m_boxGroup ), "group create" );
              m_haveBox = true;
            }
            upload( m_boxGroup );
            float lo[3], hi[3];
            check( dpcull_group_bounding_box( ctx, m_boxGroup, lo, hi ), "bounding box" );
            return dp::math::Box3f( dp::math::Vec3f( lo[0], lo[1], lo[2] ), dp::math::Vec3f( hi[0], hi[1], hi[2] ) );
          }

        protected:
          GroupCUDA( ContextSharedPtr const& context )
            : GroupBitSet()
            , m_context( context )
            , m_incarnationDevice( m_objectIncarnation - 1 )
          {
            check( dpcull_group_create( context->ctx, &m_group ), "group create" );
            check( dpcull_result_create( context->ctx, m_group, &m_result ), "result create" );
          }

        private:
          ContextSharedPtr m_context;
          dpcull_group m_group = 0;
          dpcull_result m_result = 0;   // device visibility words of the last cull
          bool m_haveBox = false;
          dpcull_group m_boxGroup = 0;
          size_t m_incarnationDevice;
          std::vector<uint32_t> m_words;
        };

        class ManagerImpl : public Manager
        {
        public:
          explicit ManagerImpl( int device )
            : m_context( std::make_shared<Context>() )
          {
            check( dpcull_ctx_create( device, nullptr, &m_context->ctx ), "context create" );
          }

          virtual ObjectSharedPtr objectCreate( PayloadSharedPtr const& userData )
          {
            return ObjectBitSet::create( userData );
          }

          virtual GroupSharedPtr groupCreate()
          {
            return GroupCUDA::create( m_context );
          }

          virtual ResultSharedPtr groupCreateResult( GroupSharedPtr const& group )
          {
            return ResultBitSet::create( std::static_pointer_cast<GroupBitSet>( group ) );
          }

          virtual void cull( GroupSharedPtr const& group, ResultSharedPtr const& result, dp::math::Mat44f const& viewProjection )
          {
            dp::util::ProfileEntry p( "cull" );
            GroupCUDASharedPtr g = std::static_pointer_cast<GroupCUDA>( group );
            uint32_t const* words = g->cull( viewProjection );
            std::static_pointer_cast<ResultBitSet>( result )->updateChanged( words );
          }

          virtual dp::math::Box3f calculateBoundingBox( GroupSharedPtr const& group ) const
          {
            return std::static_pointer_cast<GroupCUDA>( group )->box();
          }

        private:
          ContextSharedPtr m_context;
        };

      } // namespace

      Manager* Manager::create( int device )
      {
        return new ManagerImpl( device );
      }

    } // namespace cuda
  } // namespace culling
} // namespace dp

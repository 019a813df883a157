// dp/culling/cuda/src/ManagerImpl.cpp -- Mode::CUDA backend over the dpcull C ABI.
//
// Object, group and result state are the reference's own BitSet classes; only the cull
// and the bounding box run on the GPU:
//   * GroupCUDA keeps a device copy of its objects and matrices and brings it up to date
//     exactly when cpu::GroupCPU rebuilds its OBB cache (dp/culling/cpu/src/ManagerImpl.cpp:
//     114-162), so stale-cache behaviour matches the CPU backend call for call; an update
//     sends only what changed since the copy was made (objects whose box or transform
//     index differ, matrices whose contents differ), so a frame that moves a few
//     transforms uploads a few matrices;
//   * groupSetDeviceMatrices binds device-resident world matrices (for instance those a
//     dpcull transform tree propagates on the GPU) in place of the host array: no copy,
//     read at every cull;
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
            dpcull_group_destroy( m_context->ctx, m_cull.group );
            if ( m_box.group ) { dpcull_group_destroy( m_context->ctx, m_box.group ); }
          }

          // Device matrices used in place of the host ones (nullptr: back to the host
          // matrices of groupSetMatrices).  The library reads them at every cull.
          void setDeviceMatrices( float const* matrices, size_t count )
          {
            m_devMatrices = matrices;
            m_devCount = matrices ? count : 0;
            m_obbDirty = true;
            m_cull.valid = m_box.valid = false;
          }

          // GroupCPU::updateOBBs (dp/culling/cpu/src/ManagerImpl.cpp:114-162): the device
          // copy is brought up to date only when the reference would rebuild its cache.
          void update()
          {
            m_obbDirty |= !m_cull.valid || ( m_cull.incarnation != m_objectIncarnation );
            if ( m_obbDirty )
            {
              sync( m_cull );
              m_obbDirty = false;
            }
          }

          // Visibility words of the current objects under `vp` (ResultBitSet layout).
          uint32_t const* cull( dp::math::Mat44f const& vp )
          {
            update();
            dpcull_ctx ctx = m_context->ctx;
            check( dpcull_cull( ctx, m_cull.group, m_result, vp.getPtr() ), "cull" );
            size_t bits = 0;
            m_words.resize( ( m_objects.size() + 31 ) / 32 + 1 );
            check( dpcull_result_bits( ctx, m_result, m_words.data(), m_words.size(), &bits ), "result bits" );
            return m_words.data();
          }

          // ManagerBitSet::calculateBoundingBox from the current objects and matrices: a
          // second device copy, kept apart from the cull's (whose contents stay those of its
          // last rebuild, like the reference's cache) and synchronised the same way.
          dp::math::Box3f box()
          {
            if ( !m_box.group )
            {
              check( dpcull_group_create( m_context->ctx, &m_box.group ), "group create" );
            }
            sync( m_box );
            float lo[3], hi[3];
            check( dpcull_group_bounding_box( m_context->ctx, m_box.group, lo, hi ), "bounding box" );
            return dp::math::Box3f( dp::math::Vec3f( lo[0], lo[1], lo[2] ), dp::math::Vec3f( hi[0], hi[1], hi[2] ) );
          }

        protected:
          GroupCUDA( ContextSharedPtr const& context )
            : GroupBitSet()
            , m_context( context )
          {
            check( dpcull_group_create( context->ctx, &m_cull.group ), "group create" );
            check( dpcull_result_create( context->ctx, m_cull.group, &m_result ), "result create" );
          }

        private:
          // One device copy of the group and the host state it was last synchronised with.
          struct DeviceCopy
          {
            dpcull_group group = 0;
            bool valid = false;               // holds a complete upload
            size_t incarnation = 0;           // object incarnation of the copy
            std::vector<float> lower, extent; // planar [3][n], as uploaded
            std::vector<uint32_t> xform;
            std::vector<float> matrices;      // count x 16, as uploaded (host matrices only)
          };

          // The current objects in the device layout.
          void pack( std::vector<float>& lower, std::vector<float>& extent, std::vector<uint32_t>& xform ) const
          {
            size_t const n = m_objects.size();
            lower.resize( 3 * n );
            extent.resize( 3 * n );
            xform.resize( n );
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
          }

          // Brings a device copy up to date with the current objects and matrices, as the
          // reference's rebuild reads them: every object after objects were added or removed,
          // otherwise only those whose box or transform index differ from the copy; every
          // matrix when their count changed, otherwise only those whose contents differ (the
          // ones groupMatrixChanged marked, and any the caller changed without marking,
          // which the reference's rebuild also picks up).
          void sync( DeviceCopy& d )
          {
            dpcull_ctx ctx = m_context->ctx;
            size_t const n = m_objects.size();
            std::vector<float> lower, extent;
            std::vector<uint32_t> xform;
            pack( lower, extent, xform );
            if ( !d.valid || d.incarnation != m_objectIncarnation || d.xform.size() != n )
            {
              check( dpcull_group_set_objects( ctx, d.group, n, lower.data(), extent.data(), xform.data() ), "set objects" );
            }
            else
            {
              std::vector<uint32_t> idx;
              for ( size_t i = 0; i < n; ++i )
              {
                bool same = xform[i] == d.xform[i];
                for ( int c = 0; c < 3 && same; ++c )
                {
                  same = !std::memcmp( &lower[c * n + i], &d.lower[c * n + i], 4 ) &&
                         !std::memcmp( &extent[c * n + i], &d.extent[c * n + i], 4 );
                }
                if ( !same ) { idx.push_back( uint32_t( i ) ); }
              }
              if ( idx.size() > n / 4 )
              {
                check( dpcull_group_set_objects( ctx, d.group, n, lower.data(), extent.data(), xform.data() ), "set objects" );
              }
              else if ( !idx.empty() )
              {
                size_t const k = idx.size();
                std::vector<float> lo( 3 * k ), ex( 3 * k );
                std::vector<uint32_t> xf( k );
                for ( size_t j = 0; j < k; ++j )
                {
                  for ( int c = 0; c < 3; ++c )
                  {
                    lo[c * k + j] = lower[c * n + idx[j]];
                    ex[c * k + j] = extent[c * n + idx[j]];
                  }
                  xf[j] = xform[idx[j]];
                }
                check( dpcull_group_update_objects( ctx, d.group, k, idx.data(), lo.data(), ex.data(), xf.data() ), "update objects" );
              }
            }
            if ( m_devMatrices )
            {
              check( dpcull_group_bind_device_matrices( ctx, d.group, m_devMatrices, m_devCount ), "bind matrices" );
              d.matrices.clear();
            }
            else
            {
              size_t const count = getMatricesCount(), stride = count ? getMatricesStride() : 64;
              char const* base = static_cast<char const*>( count ? getMatrices() : nullptr );
              if ( !d.valid || d.matrices.size() != 16 * count )
              {
                check( dpcull_group_set_matrices( ctx, d.group, base, count, stride ), "set matrices" );
                d.matrices.resize( 16 * count );
                for ( size_t i = 0; i < count; ++i ) { std::memcpy( &d.matrices[16 * i], base + i * stride, 64 ); }
              }
              else
              {
                std::vector<uint32_t> idx;
                for ( size_t i = 0; i < count; ++i )
                {
                  if ( std::memcmp( &d.matrices[16 * i], base + i * stride, 64 ) )
                  {
                    idx.push_back( uint32_t( i ) );
                    std::memcpy( &d.matrices[16 * i], base + i * stride, 64 );
                  }
                }
                if ( !idx.empty() )
                {
                  check( dpcull_group_update_matrices( ctx, d.group, idx.size(), idx.data(), base, stride ), "update matrices" );
                }
              }
            }
            d.lower.swap( lower );
            d.extent.swap( extent );
            d.xform.swap( xform );
            d.incarnation = m_objectIncarnation;
            d.valid = true;
          }

          ContextSharedPtr m_context;
          DeviceCopy m_cull;                    // what the cull reads
          DeviceCopy m_box;                     // what calculateBoundingBox reads
          dpcull_result m_result = 0;           // device visibility words of the last cull
          float const* m_devMatrices = nullptr; // groupSetDeviceMatrices
          size_t m_devCount = 0;
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

          virtual void groupSetDeviceMatrices( GroupSharedPtr const& group, float const* matrices, size_t count )
          {
            std::static_pointer_cast<GroupCUDA>( group )->setDeviceMatrices( matrices, count );
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

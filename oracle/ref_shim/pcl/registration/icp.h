/* Stand-in for PCL's ICP classes: the reference's registration header
 * declares members of these types; the sources compiled against the shims
 * never run them (test oracle only). */
#pragma once
#include <memory>
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>
namespace pcl {
template <class S, class T>
class IterativeClosestPoint {
  public:
    using Ptr = std::shared_ptr<IterativeClosestPoint<S, T>>;
};
template <class S, class T>
class IterativeClosestPointWithNormals {
  public:
    using Ptr = std::shared_ptr<IterativeClosestPointWithNormals<S, T>>;
};
}  // namespace pcl

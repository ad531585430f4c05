/* Minimal stand-in for pcl::PointCloud (test oracle only). */
#pragma once
#include <algorithm>
#include <memory>
#include <vector>
namespace pcl {
template <class T>
class PointCloud : public std::vector<T> {
  public:
    using Ptr = std::shared_ptr<PointCloud<T>>;
    PointCloud& operator+=(const PointCloud& o) {
        this->insert(this->end(), o.begin(), o.end());
        return *this;
    }
};
}  // namespace pcl

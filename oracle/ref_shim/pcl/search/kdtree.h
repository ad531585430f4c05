/* Stand-in for pcl::search::KdTree (test oracle only): an exact k-nearest
 * search by brute force.  Squared distances are accumulated in float, x then
 * y then z, and returned ascending; among equal distances the lower point
 * index comes first (PCL's FLANN tree fixes no order for ties).  Fewer than
 * k results when the cloud is smaller, as PCL returns. */
#pragma once
#include <algorithm>
#include <numeric>
#include <vector>
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>
namespace pcl {
namespace search {
template <class T>
class KdTree {
  public:
    void setInputCloud(const typename PointCloud<T>::Ptr& c) { cloud_ = c; }
    int nearestKSearch(const T& p, int k, std::vector<int>& idx, std::vector<float>& dis) const {
        const int n = cloud_ ? (int)cloud_->size() : 0;
        std::vector<float> d(n);
        for (int i = 0; i < n; ++i) {
            const T& q = (*cloud_)[i];
            float a = (q.x - p.x) * (q.x - p.x);
            a = a + (q.y - p.y) * (q.y - p.y);
            a = a + (q.z - p.z) * (q.z - p.z);
            d[i] = a;
        }
        std::vector<int> order(n);
        std::iota(order.begin(), order.end(), 0);
        const int m = std::min(k, n);
        std::partial_sort(order.begin(), order.begin() + m, order.end(),
                          [&](int a, int b) { return d[a] < d[b] || (d[a] == d[b] && a < b); });
        idx.assign(order.begin(), order.begin() + m);
        dis.resize(m);
        for (int i = 0; i < m; ++i) dis[i] = d[idx[i]];
        return m;
    }

  private:
    typename PointCloud<T>::Ptr cloud_;
};
}  // namespace search
}  // namespace pcl

/* Stand-in for PCL's normal estimation header: the reference's registration
 * header only names point types from it (test oracle only). */
#pragma once
#include <pcl/point_cloud.h>
#include <pcl/point_types.h>

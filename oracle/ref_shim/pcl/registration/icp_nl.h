/* Stand-in for PCL's non-linear ICP header (test oracle only). */
#pragma once
#include <pcl/registration/icp.h>

/* Stand-in for PCL's GICP header (test oracle only). */
#pragma once
#include <pcl/registration/icp.h>

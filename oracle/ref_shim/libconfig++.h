/* Empty stand-in for libconfig (test oracle only). */
#pragma once
namespace libconfig {
class Config {};
}

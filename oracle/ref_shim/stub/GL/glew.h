/* Empty stand-in: the reference's host BVH/camera code includes <GL/glew.h>
 * (Core/Ray.cuh:4) but uses nothing from it. Oracle build only. */
#pragma once

/* Empty stand-in: Utils/Surface.h includes <FreeImage.h> but its declarations
 * used by the BVH/camera host path need none of it. Oracle build only. */
#pragma once

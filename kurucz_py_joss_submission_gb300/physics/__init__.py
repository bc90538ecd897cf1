"""Line opacity on the GPU."""

"""Line-list readers."""

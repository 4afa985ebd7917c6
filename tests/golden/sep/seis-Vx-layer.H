

Bin/rtm.x:   lin7@cees-gpu   Tue Jul 28 10:32:06 2015
		n1=3535
		o1=0
		d1=0.000565685
		n2=300
		o2=0
		d2=4
		sets next: in="/data/lin7/seis-Vx-layer.H@"
		data_format="xdr_float"
